"""Point-source illumination (bs_simulate_sources, the reference's
SimulateExtendedSource) and the far field (bs_get_far_field) on the GPU,
against the oracle: per source the oracle's slice, summed on the detector."""
import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import (BS_FIELD_INCIDENT, BS_FIELD_TOTAL, BS_IMG_ABSORBANCE, BS_IMG_INCIDENT, BS_IMG_INTENSITY,
                          BS_PREC_FP64, BS_PREC_MIXED, Context, abi, lib, scenes)

pytestmark = pytest.mark.gpu

TOL = {BS_PREC_FP64: 1e-10, BS_PREC_MIXED: 1e-5}


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def scene(lut_us=True):
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                        lut_us=lut_us, us_lut_r=128, us_lut_theta=160)
    s = [(0.5, -0.5, 0.0, 2.0, 1.4, 0.04), (-4.0, 3.5, 0.5, 1.2, 1.5, 0.0)]
    return p, s, scenes.mc_waves(32, 0, 0.5, seed=14)


def sources(p):
    # three point sources on the detector plane (as LoadExtendedSource places them), amplitudes 1, 0.5, 0.25
    return np.array([[*lib.plane_point(p, u, v), a] for u, v, a in ((0.5, 0.5, 1.0), (0.25, 0.5, 0.5),
                                                                    (0.5, 0.75, 0.25))])


@pytest.mark.parametrize("prec", [BS_PREC_FP64, BS_PREC_MIXED])
@pytest.mark.parametrize("lut_us", [True, False])
def test_sources_sum_matches_oracle(prec, lut_us):
    p, s, w = scene(lut_us)
    src = sources(p)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate_sources(src, prec)
        D = ctx.image(BS_IMG_INTENSITY, f64=True)
        Di = ctx.image(BS_IMG_INCIDENT, f64=True)
        A = ctx.image(BS_IMG_ABSORBANCE, f64=True)
        st = ctx.stats()
    Do = np.zeros_like(D)
    Dio = np.zeros_like(D)
    arr, ns = abi.sphere_array(s)
    for f in src:
        q = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                            lut_us=lut_us, us_lut_r=128, us_lut_theta=160, focus=tuple(f[:3]), amplitude=f[3])
        _, _, d, di = oracle_lib.simulate(q, arr, ns, w)
        Do += d
        Dio += di
    assert rel(D, Do) <= TOL[prec] and rel(Di, Dio) <= TOL[prec]
    assert rel(A, -np.log10(Do / Dio)) <= 10 * TOL[prec]
    if lut_us:
        assert st.lut_tables_built == len(s)  # built for the first source only


def test_sources_equal_separate_runs_and_keep_context_state():
    p, s, w = scene()
    src = sources(p)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate_sources(src, BS_PREC_FP64)
        D = ctx.image(BS_IMG_INTENSITY, f64=True)
        acc = np.zeros_like(D)
        for f in src:
            q = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16,
                                padding=1, us_lut_r=128, us_lut_theta=160, focus=tuple(f[:3]), amplitude=f[3])
            ctx.set_params(q)
            ctx.simulate(BS_PREC_FP64)
            acc += ctx.image(BS_IMG_INTENSITY, f64=True)
        assert rel(D, acc) < 1e-14
        # a plain simulate afterwards uses the context's own focus and amplitude again
        ctx.set_params(p)
        ctx.simulate(BS_PREC_FP64)
        one = ctx.image(BS_IMG_INTENSITY, f64=True)
    _, _, d0, _ = oracle_lib.simulate(p, *abi.sphere_array(s), w)
    assert rel(one, d0) <= 1e-10


@pytest.mark.parametrize("prec", [BS_PREC_FP64, BS_PREC_MIXED])
def test_far_field_matches_oracle(prec):
    import ctypes as C
    p, s, w = scene()
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(prec)
        far = ctx.far_field(BS_FIELD_TOTAL)
        far_i = ctx.far_field(BS_FIELD_INCIDENT)
        D = ctx.image(BS_IMG_INTENSITY, f64=True)
        U = ctx.field(BS_FIELD_TOTAL)
    ol = oracle_lib.load()
    U64 = np.ascontiguousarray(U.astype(np.complex128))
    out = np.zeros(2 * far.size)
    ol.bso_far_field(C.byref(p), U64.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
    ref = out.view(np.complex128).reshape(far.shape)
    assert rel(far, ref) <= (1e-10 if prec == BS_PREC_FP64 else 1e-5)
    # the detector intensity is |far field|^2 (ss = 1 here)
    assert rel(np.abs(far) ** 2, D) <= (1e-12 if prec == BS_PREC_FP64 else 1e-5)
    assert np.linalg.norm(far_i) > 0


PI_F = np.float32(3.14159)


def rotate_fields(F, R, c, s, centre_int):
    """nfInterpolate.cu:13-58 restated: F sampled at the pixel rotated about the centre, bilinear with
    exact weights, zero outside; coordinates in float32, each operation rounded."""
    uc = np.float32(int(R / 2.0)) if centre_int else np.float32(R / 2.0)
    iu = np.arange(R, dtype=np.float32)[None, :]
    iv = np.arange(R, dtype=np.float32)[:, None]
    du, dv = iu - uc, iv - uc
    nx = (uc + du * c) - dv * s
    ny = (uc + du * s) + dv * c
    fx, fy = np.floor(nx), np.floor(ny)
    a = (nx - fx).astype(np.float64)
    e = (ny - fy).astype(np.float64)
    i0, j0 = fx.astype(np.int64), fy.astype(np.int64)

    def at(i, j):
        ok = (i >= 0) & (i < R) & (j >= 0) & (j < R)
        return np.where(ok, F[np.clip(j, 0, R - 1), np.clip(i, 0, R - 1)], 0)
    return ((1 - a) * (1 - e) * at(i0, j0) + a * (1 - e) * at(i0 + 1, j0) + (1 - a) * e * at(i0, j0 + 1)
            + a * e * at(i0 + 1, j0 + 1))


@pytest.mark.parametrize("prec", [BS_PREC_FP64, BS_PREC_MIXED])
def test_ring_interpolation_matches_oracle_restatement(prec):
    """The reference's --interpolate 3: central source, then per ring the first source simulated and the
    others imaged from its near field rotated by their own angles (the oracle's slices, rotated in numpy,
    through the oracle's detector)."""
    import ctypes as C
    import math
    points, rings = 4, 3
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                        us_lut_r=128, us_lut_theta=160)
    s = [(0.0, 0.0, 0.0, 2.0, 1.4, 0.04)]
    w = scenes.mc_waves(32, 0, 0.5, seed=15)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate_ring_interp(points, rings, prec)
        D = ctx.image(BS_IMG_INTENSITY, f64=True)
        Di = ctx.image(BS_IMG_INCIDENT, f64=True)
    ol = oracle_lib.load()
    arr, ns = abi.sphere_array(s)
    R = oracle_lib.geom(p).R
    _, _, Do, Dio = oracle_lib.simulate(p, arr, ns, w)
    Do, Dio = Do.copy(), Dio.copy()
    step = np.float32(np.float32(2) * PI_F) / np.float32(points)
    for ring in range(1, rings):
        th = [step]
        for _ in range(points - 1):
            th.append(np.float32(th[-1] + step))
        f0 = (float(np.float32(math.cos(float(th[0]))) * np.float32(ring)),
              float(np.float32(math.sin(float(th[0]))) * np.float32(ring)), 0.0)
        q = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                            us_lut_r=128, us_lut_theta=160, focus=f0, amplitude=1.0)
        U, Uf, d, di = oracle_lib.simulate(q, arr, ns, w)
        Do += d
        Dio += di
        for a in th[1:]:
            c, sn = np.float32(math.cos(float(a))), np.float32(math.sin(float(a)))
            Ur = np.ascontiguousarray(rotate_fields(U.reshape(R, R), R, c, sn, True), dtype=np.complex128)
            Ufr = np.ascontiguousarray(rotate_fields(Uf.reshape(R, R), R, c, sn, False), dtype=np.complex128)
            d1, di1 = np.zeros_like(Do), np.zeros_like(Dio)
            ol.bso_detector(C.byref(p), Ur.ctypes.data_as(C.c_void_p), Ufr.ctypes.data_as(C.c_void_p),
                            d1.ctypes.data_as(C.c_void_p), di1.ctypes.data_as(C.c_void_p))
            Do += d1
            Dio += di1
    assert rel(D, Do) <= TOL[prec] and rel(Di, Dio) <= TOL[prec], (rel(D, Do), rel(Di, Dio))
