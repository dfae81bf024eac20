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



RING_CASES = [(3, 4, 3), (1, 4, 3), (2, 6, 3), (2, 8, 4), (3, 1, 2), (1, 5, 1)]


@pytest.mark.parametrize("prec", [BS_PREC_FP64, BS_PREC_MIXED])
@pytest.mark.parametrize("mode,points,rings", RING_CASES)
def test_ring_sources_match_oracle(prec, mode, points, rings):
    """The reference's --interpolate 1, 2, 3 (ring sources by rotated detector images, a radial line of
    ring samples, rotated near fields) against the oracle's restatement of the same drivers.  Mode 2 with
    6 points exercises the reference's tree sum, which leaves samples out for counts that are not powers
    of two."""
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                        us_lut_r=128, us_lut_theta=160, focus=(0.5, -0.25, 0.0), amplitude=0.75)
    s = [(0.0, 0.0, 0.0, 2.0, 1.4, 0.04)]
    w = scenes.mc_waves(32, 0, 0.5, seed=15)
    run = {1: "simulate_ring_detector", 2: "simulate_ring_line", 3: "simulate_ring_interp"}[mode]
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        getattr(ctx, run)(points, rings, prec)
        D = ctx.image(BS_IMG_INTENSITY, f64=True)
        Di = ctx.image(BS_IMG_INCIDENT, f64=True)
        st = ctx.stats()
        # the context's own focus and amplitude are kept for later runs
        ctx.simulate(prec)
        D1 = ctx.image(BS_IMG_INTENSITY, f64=True)
    Do, Dio = oracle_lib.simulate_rings(p, *abi.sphere_array(s), w, mode, points, rings)
    assert rel(D, Do) <= TOL[prec] and rel(Di, Dio) <= TOL[prec], (rel(D, Do), rel(Di, Dio))
    assert st.lut_tables_built == len(s)  # built for the first source only
    _, _, d1, _ = oracle_lib.simulate(p, *abi.sphere_array(s), w)
    assert rel(D1, d1) <= TOL[prec]


def test_ring_line_point_limit():
    p, s, w = scene()
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        with pytest.raises(RuntimeError, match="at most 1023"):
            ctx.simulate_ring_line(1024, 2, BS_PREC_MIXED)
        with pytest.raises(RuntimeError, match=">= 1"):
            ctx.simulate_ring_detector(0, 2, BS_PREC_MIXED)
