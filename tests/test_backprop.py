"""Back-propagation of the near field before the band-pass (bs_set_backpropagation,
the reference's applyBackpropagation that its Simulate() leaves commented out)
against the oracle's band-pass with the same propagator."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import (BS_FIELD_TOTAL, BS_IMG_INCIDENT, BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED, Context,
                          abi, scenes)

pytestmark = pytest.mark.gpu
TOL = {BS_PREC_FP64: 1e-10, BS_PREC_MIXED: 1e-5}


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def scene():
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                        us_lut_r=128, us_lut_theta=160)
    s = [(0.5, -0.5, 0.0, 2.0, 1.4, 0.04), (-4.0, 3.5, 0.5, 1.2, 1.5, 0.0)]
    return p, s, scenes.mc_waves(32, 0, 0.5, seed=14)


def run(p, s, w, prec, d=None):
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        if d is not None:
            ctx.set_backpropagation(True, d)
        ctx.simulate(prec)
        return (ctx.image(BS_IMG_INTENSITY, f64=True), ctx.image(BS_IMG_INCIDENT, f64=True),
                ctx.far_field(BS_FIELD_TOTAL))


@pytest.mark.parametrize("prec", [BS_PREC_FP64, BS_PREC_MIXED])
@pytest.mark.parametrize("d", [-3.0, 2.5])
def test_backprop_matches_oracle(prec, d):
    p, s, w = scene()
    D, Di, _ = run(p, s, w, prec, d)
    U, Uf, _, _ = oracle_lib.simulate(p, *abi.sphere_array(s), w)
    res = p.resolution
    Do, Dio = np.zeros(res * res), np.zeros(res * res)
    U = np.ascontiguousarray(U, dtype=np.complex128)
    Uf = np.ascontiguousarray(Uf, dtype=np.complex128)
    oracle_lib.load().bso_detector_bp(C.byref(p), U.ctypes.data_as(C.c_void_p), Uf.ctypes.data_as(C.c_void_p), d,
                                      Do.ctypes.data_as(C.c_void_p), Dio.ctypes.data_as(C.c_void_p))
    assert rel(D, Do.reshape(res, res)) <= TOL[prec] and rel(Di, Dio.reshape(res, res)) <= TOL[prec]


def test_backprop_over_zero_distance_flips_the_sign_only():
    p, s, w = scene()
    D0, Di0, F0 = run(p, s, w, BS_PREC_FP64)
    D, Di, F = run(p, s, w, BS_PREC_FP64, 0.0)
    assert np.array_equal(D, D0) and np.array_equal(Di, Di0)
    assert np.array_equal(F, -F0)
    D2, _, F2 = run(p, s, w, BS_PREC_FP64, 4.0)
    assert rel(D2, D0) > 1e-3  # a real propagation changes the image
