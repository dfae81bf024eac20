"""Loader for the oracle (test infrastructure): oracle/_build/libbimsim_oracle.so.

Only tests, __graft_entry__.smoke() and bench.py's CPU legs use this.
"""
import ctypes as C
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(REPO, "oracle", "_build", "libbimsim_oracle.so")
REF_SO = os.path.join(REPO, "oracle", "_ref", "libref_bimsim.so")
_lib = None


class Geom(C.Structure):
    _fields_ = [("R", C.c_int32), ("det_res", C.c_int32), ("crop_res", C.c_int32), ("crop_off", C.c_int32),
                ("A", C.c_double * 3), ("X", C.c_double * 3), ("Y", C.c_double * 3),
                ("kmag", C.c_double), ("sub_amp", C.c_double), ("cos_alpha", C.c_double),
                ("cos_beta", C.c_double)]


class SphereGeom(C.Structure):
    _fields_ = [("Nl", C.c_int32), ("aR", C.c_int32), ("dR", C.c_int32), ("thetaR", C.c_int32),
                ("d_min", C.c_double), ("d_max", C.c_double)]


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(ORACLE_SO):
        subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle")])
    lib = C.CDLL(ORACLE_SO)
    vp = C.c_void_p
    lib.bso_sbessel_real.argtypes = [C.c_int, C.c_double, vp, vp]
    lib.bso_sbessel_complex.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, vp, vp, vp, vp]
    lib.bso_mie.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, vp, vp]
    lib.bso_calc_nl.argtypes = [C.c_double, C.c_double]
    lib.bso_glibc_rand.argtypes = [C.c_uint, C.c_int, vp]
    lib.bso_mc_sample.argtypes = [C.c_int, vp, C.c_double, C.c_double, vp]
    lib.bso_derive.argtypes = [vp, vp]
    lib.bso_sphere_derive.argtypes = [vp, vp, vp]
    lib.bso_sphere_luts.argtypes = [vp, vp, vp, vp]
    lib.bso_uf_table.argtypes = [vp, vp, vp, vp]
    lib.bso_simulate.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_int, vp, vp, vp, vp]
    lib.bso_nearfield_rows.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]
    lib.bso_nearfield_rows_timed.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]
    lib.bso_detector.argtypes = [vp, vp, vp, vp, vp]
    lib.bso_detector_bp.argtypes = [vp, vp, vp, C.c_double, vp, vp]
    lib.bso_kk_transform.argtypes = [C.c_int, C.c_int, C.c_double, vp, vp, vp]
    lib.bso_simulate_rings.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]
    lib.bso_far_field.argtypes = [vp, vp, vp]
    lib.bso_fft.argtypes = [C.c_int, C.c_int, vp]
    lib.bso_envi_add_band.argtypes = [C.c_char_p, vp, C.c_int, C.c_int, C.c_double, C.c_int]
    _lib = lib
    return lib


def load_ref():
    if not os.path.exists(REF_SO):
        return None
    return C.CDLL(REF_SO)


def geom(params):
    g = Geom()
    load().bso_derive(C.byref(params), C.byref(g))
    return g


def sphere_geom(params, sphere):
    g = SphereGeom()
    load().bso_sphere_derive(C.byref(params), C.byref(sphere), C.byref(g))
    return g


def simulate_rings(params, spheres, ns, waves, mode, points, rings, nthreads=0):
    """Ring point sources (--interpolate mode 1, 2 or 3) -> (D, Di)."""
    lib = load()
    res = geom(params).det_res
    D = np.zeros(res * res)
    Di = np.zeros(res * res)
    w = np.ascontiguousarray(waves, dtype=np.float64).reshape(-1)
    nk = len(w) // 3
    rc = lib.bso_simulate_rings(C.byref(params), C.byref(spheres), ns, P(w) if nk else None, nk, nthreads, mode,
                                points, rings, P(D), P(Di))
    assert rc == 0, rc
    return D.reshape(res, res), Di.reshape(res, res)


def nearfield_rows(params, spheres, ns, waves, row0, row1, nthreads=0):
    """Oracle near field U (after sumUf) of pixel rows [row0, row1): complex128 (row1 - row0, R)."""
    lib = load()
    R = geom(params).R
    U = np.zeros(2 * (row1 - row0) * R)
    w = np.ascontiguousarray(waves, dtype=np.float64).reshape(-1)
    nk = len(w) // 3
    rc = lib.bso_nearfield_rows(C.byref(params), C.byref(spheres), ns, P(w) if nk else None, nk, nthreads, row0,
                                row1, P(U))
    assert rc == 0, rc
    return U.view(np.complex128).reshape(row1 - row0, R)


def simulate(params, spheres, ns, waves, nthreads=0):
    """Full oracle path -> (U, Uf, D, Di) as numpy arrays (complex128 / float64)."""
    lib = load()
    g = geom(params)
    R, res = g.R, g.det_res
    U = np.zeros(2 * R * R)
    Uf = np.zeros(2 * R * R)
    D = np.zeros(res * res)
    Di = np.zeros(res * res)
    w = np.ascontiguousarray(waves, dtype=np.float64).reshape(-1)
    nk = len(w) // 3
    lib.bso_simulate(C.byref(params), C.byref(spheres), ns, P(w) if nk else None, nk, nthreads,
                     P(U), P(Uf), P(D), P(Di))
    return (U.view(np.complex128).reshape(R, R), Uf.view(np.complex128).reshape(R, R),
            D.reshape(res, res), Di.reshape(res, res))
