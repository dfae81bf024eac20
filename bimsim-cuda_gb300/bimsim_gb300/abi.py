"""ctypes mirror of include/bimsim_gb300.h (plain structs and prototypes).

The structures below must stay byte-compatible with the C header; the CPU
test suite checks their sizes against the values the library reports.
"""
import ctypes as C

BS_OK = 0
BS_PREC_FP64 = 0
BS_PREC_MIXED = 1
BS_IMG_INTENSITY, BS_IMG_INCIDENT, BS_IMG_ABSORBANCE, BS_IMG_TRANSMITTANCE = 0, 1, 2, 3
BS_FIELD_TOTAL, BS_FIELD_INCIDENT = 0, 1

STATUS_NAMES = {0: "BS_OK", 1: "BS_ERR_ARG", 2: "BS_ERR_CUDA", 3: "BS_ERR_NOMEM", 4: "BS_ERR_STATE",
                5: "BS_ERR_IO", 6: "BS_ERR_TIMEOUT", 7: "BS_ERR_UNSUPPORTED", 8: "BS_ERR_NOTREADY"}


class Params(C.Structure):
    _fields_ = [
        ("lambda_", C.c_double),
        ("amplitude", C.c_double),
        ("k_dir", C.c_double * 3),
        ("focus", C.c_double * 3),
        ("condenser", C.c_double * 2),
        ("objective", C.c_double * 2),
        ("plane_min", C.c_double * 3),
        ("plane_max", C.c_double * 3),
        ("plane_normal", C.c_double * 3),
        ("resolution", C.c_int32),
        ("padding", C.c_int32),
        ("supersample", C.c_int32),
        ("field_order", C.c_int32),
        ("scalar", C.c_int32),
        ("plane_wave", C.c_int32),
        ("lut_uf", C.c_int32),
        ("lut_us", C.c_int32),
        ("us_lut_r", C.c_int32),
        ("us_lut_theta", C.c_int32),
        ("uf_lut_r", C.c_int32),
        ("reserved", C.c_int32),
    ]


class Sphere(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("a", C.c_double),
                ("n_re", C.c_double), ("n_im", C.c_double)]


class Info(C.Structure):
    _fields_ = [("nf_res", C.c_int32), ("det_res", C.c_int32), ("n_spheres", C.c_int32),
                ("n_waves", C.c_int32), ("uf_lut_r", C.c_int32), ("us_lut_theta", C.c_int32),
                ("device_bytes", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_uf", C.c_double), ("ms_mie", C.c_double),
                ("ms_lut", C.c_double), ("ms_us", C.c_double), ("ms_detector", C.c_double),
                ("kernel_launches", C.c_int64), ("us_interactions", C.c_int64),
                ("lut_chunks_staged", C.c_int64), ("lut_chunks_total", C.c_int64),
                ("lut_tables_built", C.c_int64), ("lut_staged_predicted", C.c_double),
                ("lut_wave_chunk", C.c_int64)]


class ServerConfig(C.Structure):
    _fields_ = [("workers", C.c_int32), ("dry_run", C.c_int32), ("hbm_budget", C.c_uint64)]


class Request(C.Structure):
    _fields_ = [("params", Params), ("spheres", C.c_void_p), ("n_spheres", C.c_int32), ("n_waves", C.c_int32),
                ("waves", C.c_void_p), ("precision", C.c_int32), ("image", C.c_int32)]


class ResultInfo(C.Structure):
    _fields_ = [("ms_queued", C.c_double), ("ms_total", C.c_double), ("ms_gpu", C.c_double),
                ("status", C.c_int32), ("lut_reused", C.c_int32), ("worker", C.c_int32), ("reserved", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("running", C.c_int64), ("lut_reuses", C.c_int64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("bytes_in_use", C.c_uint64),
                ("bytes_peak", C.c_uint64), ("hbm_budget", C.c_uint64)]


def make_params(lam=1.0, amplitude=1.0, k_dir=(0.0, 0.0, 1.0), focus=(0.0, 0.0, 0.0),
                condenser=(0.0, 1.0), objective=(0.0, 1.0), xy=None, plane=None,
                resolution=256, padding=1, supersample=None, field_order=10, scalar=True,
                plane_wave=False, lut_uf=False, lut_us=True, us_lut_r=0, us_lut_theta=0, uf_lut_r=0):
    """Build a Params the way the reference's LoadParameters would.

    xy=(size, z) gives the --xy plane (arguments.h:350-366); plane=(pmin, pmax, normal)
    gives an explicit plane.  supersample=None applies the reference's automatic
    rule ss = ceil(2 s / (res lambda)) when s/res > lambda/2 (arguments.h:411-418).
    """
    p = Params()
    p.lambda_ = lam
    p.amplitude = amplitude
    p.k_dir[:] = list(k_dir)
    p.focus[:] = list(focus)
    p.condenser[:] = list(condenser)
    p.objective[:] = list(objective)
    s = 40.0
    if xy is not None:
        s, z = xy
        pmin, pmax, nrm = (-s / 2, -s / 2, z), (s / 2, s / 2, z), (0.0, 0.0, 1.0)
    elif plane is not None:
        pmin, pmax, nrm = plane
    else:
        pmin, pmax, nrm = (-5.0, 0.0, -5.0), (5.0, 0.0, 5.0), (0.0, 1.0, 0.0)
    p.plane_min[:] = list(pmin)
    p.plane_max[:] = list(pmax)
    p.plane_normal[:] = list(nrm)
    p.resolution = resolution
    p.padding = padding
    if supersample is None:
        import math
        import numpy as np
        dx = np.float32(s) / np.float32(resolution)
        ss = 1
        if dx > np.float32(lam) / 2.0:
            ss = int(math.ceil(2 * np.float32(s) / (np.float32(resolution) * np.float32(lam))))
        supersample = ss
    p.supersample = supersample
    p.field_order = field_order
    p.scalar = 1 if scalar else 0
    p.plane_wave = 1 if plane_wave else 0
    p.lut_uf = 1 if lut_uf else 0
    p.lut_us = 1 if lut_us else 0
    p.us_lut_r = us_lut_r
    p.us_lut_theta = us_lut_theta
    p.uf_lut_r = uf_lut_r
    return p


def sphere_array(spheres):
    """spheres: iterable of (x, y, z, a, n_re, n_im) -> ctypes array."""
    spheres = list(spheres)
    arr = (Sphere * max(1, len(spheres)))()
    for i, s in enumerate(spheres):
        arr[i] = Sphere(*[float(v) for v in s])
    return arr, len(spheres)
