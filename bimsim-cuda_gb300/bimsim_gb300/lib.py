"""ctypes binding of libbimsim_gb300.so and a thin context wrapper."""
import ctypes as C
import os

import numpy as np

from . import abi

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_LIB = None


class BimsimError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def library_path():
    return os.path.join(PKG, "lib", "libbimsim_gb300.so")


def library():
    """Load the CUDA library; raises if it was not built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                           "or python -m bimsim_gb300.build")
    lib = C.CDLL(path)
    vp, i32, sz = C.c_void_p, C.c_int32, C.c_size_t
    proto = {
        "bs_version": ([], C.c_char_p),
        "bs_last_error": ([], C.c_char_p),
        "bs_create": ([vp, C.POINTER(vp)], C.c_int),
        "bs_destroy": ([vp], C.c_int),
        "bs_set_spheres": ([vp, vp, i32], C.c_int),
        "bs_set_waves": ([vp, vp, i32], C.c_int),
        "bs_sample_waves_compat": ([vp, i32], C.c_int),
        "bs_set_lut_budget": ([vp, sz], C.c_int),
        "bs_simulate": ([vp, C.c_int], C.c_int),
        "bs_get_image": ([vp, C.c_int, vp, sz], C.c_int),
        "bs_get_image_f64": ([vp, C.c_int, vp, sz], C.c_int),
        "bs_get_field": ([vp, C.c_int, vp, sz], C.c_int),
        "bs_write_envi": ([vp, C.c_int, C.c_char_p, i32, C.c_double], C.c_int),
        "bs_envi_add_band": ([C.c_char_p, vp, i32, i32, C.c_double, i32], C.c_int),
        "bs_get_info": ([vp, vp], C.c_int),
        "bs_get_stats": ([vp, vp], C.c_int),
        "bs_get_mie": ([vp, i32, vp, vp, i32], C.c_int),
        "bs_get_lut": ([vp, i32, i32, vp, sz], C.c_int),
        "bs_measure_fma_peak": ([vp, vp], C.c_int),
        "bs_mie_noalloc": ([vp, i32, i32, C.c_double, vp, vp, vp], C.c_int),
        "bs_set_params": ([vp, vp], C.c_int),
        "bs_sweep": ([vp, vp, i32, vp, C.c_int, C.c_int, vp, C.c_char_p, i32], C.c_int),
        "bs_simulate_sources": ([vp, vp, i32, C.c_int], C.c_int),
        "bs_simulate_ring_interp": ([vp, i32, i32, C.c_int], C.c_int),
    "bs_simulate_ring_detector": ([vp, i32, i32, C.c_int], C.c_int),
    "bs_simulate_ring_line": ([vp, i32, i32, C.c_int], C.c_int),
        "bs_plane_point": ([vp, C.c_double, C.c_double, vp], C.c_int),
        "bs_get_far_field": ([vp, C.c_int, vp, sz], C.c_int),
        "bs_material_eval": ([C.c_char_p, vp, i32, vp], C.c_int),
    "bs_material_kk": ([C.c_char_p, C.c_double, i32, i32, vp, vp], C.c_int),
        "bs_set_lut_reuse": ([vp, i32], C.c_int),
        "bs_set_stream_priority": ([vp, i32], C.c_int),
        "bs_set_lut_staging": ([vp, i32], C.c_int),
    "bs_set_lut_wave_chunk": ([vp, i32], C.c_int),
    "bs_set_backpropagation": ([vp, i32, C.c_double], C.c_int),
        "bs_release_buffers": ([vp], C.c_int),
        "bs_estimate_bytes": ([vp, vp, i32, i32, C.c_int, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
        "bs_server_create": ([vp, C.POINTER(vp)], C.c_int),
        "bs_server_destroy": ([vp], C.c_int),
        "bs_submit": ([vp, vp, C.POINTER(C.c_uint64)], C.c_int),
        "bs_poll": ([vp, C.c_uint64, C.POINTER(i32)], C.c_int),
        "bs_wait": ([vp, C.c_uint64, C.c_double], C.c_int),
        "bs_fetch": ([vp, C.c_uint64, vp, sz, vp], C.c_int),
        "bs_server_get_stats": ([vp, vp], C.c_int),
    }
    for name, (args, res) in proto.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _LIB = lib
    return lib


def measure_fma_peak():
    """(fp32, fp64) FMA throughput of the current GPU in TFLOP/s."""
    lib = library()
    a, b = C.c_double(), C.c_double()
    st = lib.bs_measure_fma_peak(C.byref(a), C.byref(b))
    if st != 0:
        raise BimsimError(st, "FMA peak measurement failed")
    return a.value, b.value


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One simulation context (owns device memory and a CUDA stream)."""

    def __init__(self, params):
        self.lib = library()
        self.params = params
        h = C.c_void_p()
        self._check(self.lib.bs_create(C.byref(params), C.byref(h)))
        self.h = h

    def _check(self, st):
        if st != 0:
            raise BimsimError(st, self.lib.bs_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.bs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_spheres(self, spheres):
        arr, n = spheres if isinstance(spheres, tuple) else abi.sphere_array(spheres)
        self._check(self.lib.bs_set_spheres(self.h, C.cast(arr, C.c_void_p), n))

    def set_waves(self, dirs):
        d = np.ascontiguousarray(dirs, dtype=np.float64).reshape(-1)
        self._check(self.lib.bs_set_waves(self.h, _p(d), len(d) // 3))

    def sample_waves_compat(self, nk):
        self._check(self.lib.bs_sample_waves_compat(self.h, nk))

    def set_lut_budget(self, nbytes):
        self._check(self.lib.bs_set_lut_budget(self.h, nbytes))

    def simulate(self, precision=abi.BS_PREC_MIXED):
        self._check(self.lib.bs_simulate(self.h, precision))

    def info(self):
        i = abi.Info()
        self._check(self.lib.bs_get_info(self.h, C.byref(i)))
        return i

    def stats(self):
        s = abi.Stats()
        self._check(self.lib.bs_get_stats(self.h, C.byref(s)))
        return s

    def image(self, kind=abi.BS_IMG_INTENSITY, f64=False):
        res = self.params.resolution
        if f64:
            out = np.zeros(res * res, dtype=np.float64)
            self._check(self.lib.bs_get_image_f64(self.h, kind, _p(out), out.size))
        else:
            out = np.zeros(res * res, dtype=np.float32)
            self._check(self.lib.bs_get_image(self.h, kind, _p(out), out.size))
        return out.reshape(res, res)

    def field(self, kind=abi.BS_FIELD_TOTAL):
        R = self.info().nf_res
        out = np.zeros(2 * R * R, dtype=np.float64)
        self._check(self.lib.bs_get_field(self.h, kind, _p(out), R * R))
        return out.view(np.complex128).reshape(R, R)

    def far_field(self, kind=abi.BS_FIELD_TOTAL):
        """Band-passed, cropped far field (res*ss)^2 complex of the last run."""
        n = self.params.resolution * self.params.supersample
        out = np.zeros(2 * n * n, dtype=np.float64)
        self._check(self.lib.bs_get_far_field(self.h, kind, _p(out), n * n))
        return out.view(np.complex128).reshape(n, n)

    def mie(self, sphere, nl):
        A = np.zeros(2 * (nl + 1))
        B = np.zeros(2 * (nl + 1))
        self._check(self.lib.bs_get_mie(self.h, sphere, _p(A), _p(B), nl + 1))
        return A.view(np.complex128), B.view(np.complex128)

    def lut(self, sphere, which, rows, thetaR):
        out = np.zeros(2 * rows * thetaR)
        self._check(self.lib.bs_get_lut(self.h, sphere, which, _p(out), rows * thetaR))
        return out.view(np.complex128).reshape(rows, thetaR)

    def write_envi(self, kind, path, append, band_value):
        self._check(self.lib.bs_write_envi(self.h, kind, path.encode(), 1 if append else 0, band_value))

    def sweep(self, lambdas, n_table, precision=abi.BS_PREC_MIXED, kind=abi.BS_IMG_INTENSITY, envi_path=None,
              band_as_nu=False, images=True):
        """Images (nl, res, res) float32 of a spectral sweep; n_table: (nl, ns) complex indices."""
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        nt = np.ascontiguousarray(np.asarray(n_table, dtype=np.complex128)).view(np.float64)
        res = self.params.resolution
        out = np.zeros((len(lam), res, res), dtype=np.float32) if images else None
        self._check(self.lib.bs_sweep(self.h, _p(lam), len(lam), _p(nt) if nt.size else None, precision, kind,
                                      _p(out) if out is not None else None,
                                      envi_path.encode() if envi_path else None, 1 if band_as_nu else 0))
        return out

    def simulate_sources(self, sources, precision=abi.BS_PREC_MIXED):
        """sources: (n, 4) rows of focus x, y, z and amplitude; detector images sum over them."""
        a = np.ascontiguousarray(sources, dtype=np.float64).reshape(-1, 4)
        self._check(self.lib.bs_simulate_sources(self.h, _p(a), len(a), precision))

    def simulate_ring_interp(self, points, rings, precision=abi.BS_PREC_MIXED):
        """The reference's --interpolate 3: ring sources by rotating each ring's first near field."""
        self._check(self.lib.bs_simulate_ring_interp(self.h, points, rings, precision))

    def simulate_ring_detector(self, points, rings, precision=abi.BS_PREC_MIXED):
        """The reference's --interpolate 1: ring sources by rotating each ring's first detector image."""
        self._check(self.lib.bs_simulate_ring_detector(self.h, points, rings, precision))

    def simulate_ring_line(self, points, rings, precision=abi.BS_PREC_MIXED):
        """The reference's --interpolate 2: detector images from a radial line of ring samples."""
        self._check(self.lib.bs_simulate_ring_line(self.h, points, rings, precision))

    def set_params(self, params):
        self._check(self.lib.bs_set_params(self.h, C.byref(params)))
        self.params = params

    def set_lut_staging(self, mode):
        """0 model-chosen, 1 staged kernel, 2 texture-only kernel (same results)."""
        self._check(self.lib.bs_set_lut_staging(self.h, mode))

    def set_backpropagation(self, enable, d=0.0):
        """Propagate U over d um before the band-pass (the reference's disabled applyBackpropagation)."""
        self._check(self.lib.bs_set_backpropagation(self.h, int(bool(enable)), float(d)))

    def set_lut_wave_chunk(self, chunk):
        """Waves per chunk of the mixed LUT kernel: 0 chooses per run, else 16, 32 or 64."""
        self._check(self.lib.bs_set_lut_wave_chunk(self.h, chunk))

    def set_lut_reuse(self, enable):
        self._check(self.lib.bs_set_lut_reuse(self.h, 1 if enable else 0))

    def release_buffers(self):
        self._check(self.lib.bs_release_buffers(self.h))


def envi_add_band(path, band, band_value, append):
    """Write (append=False) or append one float32 band of a host image to an ENVI file."""
    lib = library()
    b = np.ascontiguousarray(band, dtype=np.float32)
    lines, samples = b.shape
    st = lib.bs_envi_add_band(str(path).encode(), _p(b), samples, lines, float(band_value), 1 if append else 0)
    if st != 0:
        raise BimsimError(st, lib.bs_last_error().decode())


def material_eval(path, lambdas):
    """Complex refractive index of a material file at each wavelength (um)."""
    lib = library()
    lam = np.ascontiguousarray(lambdas, dtype=np.float64).reshape(-1)
    out = np.zeros(2 * lam.size)
    st = lib.bs_material_eval(str(path).encode(), _p(lam), lam.size, _p(out))
    if st != 0:
        raise BimsimError(st, lib.bs_last_error().decode())
    return out.view(np.complex128)


def material_kk(path, n0, n_samples=0, pf=2):
    """Kramers-Kronig real index of a material file: (wavelengths, n + i kappa)."""
    lib = library()
    lam = np.zeros(n_samples if n_samples else 16384)  # 16384 = BS_KK_MAX_SAMPLES
    out = np.zeros(2 * lam.size)
    st = lib.bs_material_kk(str(path).encode(), float(n0), int(n_samples), int(pf), _p(lam), _p(out))
    if st != 0:
        raise BimsimError(st, lib.bs_last_error().decode())
    n = n_samples if n_samples else int(np.count_nonzero(lam))  # wavelengths are positive
    return lam[:n].copy(), out[:2 * n].view(np.complex128).copy()


def plane_point(params, u, v):
    """Point A + u X + v Y of the detector plane (microscopeStruct::pos)."""
    lib = library()
    out = np.zeros(3)
    st = lib.bs_plane_point(C.byref(params), u, v, _p(out))
    if st != 0:
        raise BimsimError(st, lib.bs_last_error().decode())
    return out


def estimate_bytes(params, spheres, n_waves, precision=abi.BS_PREC_MIXED, lut_budget=0):
    """Device bytes a context holds after simulating this scene (host-only estimate)."""
    lib = library()
    arr, n = abi.sphere_array(spheres)
    out = C.c_uint64()
    st = lib.bs_estimate_bytes(C.byref(params), C.cast(arr, C.c_void_p), n, n_waves, precision, lut_budget,
                               C.byref(out))
    if st != 0:
        raise BimsimError(st, lib.bs_last_error().decode())
    return out.value


class Server:
    """Serving front end: submit slice requests, poll or wait, fetch images."""

    def __init__(self, workers=4, hbm_budget=0, dry_run=False):
        self.lib = library()
        cfg = abi.ServerConfig(workers, 1 if dry_run else 0, hbm_budget)
        h = C.c_void_p()
        self._check(self.lib.bs_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._res = {}

    def _check(self, st):
        if st != 0:
            raise BimsimError(st, self.lib.bs_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.bs_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, params, spheres, waves=None, n_waves=None, precision=abi.BS_PREC_MIXED,
               image=abi.BS_IMG_INTENSITY):
        """waves: (nk, 3) unit directions, or None with n_waves for the compat sampler."""
        arr, n = abi.sphere_array(spheres)
        q = abi.Request()
        q.params = params
        q.spheres = C.cast(arr, C.c_void_p)
        q.n_spheres = n
        keep = None
        if waves is not None:
            keep = np.ascontiguousarray(waves, dtype=np.float64).reshape(-1)
            q.waves = _p(keep)
            q.n_waves = keep.size // 3
        else:
            q.waves = None
            q.n_waves = n_waves or 0
        q.precision = precision
        q.image = image
        t = C.c_uint64()
        self._check(self.lib.bs_submit(self.h, C.byref(q), C.byref(t)))
        self._res[t.value] = params.resolution
        return t.value

    def poll(self, ticket):
        d = C.c_int32()
        self._check(self.lib.bs_poll(self.h, ticket, C.byref(d)))
        return bool(d.value)

    def wait(self, ticket, timeout=-1.0):
        self._check(self.lib.bs_wait(self.h, ticket, timeout))

    def fetch(self, ticket):
        """(image float32 res x res, ResultInfo); raises if the run failed."""
        res = self._res.pop(ticket)
        out = np.zeros(res * res, dtype=np.float32)
        info = abi.ResultInfo()
        self._check(self.lib.bs_fetch(self.h, ticket, _p(out), out.size, C.byref(info)))
        return out.reshape(res, res), info

    def stats(self):
        s = abi.ServerStats()
        self._check(self.lib.bs_server_get_stats(self.h, C.byref(s)))
        return s
