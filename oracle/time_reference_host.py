"""TEST INFRASTRUCTURE (a measurement of the reference, not product code): time the reference's own
host special-function work, single-threaded, as its executable runs it.

    make -C oracle ref REF_DIR=<reference checkout>
    python oracle/time_reference_host.py

Loads oracle/_ref/libref_bimsim.so (the reference's bessjy.cpp, cbessjy.cpp, gamma.cpp,
sphere.cpp, nearfield.cpp compiled in place) and times, on the 50-sphere scene of the 1024^2
benchmark slice (seeded, bimsim_gb300.scenes.config2):

  * sphere::calcCoeff (sphere.cpp:21-97): Mie coefficients, per sphere
  * the host half of sphere::calcUp (sphere.cpp:222-272): calcHankelLut over the table's radii
    and calcBesselLut over the interior radii (sphere.cpp:99-203), per sphere, at the benchmark's
    4096 radial samples (the reference's own default is 2 x the near-field resolution, 6144)
  * nearfieldStruct::calcBesselLut (nearfield.cpp:222-283): the incident-field table, per
    wavelength, at 4096 radii and field order 10

The reference runs these serially on one core before its GPU kernels.  Writes
profiles/reference_host_timings.json with the host it ran on.
"""
import ctypes as C
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "bimsim-cuda_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))


def cpu_name():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    import oracle_lib
    from bimsim_gb300 import abi, scenes
    path = os.path.join(HERE, "_ref", "libref_bimsim.so")
    if not os.path.exists(path):
        sys.exit("build oracle/_ref first: make -C oracle ref REF_DIR=<checkout>")
    r = C.CDLL(path)
    vp = C.c_void_p
    r.ref_calc_coeff.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, vp, vp]
    r.ref_hankel_lut.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, vp]
    r.ref_bessel_lut.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, vp]
    r.ref_uf_bessel_lut.argtypes = [C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, vp]
    r.ref_calc_nl.argtypes = [C.c_float, C.c_float]
    p, spheres, _ = scenes.config2()
    lam = p.lambda_
    k = 2 * float(np.float32(3.14159)) / lam
    t_coef = t_up = 0.0
    for s in spheres:
        a, nre, nim = s[3], s[4], s[5]
        nl = r.ref_calc_nl(a, lam)
        A = np.zeros(2 * nl + 2)
        B = np.zeros(2 * nl + 2)
        t0 = time.perf_counter()
        r.ref_calc_coeff(a, lam, nre, nim, A.ctypes.data_as(vp), B.ctypes.data_as(vp))
        t1 = time.perf_counter()
        g = oracle_lib.sphere_geom(p, abi.Sphere(*s))
        h = np.zeros(2 * g.dR * (nl + 1))
        j = np.zeros(2 * max(g.aR, 1) * (nl + 1))
        t2 = time.perf_counter()
        r.ref_hankel_lut(a, k, g.d_min, g.d_max, nl, g.dR, h.ctypes.data_as(vp))
        r.ref_bessel_lut(a, k, nre, nim, nl, g.aR, j.ctypes.data_as(vp))
        t3 = time.perf_counter()
        t_coef += t1 - t0
        t_up += t3 - t2
    dR, m = p.uf_lut_r, p.field_order
    uf = np.zeros(dR * (m + 1))
    dmin, dmax = C.c_double(), C.c_double()  # the table's distance range, as the oracle derives it
    oracle_lib.load().bso_uf_table(C.byref(p), uf.ctypes.data_as(vp), C.byref(dmin), C.byref(dmax))
    t0 = time.perf_counter()
    r.ref_uf_bessel_lut(lam, m, dmin.value, dmax.value, dR, uf.ctypes.data_as(vp))
    t_uf = time.perf_counter() - t0
    ns = len(spheres)
    out = {
        "host": cpu_name(), "machine": platform.machine(), "threads": 1,
        "scene": "1024^2 benchmark slice: 50 spheres a~U(1,5) um, lambda 3 um, tables of 4096 radii",
        "calcCoeff_ms_per_sphere": 1e3 * t_coef / ns,
        "calcUp_host_luts_ms_per_sphere": 1e3 * t_up / ns,
        "calcBesselLut_uf_ms_per_wavelength": 1e3 * t_uf,
        "slice_host_ms": 1e3 * (t_coef + t_up + t_uf),
        "source": "oracle/time_reference_host.py on oracle/_ref/libref_bimsim.so",
    }
    dst = os.path.join(REPO, "profiles", "reference_host_timings.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
