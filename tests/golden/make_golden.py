"""Generate the golden vectors under tests/golden/ from the reference's own code.

Run where the reference checkout exists (it is not available on the GPU host):

    make -C oracle ref
    python tests/golden/make_golden.py

It loads oracle/_ref/libref_bimsim.so, i.e. the reference's bessjy.cpp,
cbessjy.cpp, gamma.cpp, sphere.cpp, montecarlo.cpp, nearfield.cpp,
rts/envi/envi.h and rts/optics/material.h (its Kramers-Kronig routine over the
FFTW stand-in oracle/ref_stub/fftw3.h) compiled in place (oracle/Makefile), and records what those
functions return on a fixed grid of inputs.  The CPU tests then check the
oracle against these files on any machine.
"""
import ctypes as C
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(REPO, "oracle", "_ref", "libref_bimsim.so")


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def f32(x):
    return float(np.float32(x))


def cplx_list(v):
    return [[float(v[2 * i]), float(v[2 * i + 1])] for i in range(len(v) // 2)]


def main(out_dir=HERE):
    if not os.path.exists(LIB):
        sys.exit("build oracle/_ref first: make -C oracle ref")
    r = C.CDLL(LIB)
    out = {}

    # spherical Bessel functions of a real argument (bessjyv_sph, bessjy.cpp:709-728)
    real = []
    for N in (6, 25, 82):
        for x in (0.07, 0.5, 1.0, 2.0, 5.3, 9.5, 11.9, 12.1, 20.0, 47.0, 150.0, 300.0):
            j = np.zeros(N + 1)
            y = np.zeros(N + 1)
            r.ref_bessjyv_sph(N, C.c_double(x), P(j), P(y))
            real.append({"N": N, "x": x, "j": j.tolist(), "y": y.tolist()})
    out["bessel_real"] = real

    # complex argument (cbessjyva_sph, cbessjy.cpp:718-737), including |z| > 12 on the real axis
    cpx = []
    for N in (6, 25, 82):
        for z in (0.3 + 0.01j, 2 + 0.1j, 8.4 + 0.2j, 10.5 + 0j, 12.566 + 0j, 14.0 + 0.35j,
                  16.8 + 0.5j, 40 + 1j, 62.83 + 0j, 100 + 2j):
            a = [np.zeros(2 * N + 2) for _ in range(4)]
            r.ref_cbessjyva_sph(N, C.c_double(z.real), C.c_double(z.imag), *[P(t) for t in a])
            cpx.append({"N": N, "z": [z.real, z.imag], "j": a[0].tolist(), "y": a[1].tolist(),
                        "jp": a[2].tolist(), "yp": a[3].tolist()})
    out["bessel_complex"] = cpx

    # Nl (sphere.h:71-74)
    nl = []
    for a in np.linspace(0.5, 25.0, 50):
        for lam in (2.0, 2.5, 3.0, 7.3, 12.5):
            nl.append([f32(a), f32(lam), int(r.ref_calc_nl(C.c_float(a), C.c_float(lam)))])
    out["calc_nl"] = nl

    # Mie coefficients as the reference stores them (sphere.cpp:21-97)
    mie = []
    for a, lam, nre, nim in ((5, 2.5, 1.4, 0.05), (1, 3, 1.2, 0.0), (4.7, 3, 1.6, 0.05),
                             (2.5, 2.0, 1.45, 0.1), (20, 2, 1.5, 0.02), (0.5, 7.3, 1.3, 0.001),
                             (3.3, 12.5, 1.45, 0.08)):
        Nl = r.ref_calc_nl(C.c_float(a), C.c_float(lam))
        A = np.zeros(2 * Nl + 2)
        B = np.zeros(2 * Nl + 2)
        r.ref_calc_coeff(C.c_float(a), C.c_float(lam), C.c_float(nre), C.c_float(nim), P(A), P(B))
        # k as calcCoeff forms it: 2*PI/lambda in single precision (PI = 3.14159f)
        k = f32(np.float32(2.0) * np.float32(3.14159) / np.float32(lam))
        mie.append({"a": f32(a), "lambda": f32(lam), "n": [f32(nre), f32(nim)], "k": k, "Nl": Nl,
                    "A": cplx_list(A), "B": cplx_list(B)})
    out["mie"] = mie

    # Hankel and internal Bessel tables (sphere.cpp:99-203)
    tabs = []
    for a, lam, dmin, dmax, Nl, rR, aR, nre, nim in ((2.0, 3.0, 0.0, 80.0, 10, 9, 7, 1.4, 0.05),
                                                     (5.0, 2.5, 0.0, 40.0, 24, 7, 6, 1.4, 0.05)):
        k = f32(np.float32(2.0) * np.float32(3.14159) / np.float32(lam))
        h = np.zeros(2 * rR * (Nl + 1))
        r.ref_hankel_lut(C.c_float(a), C.c_float(k), C.c_float(dmin), C.c_float(dmax), Nl, rR, P(h))
        j = np.zeros(2 * aR * (Nl + 1))
        r.ref_bessel_lut(C.c_float(a), C.c_float(k), C.c_float(nre), C.c_float(nim), Nl, aR, P(j))
        tabs.append({"a": a, "k": k, "dmin": dmin, "dmax": dmax, "Nl": Nl, "rR": rR, "aR": aR,
                     "n": [nre, nim], "h": cplx_list(h), "j": cplx_list(j)})
    out["sphere_tables"] = tabs

    # incident-field Bessel table (nearfield.cpp:222-283)
    uft = []
    for lam, m, dmin, dmax, dR in ((3.0, 10, 0.0, 70.0, 11), (2.5, 6, 1.5, 30.0, 9)):
        t = np.zeros(dR * (m + 1))
        r.ref_uf_bessel_lut(C.c_float(lam), m, C.c_float(dmin), C.c_float(dmax), dR, P(t))
        uft.append({"lambda": lam, "m": m, "dmin": dmin, "dmax": dmax, "dR": dR, "j": t.tolist()})
    out["uf_table"] = uft

    # glibc rand() after srand(0), and mcSampleNA (montecarlo.cpp:9-71)
    seq = np.zeros(700, dtype=np.int32)
    r.ref_rand(0, 700, P(seq))
    out["rand_seed0"] = seq.tolist()
    mc = []
    for kd, nin, nout, nk in (((0.0, 0.0, 1.0), 0.0, 0.5, 64), ((0.3, 0.2, float(np.sqrt(0.87))), 0.2, 0.5, 64),
                              ((0.0, 0.0, 1.0), 0.0, 1.0, 32)):
        kd32 = [f32(v) for v in kd]
        o = np.zeros(3 * nk)
        r.ref_mc_sample(nk, C.c_float(kd32[0]), C.c_float(kd32[1]), C.c_float(kd32[2]),
                        C.c_float(nin), C.c_float(nout), P(o))
        mc.append({"k": kd32, "na": [f32(nin), f32(nout)], "nk": nk, "dirs": o.tolist()})
    out["mc"] = mc

    # quad distances (rts/math/quad.h:179-205) in the reference's single precision
    qd = []
    for pmin, pmax, nrm, sc, pt in (((-10, -10, 0), (10, 10, 0), (0, 0, 1), 5, (0, 0, 0)),
                                    ((-50, -50, 0), (50, 50, 0), (0, 0, 1), 3, (12.5, -7.25, 3.0)),
                                    ((-5, 0, -5), (5, 0, 5), (0, 1, 0), 3, (40, 2, 1)),
                                    ((-50, -50, 0), (50, 50, 0), (0, 0, 1), 3, (400, 300, -20)),
                                    ((-20, -20, 4), (20, 20, 4), (0, 0, 1), 1, (-30, 5, 0))):
        a32 = [np.array(v, dtype=np.float32) for v in (pmin, pmax, nrm, pt)]
        dm = C.c_float()
        dx = C.c_float()
        r.ref_quad_dist(P(a32[0]), P(a32[1]), P(a32[2]), C.c_float(sc), P(a32[3]), C.byref(dm), C.byref(dx))
        qd.append({"pmin": pmin, "pmax": pmax, "normal": nrm, "scale": sc, "p": pt,
                   "dmin": dm.value, "dmax": dx.value})
    out["quad"] = qd

    # ENVI bytes: one band written, a second appended (scalarslice.cu:146-166)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "band")
        b1 = (np.arange(12, dtype=np.float32) * 0.25 - 1.0)
        b2 = (np.arange(12, dtype=np.float32) ** 2).astype(np.float32)
        env = {"b1": b1.tolist(), "b2": b2.tolist(), "samples": 4, "lines": 3, "wl": [3.0, 3333.3333]}
        r.ref_envi_add_band(path.encode(), P(b1), 4, 3, C.c_double(3.0), 0)
        env["hdr_1"] = open(path + ".hdr").read()
        env["dat_1"] = open(path, "rb").read().hex()
        r.ref_envi_add_band(path.encode(), P(b2), 4, 3, C.c_double(3333.3333), 1)
        env["hdr_2"] = open(path + ".hdr").read()
        env["dat_2"] = open(path, "rb").read().hex()
    out["envi"] = env

    # material files (rts/optics/material.h, rts/math/function.h): parsing, sorting, the swapped
    # interpolation weights, end clamping, wavenumber and absorbance columns, dropped signs
    cases = {
        "microns_unsorted": "4.0 1.50 0.02\n2.0 1.40 0.00\n3.0 1.45 0.10\n6.0 1.30 0.05\n",
        "header_wavenumber": "# measured [wavenumber,n,k]\n2500 1.41 0.01\n2000 1.43 0.03\n1000 1.38 0.2\n",
        "absorbance": "#[microns,n,A]\n2.5 1.42 0.3\n5.0 1.44 0.9\n10.0 1.40 0.1\n",
        "comments_signs": "# plain file\n3.0 1.4 -0.05\n# a comment row\n5.0 1.6 0.07\n4.0 1.5 .5\n",
        "duplicates": "3.0 1.4 0.01\n3.0 1.6 0.03\n5.0 1.5 0.02\n",
    }
    lams = np.array([1.0, 2.0, 2.5, 3.0, 3.25, 3.5, 4.0, 4.75, 5.0, 5.5, 7.0, 12.0], dtype=np.float64)
    mats = {}
    with tempfile.TemporaryDirectory() as td:
        for name, text in cases.items():
            path = os.path.join(td, name + ".txt")
            open(path, "w").write(text)
            res = np.zeros(2 * lams.size)
            r.ref_material_eval(path.encode(), lams.size, P(lams), P(res))
            mats[name] = {"text": text, "lambda": lams.tolist(), "n": res.tolist()}
    out["material"] = mats

    # Kramers-Kronig (material<double>::computeN, material.h:257-432, with the FFTW stand-in
    # oracle/ref_stub/fftw3.h): resampling grid, float k and alpha, zero padding, the FFT Hilbert
    # multiplier and n = Re(chi1) / (2 n0) + n0
    lam = np.linspace(2.5, 12.5, 120)
    kap = 0.08 * 0.3 ** 2 / ((lam - 6.0) ** 2 + 0.3 ** 2)
    band = "".join(f"{l:.6f} 1.5 {k:.8f}\n" for l, k in zip(lam, kap))
    nu = np.linspace(3800.0, 900.0, 150)
    absb = 0.6 * 30.0 ** 2 / ((nu - 1650.0) ** 2 + 30.0 ** 2) + 0.2 * 25.0 ** 2 / ((nu - 1240.0) ** 2 + 25.0 ** 2)
    wn = "# FTIR [wavenumber,n,A]\n" + "".join(f"{v:.3f} 1.45 {a:.7f}\n" for v, a in zip(nu, absb))
    kk_cases = {"band_default": (band, 1.5, 0, 2), "band_64_pf1": (band, 1.5, 64, 1),
                "band_200_pf3": (band, 1.5, 200, 3), "wavenumber_absorbance": (wn, 1.45, 0, 4)}
    r.ref_material_kk.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_double, C.c_void_p, C.c_void_p]
    kks = {}
    with tempfile.TemporaryDirectory() as td:
        for name, (text, n0, ns, pf) in kk_cases.items():
            path = os.path.join(td, name + ".txt")
            open(path, "w").write(text)
            N = ns or (len(text.strip().splitlines()) - text.startswith("#"))
            lams, nk = np.zeros(N), np.zeros(2 * N)
            got = r.ref_material_kk(path.encode(), n0, ns, float(pf), P(lams), P(nk))
            assert got == N, (name, got, N)
            kks[name] = {"text": text, "n0": n0, "n_samples": ns, "pf": pf, "lambda": lams.tolist(),
                         "n": nk[0::2].tolist(), "k": nk[1::2].tolist()}
    out["material_kk"] = kks

    for key, val in out.items():
        with open(os.path.join(out_dir, key + ".json"), "w") as fh:
            json.dump(val, fh, separators=(",", ":"))
    print("wrote", ", ".join(sorted(out)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
