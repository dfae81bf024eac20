"""Pin the oracle to the reference: golden vectors produced by the reference's own
host code (tests/golden/make_golden.py, oracle/_ref), checked on CPU."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import oracle_lib
from oracle_lib import P
from bimsim_gb300 import abi


def _finite(a):
    a = np.asarray(a, dtype=np.float64)
    return np.isfinite(a) & (np.abs(a) < 1e300)


def test_bessel_real(oracle, golden):
    for case in golden("bessel_real"):
        N, x = case["N"], case["x"]
        j = np.zeros(N + 1)
        y = np.zeros(N + 1)
        oracle.bso_sbessel_real(N, x, P(j), P(y))
        for mine, ref in ((j, np.array(case["j"])), (y, np.array(case["y"]))):
            m = _finite(ref)
            np.testing.assert_allclose(mine[m], ref[m], rtol=2e-9, atol=1e-13, err_msg=f"N={N} x={x}")


def test_bessel_complex(oracle, golden):
    for case in golden("bessel_complex"):
        N = case["N"]
        zr, zi = case["z"]
        out = [np.zeros(2 * N + 2) for _ in range(4)]
        oracle.bso_sbessel_complex(N, zr, zi, 1, *[P(t) for t in out])
        names = ["j", "y", "jp", "yp"]
        for name, mine in zip(names, out):
            if name in ("y", "yp") and zi != 0:
                continue  # y at a complex argument (k n a) is never used by the path
            ref = np.array(case[name])
            mine = mine[0::2] + 1j * mine[1::2]
            ref = ref[0::2] + 1j * ref[1::2]
            m = np.isfinite(ref) & (np.abs(ref) < 1e300)
            np.testing.assert_allclose(mine[m], ref[m], rtol=2e-9, atol=1e-13, err_msg=f"{name} N={N} z={zr}+{zi}j")


def test_bessel_typo_matters(oracle):
    """cbessjy.cpp:541 changes y_0 for |z| > 12; the restatement reproduces it."""
    N = 4
    a = [np.zeros(2 * N + 2) for _ in range(4)]
    b = [np.zeros(2 * N + 2) for _ in range(4)]
    oracle.bso_sbessel_complex(N, 13.5, 0.0, 1, *[P(t) for t in a])
    oracle.bso_sbessel_complex(N, 13.5, 0.0, 0, *[P(t) for t in b])
    assert abs(a[1][0] - b[1][0]) > 1e-3          # y_0 differs by j_0
    assert abs(a[1][2] - b[1][2]) < 1e-15         # y_1 exact in both


def test_calc_nl(oracle, golden):
    for a, lam, nl in golden("calc_nl"):
        assert oracle.bso_calc_nl(a, lam) == nl, (a, lam)


def test_mie_against_reference_storage(oracle, golden):
    for case in golden("mie"):
        Nl = case["Nl"]
        assert oracle.bso_calc_nl(case["a"], case["lambda"]) == Nl
        A = np.zeros(2 * Nl + 2)
        B = np.zeros(2 * Nl + 2)
        oracle.bso_mie(case["k"], case["a"], case["n"][0], case["n"][1], Nl, P(A), P(B))
        for mine, ref in ((A, case["A"]), (B, case["B"])):
            mine = mine[0::2] + 1j * mine[1::2]
            ref = np.array([complex(*v) for v in ref])
            # the reference rounds each component to float
            err = np.abs(mine - ref)
            tol = 1.5e-7 * np.abs(ref) + 1e-12
            assert np.all(err <= tol), (case["a"], case["lambda"], np.max(err / np.abs(ref)))


def test_sphere_tables(oracle, golden):
    """Hankel (j, y)(k r) and internal j(k n r) tables of sphere.cpp:99-203."""
    f = np.float32
    for t in golden("sphere_tables"):
        Nl, rR, aR = t["Nl"], t["rR"], t["aR"]
        a, k = f(t["a"]), f(t["k"])
        r0 = max(a, f(t["dmin"]))
        dr = f((f(t["dmax"]) - r0) / f(rR - 1))
        h = np.array([complex(*v) for v in t["h"]]).reshape(rR, Nl + 1)
        for ir in range(rR):
            r = f(f(ir) * dr + r0)
            j = np.zeros(Nl + 1)
            y = np.zeros(Nl + 1)
            oracle.bso_sbessel_real(Nl, float(f(k * r)), P(j), P(y))
            np.testing.assert_allclose(j + 1j * y, h[ir], rtol=2e-6, atol=1e-30)
        jt = np.array([complex(*v) for v in t["j"]]).reshape(aR, Nl + 1)
        n = complex(f(t["n"][0]), f(t["n"][1]))
        da = f(a / f(aR - 1))
        assert jt[0, 0] == 1 and np.all(jt[0, 1:] == 0)
        for ia in range(1, aR):
            r = f(f(ia) * da)
            knr = complex(np.complex64(np.complex64(k * n) * r))
            out = [np.zeros(2 * Nl + 2) for _ in range(4)]
            oracle.bso_sbessel_complex(Nl, knr.real, knr.imag, 1, *[P(x) for x in out])
            mine = out[0][0::2] + 1j * out[0][1::2]
            np.testing.assert_allclose(mine, jt[ia], rtol=2e-6, atol=1e-30)


def test_uf_table(oracle, golden):
    """Incident-field Bessel table of nearfield.cpp:222-283 (NaN/Inf patched)."""
    f = np.float32
    for t in golden("uf_table"):
        m, dR = t["m"], t["dR"]
        k = f(f(2) * f(3.14159) / f(t["lambda"]))
        dmin, dmax = f(t["dmin"]), f(t["dmax"])
        dr = f((dmax - dmin) / f(dR - 1))
        ref = np.array(t["j"]).reshape(dR, m + 1)
        for i in range(dR):
            d = f(f(i) * dr + dmin)
            kd = float(f(k * d))
            j = np.zeros(m + 1)
            y = np.zeros(m + 1)
            oracle.bso_sbessel_real(m, kd, P(j), P(y))
            bad = ~np.isfinite(j)
            j[bad] = 0.0
            if kd == 0:
                j[0] = 1.0
            np.testing.assert_allclose(j, ref[i], rtol=2e-6, atol=1e-30)


def test_glibc_rand(oracle, golden):
    ref = np.array(golden("rand_seed0"), dtype=np.int32)
    out = np.zeros(len(ref), dtype=np.int32)
    oracle.bso_glibc_rand(0, len(ref), P(out))
    assert np.array_equal(out, ref)


def test_mc_sample(oracle, golden):
    for case in golden("mc"):
        k = np.array(case["k"], dtype=np.float64)
        out = np.zeros(3 * case["nk"])
        oracle.bso_mc_sample(case["nk"], P(k), case["na"][0], case["na"][1], P(out))
        # bit-identical on the machine that made the vectors; libm float may differ by an ulp elsewhere
        np.testing.assert_allclose(out, case["dirs"], rtol=0, atol=2e-7)


def test_quad_distances(oracle, golden):
    for q in golden("quad"):
        pad = (q["scale"] - 1) // 2
        p = abi.make_params(plane=(q["pmin"], q["pmax"], q["normal"]), padding=pad, resolution=8, supersample=1)
        s = abi.Sphere(*q["p"], 1.0, 1.4, 0.0)
        g = oracle_lib.sphere_geom(p, s)
        assert g.d_min == pytest.approx(q["dmin"], rel=1e-5, abs=1e-5)
        assert g.d_max == pytest.approx(q["dmax"], rel=1e-6)


def test_envi_bytes(oracle, golden):
    e = golden("envi")
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "band")
        b1 = np.array(e["b1"], dtype=np.float32)
        b2 = np.array(e["b2"], dtype=np.float32)
        oracle.bso_envi_add_band(path.encode(), P(b1), e["samples"], e["lines"], e["wl"][0], 0)
        assert open(path + ".hdr").read() == e["hdr_1"]
        assert open(path, "rb").read().hex() == e["dat_1"]
        oracle.bso_envi_add_band(path.encode(), P(b2), e["samples"], e["lines"], e["wl"][1], 1)
        assert open(path + ".hdr").read() == e["hdr_2"]
        assert open(path, "rb").read().hex() == e["dat_2"]


@pytest.mark.parametrize("n", [1, 2, 12, 96, 160, 384, 97, 127, 250])
def test_oracle_fft(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    buf = np.ascontiguousarray(x).view(np.float64).copy()
    oracle.bso_fft(n, -1, P(buf))
    np.testing.assert_allclose(buf.view(np.complex128), np.fft.fft(x), rtol=0, atol=1e-12 * n)
    oracle.bso_fft(n, +1, P(buf))
    np.testing.assert_allclose(buf.view(np.complex128) / n, x, rtol=0, atol=1e-12 * n)


def test_live_reference_bessel(oracle, ref_lib):
    """Where the reference was built here, compare on a denser grid too."""
    vp = C.c_void_p
    ref_lib.ref_bessjyv_sph.argtypes = [C.c_int, C.c_double, vp, vp]
    rng = np.random.default_rng(7)
    for x in rng.uniform(0.2, 250.0, 60):
        N = 40
        a, b, c, d = (np.zeros(N + 1) for _ in range(4))
        oracle.bso_sbessel_real(N, x, P(a), P(b))
        ref_lib.ref_bessjyv_sph(N, x, P(c), P(d))
        for mine, ref in ((a, c), (b, d)):
            m = _finite(ref)
            np.testing.assert_allclose(mine[m], ref[m], rtol=2e-9, atol=1e-13)
