"""Kramers-Kronig real index of a material file (bs_material_kk, the
reference's material::computeN, rts/optics/material.h:257-432): the oracle's
FFT restatement against numpy and against the reference's own routine
(golden material_kk.json, recorded from material<double>::computeN compiled in
place over an FFTW stand-in) on the CPU; the GPU routine against the oracle and
against the same goldens."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import BimsimError, lib

PI_F = float(np.float32(3.14159))


def lorentz_file(path, n=120, lam0=6.0, width=0.3, peak=0.08):
    """A microns,n,k table with one Lorentzian absorption band (kappa), n = 1.5."""
    lam = np.linspace(2.5, 12.5, n)
    kap = peak * width ** 2 / ((lam - lam0) ** 2 + width ** 2)
    path.write_text("".join(f"{l:.6f} 1.5 {k:.8f}\n" for l, k in zip(lam, kap)))
    return lam, kap


def oracle_kk(lam, kap, n0, pf):
    out = np.zeros(len(lam))
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    kap = np.ascontiguousarray(kap, dtype=np.float64)
    oracle_lib.load().bso_kk_transform(len(lam), pf, n0, lam.ctypes.data_as(C.c_void_p),
                                       kap.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
    return out


def numpy_kk(lam, kap, n0, pf):
    """The same steps with numpy's FFT (forward e^-i, inverse unnormalised then / M)."""
    N = len(lam)
    M = N * pf
    k = np.array([np.float32(2 * np.float32(PI_F) / l) for l in lam], dtype=np.float64)
    alpha = np.array([np.float32(kk * np.float64(2 * np.float32(ki))) for kk, ki in zip(kap, k)], dtype=np.float64)
    chi2 = np.zeros(M, dtype=np.complex128)
    chi2[:N] = -alpha * (n0 / k)
    F = np.fft.fft(chi2)
    f = np.arange(M)
    F = np.where(f == 0, 0, np.where(f < M / 2.0, 1j * F, -1j * F))
    chi1 = np.fft.ifft(F)  # already / M
    return chi1[:N].real / (2 * n0) + n0


@pytest.mark.parametrize("pf", [1, 2, 3])
def test_oracle_transform_matches_numpy(pf):
    rng = np.random.default_rng(3)
    lam = np.sort(rng.uniform(2.5, 12.5, 97))
    kap = rng.uniform(0, 0.1, 97)
    a, b = oracle_kk(lam, kap, 1.45, pf), numpy_kk(lam, kap, 1.45, pf)
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b - 1.45))


KK_GOLDEN = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "material_kk.json")))


@pytest.mark.parametrize("name", sorted(KK_GOLDEN))
def test_oracle_transform_matches_the_references_computeN(name):
    """Given the reference's own resampled kappa, the oracle's transform gives its n (to rounding)."""
    g = KK_GOLDEN[name]
    lam, kap, n = np.array(g["lambda"]), np.array(g["k"]), np.array(g["n"])
    assert np.all(np.diff(lam) > 0) and np.max(np.abs(n - g["n0"])) > 1e-3
    o = oracle_kk(lam, kap, g["n0"], g["pf"])
    assert np.max(np.abs(o - n)) <= 1e-13 * np.max(np.abs(n - g["n0"])), np.max(np.abs(o - n))


def _sin_pi_ratio(a, M):
    """sin(pi a / M) with a reduced in integers to a ratio in [0, 1/2], as kk_kernel_g does."""
    r = a % (2 * M)
    sign = np.where(r >= M, -1.0, 1.0)
    r = np.where(r >= M, r - M, r)
    r = np.where(2 * r > M, M - r, r)
    return sign * np.sin(np.pi * (r / M))


@pytest.mark.parametrize("M", [2, 7, 8, 300, 1001, 16384 * 16 - 1, 16384 * 16])
def test_closed_form_convolution_kernel(M):
    """The GPU routine convolves with g(m) = -(2/M) sin(K t) sin((K+1) t) / sin(t), t = pi m / M,
    K = ceil(M/2) - 1: the real part of the inverse FFT of the reference's multiplier (i below M/2,
    -i from M/2, 0 at DC), to an ulp of its largest value at every m."""
    m = np.arange(1, M, dtype=np.int64)
    K = (M + 1) // 2 - 1
    g = np.zeros(M)
    g[1:] = -2.0 * (_sin_pi_ratio(K * m, M) * _sin_pi_ratio((K + 1) * m, M) / _sin_pi_ratio(m, M)) / M
    f = np.arange(M)
    H = np.where(f == 0, 0, np.where(f < M / 2.0, 1j, -1j))
    ref = np.fft.ifft(H).real
    assert np.max(np.abs(g - ref)) <= 4e-16 * max(np.max(np.abs(ref)), 1e-300) + 1e-17


def test_oracle_absorption_band_gives_dispersion():
    # a Lorentzian band in kappa gives the familiar dispersive wiggle in n: above n0 on the long-wavelength
    # side of the band and below it on the short side
    nu = np.linspace(4000, 800, 400)
    lam = 1e4 / nu
    kap = 0.05 * 40 ** 2 / ((nu - 1700) ** 2 + 40 ** 2)
    n = oracle_kk(lam, kap, 1.5, 2)
    i = np.argmin(np.abs(nu - 1700))
    assert n[i + 10] > 1.5 > n[i - 10]


@pytest.mark.gpu
@pytest.mark.parametrize("n_samples,pf", [(0, 2), (256, 2), (300, 3), (64, 1), (16384, 16), (16384, 3)])
def test_gpu_kk_matches_oracle(tmp_path, n_samples, pf):
    path = tmp_path / "band.txt"
    lam_f, _ = lorentz_file(path)
    lam, n = lib.material_kk(path, 1.5, n_samples, pf)
    N = n_samples or len(lam_f)
    assert len(lam) == N and np.all(np.diff(lam) > 0)
    nu = 1e4 / lam
    assert np.allclose(np.diff(nu), (nu[-1] - nu[0]) / (N - 1), rtol=1e-9)  # even in wavenumber
    # kappa is the file's, interpolated in double precision as material<double>::getN does (function.h:44-75:
    # the first row with a larger wavelength bounds the interval, the weights are swapped, the ends clamp)
    rows = np.array([[float(x) for x in line.split()] for line in path.read_text().splitlines()])
    fl, fk = rows[:, 0], rows[:, 2]
    i = np.searchsorted(fl, lam, side="right")
    inner = (i > 0) & (i < len(fl))
    ii = np.clip(i, 1, len(fl) - 1)
    a = (lam - fl[ii - 1]) / (fl[ii] - fl[ii - 1])
    k64 = np.where(inner, fk[ii - 1] * a + fk[ii] * (1.0 - a), np.where(i == 0, fk[0], fk[-1]))
    assert np.max(np.abs(n.imag - k64)) <= 1e-15 * np.max(np.abs(k64))
    ref = oracle_kk(lam, n.imag, 1.5, pf)
    assert np.max(np.abs(n.real - ref)) <= 1e-10 * np.max(np.abs(ref - 1.5)), np.max(np.abs(n.real - ref))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(KK_GOLDEN))
def test_gpu_kk_matches_the_references_computeN(tmp_path, name):
    """bs_material_kk against the reference's own material<double>::computeN: the same wavelength grid and
    kappa (bit-identical), n to the transform's rounding."""
    g = KK_GOLDEN[name]
    path = tmp_path / "m.txt"
    path.write_text(g["text"])
    lam, n = lib.material_kk(path, g["n0"], g["n_samples"], g["pf"])
    ref_n = np.array(g["n"])
    np.testing.assert_allclose(lam, g["lambda"], rtol=1e-15, atol=0)
    assert np.array_equal(n.imag, np.array(g["k"]))
    assert np.max(np.abs(n.real - ref_n)) <= 1e-10 * np.max(np.abs(ref_n - g["n0"]))


@pytest.mark.gpu
def test_gpu_kk_rejects_bad_arguments(tmp_path):
    path = tmp_path / "band.txt"
    lorentz_file(path)
    with pytest.raises(BimsimError):
        lib.material_kk(path, 1.5, 16385, 2)
    with pytest.raises(BimsimError):
        lib.material_kk(tmp_path / "missing.txt", 1.5)
    with pytest.raises(BimsimError):
        lib.material_kk(path, 1.5, 64, 17)
