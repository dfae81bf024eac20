"""Spectral-sweep inputs without a GPU: the Lorentzian material model and its
Kramers-Kronig index change (discrete Hilbert transform) against the
analytic transform of a single band."""
import numpy as np

from bimsim_gb300 import scenes


def test_single_band_kk_matches_analytic_transform():
    nu = np.linspace(1.0 / 40.0, 1.0, 1 << 16)
    c, w, pk = 6.0, 0.1, 0.08
    kap = scenes.lorentz_kappa(nu, [c], [w], [pk])
    dn = scenes.hilbert_dn(nu, kap)
    nc, g = 1.0 / c, 0.5 * w / (c * c)
    exact = -pk * g * (nu - nc) / ((nu - nc) ** 2 + g * g)
    band = np.abs(nu - nc) < 50 * g
    assert np.max(np.abs(dn[band] - exact[band])) < 2e-3 * pk
    # normal dispersion: index raised below the band (lower wavenumber), lowered above
    assert dn[np.argmin(np.abs(nu - (nc - g)))] > 0 > dn[np.argmin(np.abs(nu - (nc + g)))]


def test_material_and_config3_shapes():
    lam = np.linspace(2.5, 12.5, 512)
    n = scenes.lorentz_material(lam, seed=30)
    assert n.shape == (512,)
    assert np.all(n.imag >= 0) and n.imag.max() <= 0.1 + 1e-12
    assert np.all(np.abs(n.real - 1.45) < 0.1)
    p, s, w, lambdas, table = scenes.config3(n_lambda=16, resolution=64, n_spheres=6, samples=32)
    assert table.shape == (16, 6) and len(s) == 6 and w.shape == (32, 3)
    assert np.array_equal(table[:, 0], table[:, 3])  # sphere i uses material i % 3
