"""Spectral sweep on the GPU (bs_sweep): every band equals a separate
bs_simulate at that wavelength bit for bit, matches the oracle within the
parity tolerances, and lands in the ENVI file as one band per wavelength."""
import os

import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import BS_IMG_ABSORBANCE, BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED, Context, abi, scenes

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL_MIXED_IMG = 1e-5


def small_sweep():
    lambdas = np.array([2.5, 4.0, 7.25, 12.5])
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                        lut_uf=True, us_lut_r=128, us_lut_theta=160, uf_lut_r=128)
    s = [(0.5, -0.5, 0.0, 2.0, 1.4, 0.0), (-4.5, 4.0, 0.5, 1.2, 1.4, 0.0)]
    mats = [scenes.lorentz_material(lambdas, seed=31), scenes.lorentz_material(lambdas, seed=32)]
    table = np.stack(mats, axis=1)
    return p, s, scenes.mc_waves(48, 0, 0.5, seed=12), lambdas, table


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec", [BS_PREC_FP64, BS_PREC_MIXED])
def test_sweep_bands_equal_single_runs_and_oracle(prec):
    p, s, w, lambdas, table = small_sweep()
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        imgs = ctx.sweep(lambdas, table, precision=prec)
    for l, lam in enumerate(lambdas):
        q = abi.make_params(lam=lam, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                            supersample=p.supersample, lut_uf=True, us_lut_r=128, us_lut_theta=160, uf_lut_r=128)
        sl = [(x, y, z, a, table[l, i].real, table[l, i].imag) for i, (x, y, z, a, _, _) in enumerate(s)]
        with Context(q) as ctx:
            ctx.set_spheres(sl)
            ctx.set_waves(w)
            ctx.simulate(prec)
            single = ctx.image(BS_IMG_INTENSITY)
        assert np.array_equal(imgs[l], single)
        arr, ns = abi.sphere_array(sl)
        _, _, D, _ = oracle_lib.simulate(q, arr, ns, w)
        tol = TOL64 if prec == BS_PREC_FP64 else TOL_MIXED_IMG
        # float32 images: compare at float32 resolution for the FP64 path
        assert rel(imgs[l].astype(np.float64), D) <= max(tol, 2e-7), (lam, rel(imgs[l].astype(np.float64), D))


def test_sweep_writes_one_envi_band_per_wavelength(tmp_path):
    p, s, w, lambdas, table = small_sweep()
    path = str(tmp_path / "sweep_a")
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        imgs = ctx.sweep(lambdas, table, precision=BS_PREC_MIXED, kind=BS_IMG_ABSORBANCE, envi_path=path,
                         band_as_nu=True)
    raw = np.fromfile(path, dtype="<f4").reshape(len(lambdas), 16, 16)
    assert np.array_equal(raw, imgs)
    hdr = open(path + ".hdr").read()
    assert "bands = 4" in hdr
    wl = hdr.split("wavelength = {")[1].split("}")[0]
    vals = [float(v) for v in wl.replace("\n", " ").split(",")]
    assert np.allclose(vals, 1e4 / lambdas, rtol=1e-6)  # band value 1e4/lambda with band_as_nu
