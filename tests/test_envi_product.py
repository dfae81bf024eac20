"""The product's ENVI output (bs_write_envi on a context's detector images) byte for byte against
the oracle's restatement of the reference's EnviFile (bso_envi_add_band), which the CPU suite pins to
the reference's own bytes: one band written, a second appended, with the --nu band value 1e4/lambda
(fileout.cu:58-61)."""
import os

import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import BS_IMG_ABSORBANCE, BS_IMG_INTENSITY, BS_PREC_MIXED, Context, abi, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("as_nu", [False, True])
def test_write_envi_bytes_equal_the_oracle_writer(tmp_path, as_nu):
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                        us_lut_theta=200)
    s = [(0, 0, 0, 2.5, 1.4, 0.05), (4.5, -3.0, 0.8, 1.1, 1.55, 0.01)]
    orc = oracle_lib.load()
    mine = {k: str(tmp_path / f"mine_{k}") for k in ("int", "abs")}
    theirs = {k: str(tmp_path / f"oracle_{k}") for k in ("int", "abs")}
    with Context(p) as ctx:
        ctx.set_spheres(s)
        for band, lam in enumerate((3.0, 3.5)):
            p.lambda_ = lam
            ctx.set_params(p)
            ctx.set_waves(scenes.mc_waves(24, 0, 0.5, seed=3 + band))
            ctx.simulate(BS_PREC_MIXED)
            value = 1e4 / lam if as_nu else lam
            for key, kind in (("int", BS_IMG_INTENSITY), ("abs", BS_IMG_ABSORBANCE)):
                ctx.write_envi(kind, mine[key], band > 0, value)
                img = np.ascontiguousarray(ctx.image(kind), dtype=np.float32)
                rc = orc.bso_envi_add_band(theirs[key].encode(), oracle_lib.P(img), p.resolution, p.resolution,
                                           value, 1 if band > 0 else 0)
                assert rc == 0
    for key in mine:
        assert open(mine[key] + ".hdr").read() == open(theirs[key] + ".hdr").read()
        assert open(mine[key], "rb").read() == open(theirs[key], "rb").read()
        assert os.path.getsize(mine[key]) == 2 * 4 * p.resolution * p.resolution
        assert "bands = 2" in open(mine[key] + ".hdr").read()
