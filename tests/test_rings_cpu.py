"""The oracle's ring-source drivers (the reference's --interpolate 1, 2, 3) on
the CPU: cases whose answer follows from the plain per-source oracle."""
import numpy as np

import oracle_lib
from bimsim_gb300 import abi, scenes


def scene():
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                        us_lut_r=96, us_lut_theta=120, focus=(0.5, -0.25, 0.0), amplitude=0.75)
    s = [(0.0, 0.0, 0.0, 2.0, 1.4, 0.04)]
    return p, abi.sphere_array(s), scenes.mc_waves(16, 0, 0.5, seed=3)


def per_source(p, arr, w, focus, amplitude):
    q = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(14, 0), resolution=16, padding=1,
                        us_lut_r=96, us_lut_theta=120, focus=focus, amplitude=amplitude)
    _, _, d, di = oracle_lib.simulate(q, *arr, w)
    return d, di


def test_one_ring_is_the_central_source():
    p, arr, w = scene()
    _, _, d, di = oracle_lib.simulate(p, *arr, w)
    for mode in (1, 3):
        D, Di = oracle_lib.simulate_rings(p, *arr, w, mode, 5, 1)
        assert np.array_equal(D, d) and np.array_equal(Di, di)


def test_one_point_per_ring_sums_the_first_sources():
    # with one point per ring nothing is rotated: central source + the source at (cos t, sin t) r, t = 2 pi
    p, arr, w = scene()
    _, _, d, di = oracle_lib.simulate(p, *arr, w)
    t = np.float32(np.float32(2) * np.float32(3.14159))
    for ring in (1, 2):
        f = (float(np.float32(np.cos(float(t))) * np.float32(ring)),
             float(np.float32(np.sin(float(t))) * np.float32(ring)), 0.0)
        dd, ddi = per_source(p, arr, w, f, 1.0)
        d, di = d + dd, di + ddi
    for mode in (1, 3):
        D, Di = oracle_lib.simulate_rings(p, *arr, w, mode, 1, 3)
        assert np.allclose(D, d, rtol=1e-14, atol=0) and np.allclose(Di, di, rtol=1e-14, atol=0)


def test_line_mode_single_radius():
    # one ring, one point: line[0] is the central source (amplitude 1) at the detector centre, the image is
    # that value at r = 0, (1 - r) times it for r < 1 and zero beyond
    p, arr, w = scene()
    d, di = per_source(p, arr, w, (0.5, -0.25, 0.0), 1.0)
    D, Di = oracle_lib.simulate_rings(p, *arr, w, 2, 1, 1)
    res = d.shape[0]
    uc = res // 2
    iu, iv = np.meshgrid(np.arange(res), np.arange(res))
    r = np.sqrt(((iu - uc) ** 2 + (iv - uc) ** 2).astype(np.float32))
    for img, ref in ((D, d), (Di, di)):
        expect = np.where(r < 1, (1 - r.astype(np.float64)) * ref[uc, uc], 0.0)
        assert np.allclose(img, expect, rtol=1e-15, atol=0)


def test_line_mode_tree_sum_drops_samples():
    # 3 samples per ring: the tree (step 1 only) adds samples 0 and 1; sample 2 never reaches the sum, so the
    # line and the image equal those of 2 samples at the same angles only when sample 2 adds nothing.  With
    # rings = 1 every sample sits at the centre: 3 points give 2 x the centre value, 4 points 4 x.
    p, arr, w = scene()
    d, _ = per_source(p, arr, w, (0.5, -0.25, 0.0), 1.0)
    uc = d.shape[0] // 2
    D3, _ = oracle_lib.simulate_rings(p, *arr, w, 2, 3, 1)
    D4, _ = oracle_lib.simulate_rings(p, *arr, w, 2, 4, 1)
    assert np.isclose(D3[uc, uc], 2 * d[uc, uc], rtol=1e-15) and np.isclose(D4[uc, uc], 4 * d[uc, uc], rtol=1e-15)
