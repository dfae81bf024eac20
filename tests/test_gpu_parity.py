"""GPU path vs the oracle, through the C ABI.

Tolerances (relative L2, ||gpu - oracle|| / ||oracle||):
  * FP64 path: 1e-10 on every output (near fields, Mie coefficients, LUTs, detector images)
  * mixed path: 1e-5 on the detector images and 1e-4 on the near field
"""
import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import (BS_FIELD_INCIDENT, BS_FIELD_TOTAL, BS_IMG_ABSORBANCE, BS_IMG_INCIDENT, BS_IMG_INTENSITY,
                          BS_IMG_TRANSMITTANCE, BS_PREC_FP64, BS_PREC_MIXED, Context, abi, scenes)

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL_MIXED_IMG = 1e-5
TOL_MIXED_FIELD = 1e-4


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) / max(np.linalg.norm(np.asarray(b).ravel()), 1e-300))


def scene(name):
    w = scenes.mc_waves
    if name == "lut":
        p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                            us_lut_theta=200)
        s = [(0, 0, 0, 2.5, 1.4, 0.05), (4.5, -3.0, 0.8, 1.1, 1.55, 0.01), (-5.0, 4.0, -1.5, 1.8, 1.25, 0.0)]
        return p, s, w(40, 0, 0.5, seed=3)
    if name == "lut_ufLUT":
        p = abi.make_params(lam=3.0, condenser=(0.1, 0.5), objective=(0.05, 0.45), xy=(14, 0.5), resolution=16,
                            padding=1, lut_uf=True, us_lut_r=150, us_lut_theta=128, uf_lut_r=200)
        s = [(1.0, 0.5, 0.0, 2.0, 1.45, 0.03), (-4.0, -3.5, 0.2, 1.3, 1.3, 0.02)]
        return p, s, w(32, 0.1, 0.5, seed=4)
    if name == "direct_cfg1":
        # config 1 at reduced size: ka = 12.57 > 12 exercises cbessjy.cpp:541
        p = abi.make_params(lam=2.5, condenser=(0, 0.5), objective=(0, 0.5), xy=(20, 0), resolution=12, padding=2,
                            lut_us=False)
        return p, [(0, 0, 0, 5.0, 1.4, 0.05)], w(24, 0, 0.5, seed=1)
    if name == "direct_multi":
        p = abi.make_params(lam=3.0, condenser=(0, 0.6), objective=(0, 0.6), xy=(16, 0), resolution=16, padding=1,
                            lut_us=False, lut_uf=True)
        s = [(0.3, -0.2, 0, 2.2, 1.5, 0.04), (5.0, 4.0, 1.0, 1.0, 1.3, 0.0)]
        return p, s, w(20, 0, 0.6, seed=5)
    if name == "direct_large":
        # ka = 62.8 (81 orders) through the sphere's centre plane: the harmonic recurrences to l = 81
        p = abi.make_params(lam=2.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(60, 0), resolution=16, padding=1,
                            lut_us=False)
        return p, [(1.0, -2.0, 0.0, 20.0, 1.4, 0.02)], w(24, 0, 0.5, seed=13)
    if name == "direct_oblique":
        # oblique incidence and an xz plane: pixel and wave directions far from the harmonic axis
        k = (np.sin(0.4), 0.2, np.cos(0.4))
        k = tuple(np.array(k) / np.linalg.norm(k))
        p = abi.make_params(lam=2.5, k_dir=k, condenser=(0.1, 0.45), objective=(0, 0.5),
                            plane=((-6, 0, -6), (6, 0, 6), (0, -1, 0)), resolution=12, padding=1, lut_us=False)
        return p, [(0.5, 1.0, -0.5, 1.6, 1.35, 0.02), (-2.0, -1.5, 2.0, 1.1, 1.5, 0.0)], w(28, 0.1, 0.45, seed=16,
                                                                                           kdir=k)
    if name == "plane_wave":
        p = abi.make_params(lam=2.0, condenser=(0, 0.5), objective=(0, 0.8), xy=(12, 0), resolution=16, padding=1,
                            plane_wave=True, us_lut_theta=256)
        return p, [(0.5, 0.0, 0.0, 2.0, 1.4, 0.02)], None
    if name == "oblique_xz":
        k = (np.sin(0.3), 0.0, np.cos(0.3))
        p = abi.make_params(lam=2.5, k_dir=k, condenser=(0, 0.4), objective=(0, 0.5),
                            plane=((-6, 0, -6), (6, 0, 6), (0, -1, 0)), resolution=12, padding=1, us_lut_theta=180)
        return p, [(0.0, 1.0, 0.0, 1.6, 1.35, 0.02)], w(28, 0, 0.4, seed=6, kdir=k)
    if name == "vector":
        p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(12, 0), resolution=12, padding=1,
                            scalar=False)
        return p, [(0, 0, 0, 2.0, 1.4, 0.05)], w(16, 0, 0.5, seed=7)
    if name == "no_spheres":
        p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(12, 0), resolution=12, padding=1)
        return p, [], w(16, 0, 0.5, seed=8)
    if name == "supersample":
        # s/res = 6/6 > lambda/2 -> ss = ceil(2 s / (res lambda)) = 2 (arguments.h:411-418)
        p = abi.make_params(lam=1.5, condenser=(0, 0.5), objective=(0, 0.5), xy=(6, 0), resolution=6, padding=1,
                            us_lut_theta=128)
        assert p.supersample == 2
        return p, [(0.2, 0.1, 0.0, 1.0, 1.4, 0.05)], w(16, 0, 0.5, seed=9)
    if name == "lut_staged":
        # 64 x 64 pixels, 4 x 4 tiles of 16 x 16, most of them clear of both spheres: their LUT windows are
        # staged in shared memory by the mixed kernel, the tiles touching a sphere use the texture path
        p = abi.make_params(lam=2.5, condenser=(0, 0.5), objective=(0, 0.5), xy=(48, 0), resolution=64, padding=1,
                            us_lut_r=100, us_lut_theta=300)
        s = [(-6.0, 5.0, 0.0, 2.0, 1.4, 0.04), (9.0, -8.0, 1.0, 1.4, 1.5, 0.01)]
        return p, s, w(256, 0, 0.5, seed=10)
    if name == "lut_many_rows":
        # 20 spheres x 30 000 table rows: their coefficient rows are computed in two batches (2^19 rows each)
        p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                            us_lut_r=30000, us_lut_theta=16)
        s = scenes.random_spheres(20, 16.0, 0.3, 0.9, seed=12)
        return p, s, w(24, 0, 0.5, seed=11)
    raise KeyError(name)


ALL = ["lut", "lut_ufLUT", "direct_cfg1", "direct_multi", "direct_large", "direct_oblique", "plane_wave",
       "oblique_xz", "vector", "no_spheres", "supersample", "lut_staged", "lut_many_rows"]
_oracle_cache = {}


def oracle_result(name):
    if name not in _oracle_cache:
        p, s, waves = scene(name)
        arr, ns = abi.sphere_array(s)
        w = waves if waves is not None else np.zeros((0, 3))
        _oracle_cache[name] = oracle_lib.simulate(p, arr, ns, w)
    return _oracle_cache[name]


def run_gpu(name, prec, budget=0, staging=0, chunk=0):
    p, s, waves = scene(name)
    ctx = Context(p)
    ctx.set_spheres(s)
    if waves is not None:
        ctx.set_waves(waves)
    if budget:
        ctx.set_lut_budget(budget)
    if staging:
        ctx.set_lut_staging(staging)
    if chunk:
        ctx.set_lut_wave_chunk(chunk)
    ctx.simulate(prec)
    out = dict(U=ctx.field(BS_FIELD_TOTAL), Uf=ctx.field(BS_FIELD_INCIDENT),
               D=ctx.image(BS_IMG_INTENSITY, f64=True), Di=ctx.image(BS_IMG_INCIDENT, f64=True),
               A=ctx.image(BS_IMG_ABSORBANCE, f64=True), T=ctx.image(BS_IMG_TRANSMITTANCE, f64=True),
               stats=ctx.stats())
    ctx.close()
    return out


@pytest.mark.parametrize("name", ALL)
def test_fp64_matches_oracle(name):
    U, Uf, D, Di = oracle_result(name)
    g = run_gpu(name, BS_PREC_FP64)
    errs = {"Uf": rel(g["Uf"], Uf), "U": rel(g["U"], U), "D": rel(g["D"], D), "Di": rel(g["Di"], Di)}
    assert max(errs.values()) <= TOL64, errs
    assert g["stats"].kernel_launches > 0


@pytest.mark.parametrize("name", ALL)
def test_mixed_matches_oracle(name):
    U, Uf, D, Di = oracle_result(name)
    g = run_gpu(name, BS_PREC_MIXED)
    img = {"D": rel(g["D"], D), "Di": rel(g["Di"], Di)}
    fld = {"U": rel(g["U"], U), "Uf": rel(g["Uf"], Uf)}
    assert max(img.values()) <= TOL_MIXED_IMG, (img, fld)
    assert max(fld.values()) <= TOL_MIXED_FIELD, (img, fld)


def test_mixed_lut_kernel_uses_both_table_paths():
    """The staged (shared-memory) and texture paths of the mixed LUT kernel both run in the
    lut_staged scene; the parity tests above cover their values."""
    g = run_gpu("lut_staged", BS_PREC_MIXED, staging=1)
    st = g["stats"]
    p, s, w = scene("lut_staged")
    tiles = (oracle_lib.geom(p).R + 15) // 16
    # tiles of 16 x 16 near-field pixels x spheres x wave chunks (64, 32 or 16 waves, chosen per run)
    ch = st.lut_wave_chunk
    assert ch in (16, 32, 64)
    assert st.lut_chunks_total == tiles * tiles * len(s) * ((len(w) + ch - 1) // ch)
    assert 0 < st.lut_chunks_staged < st.lut_chunks_total, (st.lut_chunks_staged, st.lut_chunks_total)
    g64 = run_gpu("lut_staged", BS_PREC_FP64)
    assert g64["stats"].lut_chunks_total == 0


@pytest.mark.parametrize("chunk", [16, 64])
@pytest.mark.parametrize("name", ["lut", "lut_ufLUT", "lut_staged", "oblique_xz", "supersample"])
def test_staged_and_texture_kernels_give_identical_bits(name, chunk):
    a = run_gpu(name, BS_PREC_MIXED, staging=1, chunk=chunk)
    b = run_gpu(name, BS_PREC_MIXED, staging=2, chunk=chunk)
    assert a["stats"].lut_wave_chunk == b["stats"].lut_wave_chunk == chunk
    assert b["stats"].lut_chunks_staged == 0
    assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["D"], b["D"])


@pytest.mark.parametrize("chunk", [16, 32, 64])
def test_wave_groups_with_a_short_last_chunk(chunk):
    """150 waves: full chunks plus one short group (22 or 6 waves) last, staged and texture kernels
    alike, within the mixed tolerance of the oracle."""
    p, s, _ = scene("lut_staged")
    w = scenes.mc_waves(150, 0, 0.5, seed=17)
    U, _, D, _ = oracle_lib.simulate(p, *abi.sphere_array(s), w)
    out = {}
    for staging in (1, 2):
        with Context(p) as ctx:
            ctx.set_spheres(s)
            ctx.set_waves(w)
            ctx.set_lut_staging(staging)
            ctx.set_lut_wave_chunk(chunk)
            ctx.simulate(BS_PREC_MIXED)
            out[staging] = (ctx.field(BS_FIELD_TOTAL), ctx.image(BS_IMG_INTENSITY, f64=True), ctx.stats())
    assert out[1][2].lut_chunks_staged > 0
    assert np.array_equal(out[1][0], out[2][0])
    assert rel(out[1][0], U) <= TOL_MIXED_FIELD and rel(out[1][1], D) <= TOL_MIXED_IMG


def test_wave_chunk_choice():
    """The run's chunk is one of 64, 32, 16 (64 when the texture-only kernel runs); a fixed chunk is kept;
    every chunk size gives the oracle's result within the mixed tolerance."""
    auto = run_gpu("lut_staged", BS_PREC_MIXED)["stats"]
    assert auto.lut_wave_chunk in (16, 32, 64)
    tex = run_gpu("lut_staged", BS_PREC_MIXED, staging=2)["stats"]
    assert tex.lut_wave_chunk == 64
    U, Uf, D, Di = oracle_result("lut_staged")
    for ch in (16, 32, 64):
        g = run_gpu("lut_staged", BS_PREC_MIXED, chunk=ch)
        assert g["stats"].lut_wave_chunk == ch
        assert rel(g["U"], U) <= TOL_MIXED_FIELD and rel(g["D"], D) <= TOL_MIXED_IMG, (ch, rel(g["U"], U), rel(g["D"], D))


def test_kernel_choice_model_tracks_the_staged_fraction():
    """The host model that picks the staged kernel predicts the fraction the kernel then stages."""
    g = run_gpu("lut_staged", BS_PREC_MIXED, staging=1)
    st = g["stats"]
    measured = st.lut_chunks_staged / st.lut_chunks_total
    assert abs(st.lut_staged_predicted - measured) < 0.2, (st.lut_staged_predicted, measured)
    auto = run_gpu("lut_staged", BS_PREC_MIXED)["stats"]
    threshold = 0.3 if auto.lut_wave_chunk >= 64 else 0.7  # the staged kernel's break-even fraction per chunk
    assert (auto.lut_chunks_staged > 0) == (auto.lut_staged_predicted >= threshold)


def test_mixed_rejects_tables_beyond_the_texture_limit():
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                        us_lut_r=70000, us_lut_theta=16)
    with Context(p) as ctx:
        ctx.set_spheres([(0, 0, 0, 2.0, 1.4, 0.05)])
        ctx.set_waves(scenes.mc_waves(8, 0, 0.5, seed=1))
        with pytest.raises(Exception) as e:
            ctx.simulate(BS_PREC_MIXED)
        assert "texture limit" in str(e.value)
        ctx.simulate(BS_PREC_FP64)  # the FP64 path keeps its tables in linear memory


def test_images_are_derived_consistently():
    _, _, D, Di = oracle_result("lut")
    g = run_gpu("lut", BS_PREC_FP64)
    with np.errstate(divide="ignore", invalid="ignore"):
        assert rel(g["A"], -np.log10(D / Di)) <= TOL64
        assert rel(g["T"], D / Di) <= TOL64


def test_zero_spheres_total_equals_incident():
    g = run_gpu("no_spheres", BS_PREC_FP64)
    assert np.array_equal(g["U"], g["Uf"])
    assert np.array_equal(g["D"], g["Di"])


def test_mie_coefficients_fp64():
    p, s, waves = scene("direct_cfg1")
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(waves)
        ctx.simulate(BS_PREC_FP64)
        nl = oracle_lib.load().bso_calc_nl(s[0][3], p.lambda_)
        A, B = ctx.mie(0, nl)
    Ao = np.zeros(2 * nl + 2)
    Bo = np.zeros(2 * nl + 2)
    g = oracle_lib.geom(p)
    oracle_lib.load().bso_mie(g.kmag, s[0][3], s[0][4], s[0][5], nl, oracle_lib.P(Ao), oracle_lib.P(Bo))
    assert rel(A, Ao.view(np.complex128)) <= 1e-12
    assert rel(B, Bo.view(np.complex128)) <= 1e-12


@pytest.mark.parametrize("prec,tol", [(BS_PREC_FP64, 1e-12), (BS_PREC_MIXED, 1e-6)])
def test_lut_tables(prec, tol):
    p, s, waves = scene("lut")
    lib = oracle_lib.load()
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(waves)
        ctx.simulate(prec)
        for i, sp in enumerate(s):
            sg = oracle_lib.sphere_geom(p, abi.Sphere(*sp))
            usp = np.zeros(2 * sg.dR * sg.thetaR)
            uip = np.zeros(2 * sg.aR * sg.thetaR)
            lib.bso_sphere_luts(oracle_lib.C.byref(p), oracle_lib.C.byref(abi.Sphere(*sp)), oracle_lib.P(usp),
                                oracle_lib.P(uip))
            gu = ctx.lut(i, 0, sg.dR, sg.thetaR)
            gi = ctx.lut(i, 1, sg.aR, sg.thetaR)
            assert rel(gu, usp.view(np.complex128).reshape(sg.dR, sg.thetaR)) <= tol
            assert rel(gi, uip.view(np.complex128).reshape(sg.aR, sg.thetaR)) <= tol


def test_chunked_tables_match_single_pass():
    """A LUT budget that holds one sphere at a time gives the same slice."""
    full = run_gpu("lut", BS_PREC_FP64)
    p, s, _ = scene("lut")
    one = max(oracle_lib.sphere_geom(p, abi.Sphere(*sp)).dR for sp in s) * 200 * 64 * 2
    chunked = run_gpu("lut", BS_PREC_FP64, budget=one)
    assert rel(chunked["U"], full["U"]) <= 1e-14
    assert rel(chunked["D"], full["D"]) <= 1e-14


def test_chunked_lut_budget_mixed():
    """Mixed path, one sphere's tables at a time: 8-byte entries in linear rows of thetaR + 1 entries rounded
    up to even (302 here), plus the texture planes, which count as a second copy.  Each pixel's Kahan
    compensation is carried from one sphere chunk's launch to the next, so the slice has the bits of the
    single launch."""
    full = run_gpu("lut_staged", BS_PREC_MIXED, staging=1)
    p, s, _ = scene("lut_staged")
    one = max((g.dR + g.aR) for g in (oracle_lib.sphere_geom(p, abi.Sphere(*sp)) for sp in s)) * 302 * 8 * 2
    chunked = run_gpu("lut_staged", BS_PREC_MIXED, budget=one, staging=1)
    assert chunked["stats"].lut_chunks_total == full["stats"].lut_chunks_total
    assert np.array_equal(chunked["U"], full["U"]) and np.array_equal(chunked["D"], full["D"])


def test_repeatable():
    a = run_gpu("lut", BS_PREC_MIXED)
    b = run_gpu("lut", BS_PREC_MIXED)
    assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["D"], b["D"])


def test_compat_sampler_matches_reference_rule():
    """bs_sample_waves_compat reproduces the oracle's restatement of mcSampleNA."""
    p, s, _ = scene("lut")
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.sample_waves_compat(64)
        ctx.simulate(BS_PREC_FP64)
        D = ctx.image(BS_IMG_INTENSITY, f64=True)
    lib = oracle_lib.load()
    w = np.zeros(3 * 64)
    kd = np.array(p.k_dir[:])
    lib.bso_mc_sample(64, oracle_lib.P(kd), p.condenser[0], p.condenser[1], oracle_lib.P(w))
    arr, ns = abi.sphere_array(s)
    _, _, Do, _ = oracle_lib.simulate(p, arr, ns, w.reshape(-1, 3))
    assert rel(D, Do) <= TOL64


def test_config1_full_size_fp64_matches_oracle():
    """Config 1 at its full size (256^2 over 20 um, padding 2: near field 1280^2, 400 waves, direct order
    sums, one sphere a = 5 um with ka = 12.57): FP64 GPU path vs the oracle on all host cores."""
    p, s, w = scenes.config1()
    arr, ns = abi.sphere_array(s)
    U, Uf, D, Di = oracle_lib.simulate(p, arr, ns, w)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(BS_PREC_FP64)
        errs = {"U": rel(ctx.field(BS_FIELD_TOTAL), U), "Uf": rel(ctx.field(BS_FIELD_INCIDENT), Uf),
                "D": rel(ctx.image(BS_IMG_INTENSITY, f64=True), D),
                "Di": rel(ctx.image(BS_IMG_INCIDENT, f64=True), Di)}
        ctx.simulate(BS_PREC_MIXED)
        mixed = {"D": rel(ctx.image(BS_IMG_INTENSITY, f64=True), D)}
    assert max(errs.values()) <= TOL64, errs
    assert mixed["D"] <= TOL_MIXED_IMG, mixed
