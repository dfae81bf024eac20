"""The oracle against the reference's own path run on the CPU (golden ref_sim.json, recorded by
tests/golden/make_ref_sim_golden.py from the reference's sources, .cu files included, compiled in
place for the host with CUDA stand-ins).

  * double-precision build of the reference (ptype double; every path except the LUT apply and the
    incident-field LUT, whose texture copies are hard-coded for float): near fields U, Uf and
    detector images D, Di within 1e-12 relative L2, Mie coefficients within 1e-12, the per-sphere
    tables Usp/Uip of sphere::calcUp + sphere.cu within 1e-12
  * the reference as it ships (ptype float, LUT apply through emulated texture fetches with exact
    bilinear weights): within 1e-5 (2e-5 on absorbance), the single-precision rounding of its
    arithmetic
  * the ring-source drivers (--interpolate 1, 2, 3) of the shipped reference: within 1e-5 (2e-5 on
    absorbance)
  * applyBackpropagation before the band-pass, in both builds, at the bounds of each build
  * the extended-source driver (--extended-source): the points it loads from the image and its summed
    detector images, within 1e-5
  * the vector stub (--vector): U and Uf after sumUf, at the bounds of each build
  * the parsed plane, wavelength (--nu) and Monte Carlo directions as the reference derives them
"""
import os

import numpy as np
import pytest

import oracle_lib
import ref_golden as rg
from bimsim_gb300 import abi

TOL_F64 = 1e-12
TOL_F32 = 1e-5


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) / np.linalg.norm(np.asarray(b).ravel()))


def oracle_run(rec):
    p = rg.params(rec)
    arr, ns = abi.sphere_array(rg.spheres(rec))
    return p, oracle_lib.simulate(p, arr, ns, rg.waves(rec))


@pytest.mark.parametrize("name", rg.scenes("f64"))
def test_oracle_matches_the_references_double_precision_run(name):
    rec = rg.load()[name]
    p, (U, Uf, D, Di) = oracle_run(rec)
    errs = {"U": rel(U, rg.field(rec, "U")), "Uf": rel(Uf, rg.field(rec, "Uf")), "D": rel(D, rg.image(rec, "D")),
            "Di": rel(Di, rg.image(rec, "Di"))}
    assert max(errs.values()) <= TOL_F64, errs
    with np.errstate(divide="ignore", invalid="ignore"):
        assert rel(-np.log10(D / Di), rg.image(rec, "Absorbance")) <= TOL_F64


@pytest.mark.parametrize("name", rg.scenes("f32"))
def test_oracle_within_single_precision_of_the_shipped_reference(name):
    rec = rg.load()[name]
    p, (U, Uf, D, Di) = oracle_run(rec)
    errs = {"U": rel(U, rg.field(rec, "U")), "Uf": rel(Uf, rg.field(rec, "Uf")), "D": rel(D, rg.image(rec, "D")),
            "Di": rel(Di, rg.image(rec, "Di"))}
    assert max(errs.values()) <= TOL_F32, errs
    # absorbance, a log of a ratio of nearly equal images, carries more of the float build's rounding
    with np.errstate(divide="ignore", invalid="ignore"):
        assert rel(-np.log10(D / Di), rg.image(rec, "Absorbance")) <= 2e-5


@pytest.mark.parametrize("name", rg.nearfield_scenes())
def test_oracle_vector_stub_near_fields_match_the_reference_run(name):
    """--vector: the reference's vector stub computes the incident field of nfVectorUf.cu and no scattered
    field; U and Uf after its sumUf against the oracle's (its run stops there: getFarField then writes the
    crop's y and z components through null pointers, fieldslice.cu:340-361)."""
    rec = rg.load()[name]
    assert "--vector" in rec["flags"]
    p, (U, Uf, _, _) = oracle_run(rec)
    tol = TOL_F64 if rec["build"] == "f64" else TOL_F32
    for mine, key in ((U, "U"), (Uf, "Uf")):
        ref = rg.field(rec, key)
        if not np.any(ref):  # with --lut-uf the stub's incident field is empty (nfVectorUfLut.cu:7-10)
            assert not np.any(mine), key
        else:
            assert rel(mine, ref) <= tol, (key, rel(mine, ref))


@pytest.mark.parametrize("name", rg.backprop_scenes())
def test_oracle_backpropagation_matches_the_reference_run(name):
    """applyBackpropagation (microscope.cu:423-488, 592-605) run by the reference before its band-pass,
    against the oracle's detector with the same propagator over the plane position."""
    rec = rg.load()[name]
    p, (U, Uf, _, _) = oracle_run(rec)
    res = p.resolution
    D, Di = np.zeros(res * res), np.zeros(res * res)
    U = np.ascontiguousarray(U, dtype=np.complex128)
    Uf = np.ascontiguousarray(Uf, dtype=np.complex128)
    oracle_lib.load().bso_detector_bp(oracle_lib.C.byref(p), oracle_lib.P(U), oracle_lib.P(Uf),
                                      rg.plane_position(rec), oracle_lib.P(D), oracle_lib.P(Di))
    D, Di = D.reshape(res, res), Di.reshape(res, res)
    tol = TOL_F64 if rec["build"] == "f64" else TOL_F32
    errs = {"U": rel(U, rg.field(rec, "U")), "D": rel(D, rg.image(rec, "D")), "Di": rel(Di, rg.image(rec, "Di"))}
    assert max(errs.values()) <= tol, errs
    with np.errstate(divide="ignore", invalid="ignore"):
        assert rel(-np.log10(D / Di), rg.image(rec, "Absorbance")) <= (TOL_F64 if rec["build"] == "f64" else 2e-5)
    # the propagation changes the image: the single-source run of the same scene differs
    _, _, D0, _ = oracle_lib.simulate(p, *abi.sphere_array(rg.spheres(rec)), rg.waves(rec))
    assert rel(D0, D) > 1e-3


@pytest.mark.parametrize("name", rg.source_scenes())
def test_oracle_extended_source_matches_the_references_driver(name):
    """--extended-source: the reference's LoadExtendedSource (microscope.cu:1258-1296) placed a point source
    at pos(x / width, y / height) of the detector plane with amplitude pixel / 255 for every nonzero pixel,
    x outer, y inner; its SimulateExtendedSource (:873-913) summed their detector images.  The library's
    plane mapping gives the same points, and the oracle's per-source slices sum to its images."""
    from bimsim_gb300 import lib
    rec = rg.load()[name]
    p = rg.params(rec)
    pgm = bytes.fromhex(rec["image_pgm"])
    hdr = pgm.split(b"\n", 3)
    w, h = (int(v) for v in hdr[1].split())
    px = np.frombuffer(hdr[3], np.uint8).reshape(h, w)
    expect = [(x, y) for x in range(w) for y in range(h) if px[y, x] != 0]
    src = rg.sources(rec)
    assert len(src) == len(expect)
    for (x, y), (sx, sy, sz, a) in zip(expect, src):
        u, v = float(np.float32(x) / np.float32(w)), float(np.float32(y) / np.float32(h))
        np.testing.assert_allclose(lib.plane_point(p, u, v), (sx, sy, sz), rtol=0, atol=2e-6)
        assert a == float(np.float32(px[y, x]) / np.float32(255))
    arr, ns = abi.sphere_array(rg.spheres(rec))
    D = Di = 0
    for sx, sy, sz, a in src:
        q = rg.params(rec)
        q.focus[0], q.focus[1], q.focus[2] = sx, sy, sz
        q.amplitude = a
        _, _, d, di = oracle_lib.simulate(q, arr, ns, rg.waves(rec))
        D, Di = D + d, Di + di
    errs = {"D": rel(D, rg.image(rec, "D")), "Di": rel(Di, rg.image(rec, "Di"))}
    assert max(errs.values()) <= TOL_F32, errs


@pytest.mark.parametrize("name", rg.ring_scenes())
def test_oracle_ring_drivers_within_single_precision_of_the_shipped_reference(name):
    """The oracle's restatement of the ring-source drivers (--interpolate 1: rotated detector images,
    2: the radial line of shared-memory ring sums, 3: rotated near fields; 0 with no rings: the central
    source) against the reference's own drivers run on the CPU, their ring-sum blocks as cooperative
    threads."""
    rec = rg.load()[name]
    p = rg.params(rec)
    arr, ns = abi.sphere_array(rg.spheres(rec))
    mode, points, rings = rg.rings(rec)
    if mode == 0:  # no rings: the central source alone
        _, _, D, Di = oracle_lib.simulate(p, arr, ns, rg.waves(rec))
    else:
        D, Di = oracle_lib.simulate_rings(p, arr, ns, rg.waves(rec), mode, points, rings)
    errs = {"D": rel(D, rg.image(rec, "D")), "Di": rel(Di, rg.image(rec, "Di"))}
    assert max(errs.values()) <= TOL_F32, errs
    # the line mode leaves D = Di = 0 beyond its last ring: absorbance NaN there, in both
    with np.errstate(divide="ignore", invalid="ignore"):
        A = -np.log10(D / Di)
    ref = rg.image(rec, "Absorbance")
    assert np.array_equal(np.isfinite(A), np.isfinite(ref))
    assert rel(A[np.isfinite(A)], ref[np.isfinite(ref)]) <= 2e-5


@pytest.mark.parametrize("name", rg.scenes() + rg.ring_scenes() + rg.backprop_scenes() + rg.source_scenes() +
                         rg.nearfield_scenes())
def test_mie_coefficients_match_the_reference_run(name):
    rec = rg.load()[name]
    p = rg.params(rec)
    g = oracle_lib.geom(p)
    for sp in rec["spheres"]:
        A = rg.arr(sp["A"]).view(np.complex128)
        B = rg.arr(sp["B"]).view(np.complex128)
        nl = len(A) - 1
        assert nl == int(sp["geom"][0]) == oracle_lib.load().bso_calc_nl(sp["in"][3], p.lambda_)
        Ao, Bo = np.zeros(2 * nl + 2), np.zeros(2 * nl + 2)
        oracle_lib.load().bso_mie(g.kmag, *sp["in"][3:6], nl, oracle_lib.P(Ao), oracle_lib.P(Bo))
        tol = TOL_F64 if rec["build"] == "f64" else 1e-6  # the float build stores them as float
        assert rel(Ao.view(np.complex128), A) <= tol and rel(Bo.view(np.complex128), B) <= tol


@pytest.mark.parametrize("name", rg.scenes(full=False))
def test_sphere_tables_match_the_reference_run(name):
    rec = rg.load()[name]
    p = rg.params(rec)
    for sp in rec["spheres"]:
        s = abi.Sphere(*sp["in"])
        sg = oracle_lib.sphere_geom(p, s)
        Nl, dmin, dmax, dR, thetaR, aR = (int(sp["geom"][0]), sp["geom"][1], sp["geom"][2], int(sp["geom"][3]),
                                          int(sp["geom"][4]), int(sp["geom"][5]))
        assert (sg.Nl, sg.dR, sg.thetaR, sg.aR) == (Nl, dR, thetaR, aR)
        assert sg.d_min == pytest.approx(dmin, abs=1e-12) and sg.d_max == pytest.approx(dmax, rel=1e-14)
        usp = np.zeros(2 * sg.dR * sg.thetaR)
        uip = np.zeros(2 * sg.aR * sg.thetaR)
        oracle_lib.load().bso_sphere_luts(oracle_lib.C.byref(p), oracle_lib.C.byref(s), oracle_lib.P(usp),
                                          oracle_lib.P(uip))
        rows = sp["theta_rows"]
        mine_u = usp.view(np.complex128).reshape(dR, thetaR).T[rows]  # reference layout: [theta][r]
        mine_i = uip.view(np.complex128).reshape(aR, thetaR).T[rows]
        ref_u = rg.arr(sp["Usp"]).view(np.complex128).reshape(len(rows), dR)
        ref_i = rg.arr(sp["Uip"]).view(np.complex128).reshape(len(rows), aR)
        assert rel(mine_u, ref_u) <= TOL_F64 and rel(mine_i, ref_i) <= TOL_F64


@pytest.mark.parametrize("name", rg.scenes() + rg.scenes(full=False) + rg.ring_scenes() + rg.backprop_scenes() +
                         rg.parse_scenes())
def test_parsed_geometry_matches(name):
    """The near-field quad nf.pos and the derived sizes are the oracle's (arguments.h:340-438,
    microscope.cu:700-718); --nu gives lambda = 1e4/nu in single precision (arguments.h:118-123)."""
    rec = rg.load()[name]
    p = rg.params(rec)
    g = oracle_lib.geom(p)
    np.testing.assert_allclose(list(g.A) + list(g.X) + list(g.Y), rec["nf_quad"], rtol=0, atol=1e-12)
    assert (g.R, g.det_res) == (int(rec["dims"][0]), int(rec["dims"][2]))
    # ss from the plane size, which only --xy sets (40 otherwise; arguments.h:346-418)
    fl = rec["flags"]
    kw = {"xy": (rg.plane_size(fl), rg.plane_position(rec))} if "--xy" in fl else {"plane": rg.plane(fl)}
    assert int(rec["scene"][13]) == abi.make_params(lam=p.lambda_, resolution=p.resolution, **kw).supersample
    if "--nu" in rec["flags"]:
        nu = np.float32(rec["flags"][rec["flags"].index("--nu") + 1])
        assert rec["scene"][0] == float(np.float32(10000) / nu)


@pytest.mark.parametrize("name", rg.scenes("f32") + rg.ring_scenes())
def test_reference_directions_are_the_compat_sampler(name):
    """The directions the shipped reference drew (srand(0) then mcSampleNA) are the oracle's
    restatement, which bs_sample_waves_compat reproduces on the GPU."""
    rec = rg.load()[name]
    p = rg.params(rec)
    nk = int(rec["dims"][5])
    out = np.zeros(3 * nk)
    kd = np.array(p.k_dir[:])
    oracle_lib.load().bso_mc_sample(nk, oracle_lib.P(kd), p.condenser[0], p.condenser[1], oracle_lib.P(out))
    np.testing.assert_allclose(out, rg.waves(rec).ravel(), rtol=0, atol=2e-7)


@pytest.mark.parametrize("name", rg.scenes("f32") + rg.parse_scenes())
def test_cli_parses_the_references_flags_into_its_state(name, tmp_path):
    """The `bimsim` CLI of this project, given the reference's flags, derives the state the
    shipped reference held after LoadParameters (single-precision values)."""
    import json
    import subprocess

    from bimsim_gb300 import lib
    exe = os.path.join(os.path.dirname(lib.library_path()), "bimsim")
    if not os.path.exists(exe):
        from bimsim_gb300 import build
        build.build()
    rec = rg.load()[name]
    r = subprocess.run([exe, "--dry-run"] + rg.flags_with_files(rec, tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    sc = rec["scene"]
    f = lambda v: float(np.float32(v))  # noqa: E731
    assert f(d["lambda"]) == sc[0] and f(d["amplitude"]) == sc[1]
    assert [f(v) for v in d["k"]] == sc[2:5] and [f(v) for v in d["focus"]] == sc[5:8]
    assert [f(v) for v in d["condenser"]] == sc[8:10] and [f(v) for v in d["objective"]] == sc[10:12]
    assert (d["padding"], d["supersample"], d["field_order"]) == (int(sc[12]), int(sc[13]), int(sc[14]))
    assert (d["lut_us"], d["lut_uf"], d["plane_wave"], d["samples"]) == tuple(int(v) for v in sc[15:19])
    assert d["resolution"] == int(rec["dims"][2])
    assert len(d["spheres"]) == len(rec["spheres"])
    for mine, theirs in zip(d["spheres"], rec["spheres"]):
        assert [f(v) for v in mine] == [f(v) for v in theirs["in"]]
    pmin, pmax, nrm = rg.plane(rec["flags"])
    assert [f(v) for v in d["plane_min"]] == list(pmin) and [f(v) for v in d["plane_max"]] == list(pmax)
    assert [f(v) for v in d["normal"]] == list(nrm)
