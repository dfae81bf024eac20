"""The GPU path through the C ABI, and the `bimsim` CLI run with the reference's own flags, against
the reference's own path run on the CPU (golden ref_sim.json; see tests/golden/make_ref_sim_golden.py).

  * double-precision build of the reference: the FP64 GPU path within 1e-10 relative L2 on U, Uf,
    D, Di and absorbance; the mixed path within 1e-5 on the images and 1e-4 on the near field
  * the reference as it ships (single precision): both GPU paths within 1e-5 on D and Di, 5e-5 on
    absorbance and 1e-4 on the near field.  The shipped build's own single-precision error against
    the FP64 oracle is up to 2e-6 on D, Di and 1.3e-5 on absorbance (a log of a ratio of nearly equal
    images, direct mode), hence the looser absorbance bound against it
  * the ring-source drivers (--interpolate 1, 2, 3), both precisions, within the same bounds of the
    shipped reference's drivers
  * back-propagation before the band-pass (bs_set_backpropagation) against the reference's
    applyBackpropagation in both builds, at each build's bounds
  * bs_simulate_sources over the sources of an --extended-source image against the reference's
    SimulateExtendedSource (and the CLI with that flag), at the f32 bounds
  * the vector stub's near fields (--vector), FP64 within 1e-10 of the double build, otherwise 1e-4
  * the CLI with the reference's flags (its Monte Carlo directions from the compat sampler): the
    ENVI images within the same bounds of the shipped reference's images, ring scenes included; and
    the files the reference's executable itself writes (ENVI headers and absorbance-spectrum text
    identical, band data within the bounds)
"""
import os
import subprocess

import numpy as np
import pytest

import ref_golden as rg
from bimsim_gb300 import (BS_FIELD_INCIDENT, BS_FIELD_TOTAL, BS_IMG_ABSORBANCE, BS_IMG_INCIDENT, BS_IMG_INTENSITY,
                          BS_PREC_FP64, BS_PREC_MIXED, Context, lib)

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(lib.library_path()), "bimsim")


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) / np.linalg.norm(np.asarray(b).ravel()))


def gpu_run(rec, prec):
    with Context(rg.params(rec)) as ctx:
        ctx.set_spheres(rg.spheres(rec))
        ctx.set_waves(rg.waves(rec))
        ctx.simulate(prec)
        return {"U": ctx.field(BS_FIELD_TOTAL), "Uf": ctx.field(BS_FIELD_INCIDENT),
                "D": ctx.image(BS_IMG_INTENSITY, f64=True), "Di": ctx.image(BS_IMG_INCIDENT, f64=True),
                "Absorbance": ctx.image(BS_IMG_ABSORBANCE, f64=True)}


def rel_finite(a, b):
    """rel over the finite entries, which must be the same in both (a ring-line image is 0 / 0 beyond
    its last ring, so its absorbance is NaN there)."""
    fa, fb = np.isfinite(a), np.isfinite(b)
    if not np.array_equal(fa, fb):
        return float("inf")
    return rel(np.asarray(a)[fa], np.asarray(b)[fb])


def errors(out, rec):
    return {k: rel_finite(out[k], rg.field(rec, k) if k in ("U", "Uf") else rg.image(rec, k)) for k in out}


@pytest.mark.parametrize("name", rg.scenes("f64"))
def test_gpu_matches_the_references_double_precision_run(name):
    rec = rg.load()[name]
    e64 = errors(gpu_run(rec, BS_PREC_FP64), rec)
    assert max(e64.values()) <= 1e-10, e64
    emx = errors(gpu_run(rec, BS_PREC_MIXED), rec)
    assert max(emx[k] for k in ("D", "Di", "Absorbance")) <= 1e-5, emx
    assert max(emx[k] for k in ("U", "Uf")) <= 1e-4, emx


TOL_F32 = {"D": 1e-5, "Di": 1e-5, "Absorbance": 5e-5, "U": 1e-4, "Uf": 1e-4}


@pytest.mark.parametrize("name", rg.scenes("f32"))
def test_gpu_matches_the_shipped_references_run(name):
    rec = rg.load()[name]
    for prec in (BS_PREC_FP64, BS_PREC_MIXED):
        e = errors(gpu_run(rec, prec), rec)
        assert all(e[k] <= TOL_F32[k] for k in e), (prec, e)


@pytest.mark.parametrize("name", rg.nearfield_scenes())
def test_gpu_vector_stub_near_fields_match_the_references_run(name):
    """--vector (the reference's vector stub: its incident field, no scattered field): U and Uf of both
    precisions against the reference's near fields after sumUf."""
    rec = rg.load()[name]
    for prec in (BS_PREC_FP64, BS_PREC_MIXED):
        with Context(rg.params(rec)) as ctx:
            ctx.set_spheres(rg.spheres(rec))
            ctx.set_waves(rg.waves(rec))
            ctx.simulate(prec)
            out = {"U": ctx.field(BS_FIELD_TOTAL), "Uf": ctx.field(BS_FIELD_INCIDENT)}
        if not any(np.any(rg.field(rec, k)) for k in out):  # --lut-uf: the stub's fields are empty
            assert not any(np.any(v) for v in out.values())
            continue
        e = errors(out, rec)
        if rec["build"] == "f64" and prec == BS_PREC_FP64:
            assert max(e.values()) <= 1e-10, e
        else:
            assert max(e.values()) <= 1e-4, (prec, e)


@pytest.mark.parametrize("name", rg.backprop_scenes())
def test_gpu_backpropagation_matches_the_references_run(name):
    """bs_set_backpropagation over the plane position against the reference's applyBackpropagation run
    before its band-pass (double build: FP64 within 1e-10; shipped float build: the f32 bounds)."""
    rec = rg.load()[name]
    for prec in (BS_PREC_FP64, BS_PREC_MIXED):
        with Context(rg.params(rec)) as ctx:
            ctx.set_spheres(rg.spheres(rec))
            ctx.set_waves(rg.waves(rec))
            ctx.set_backpropagation(True, rg.plane_position(rec))
            ctx.simulate(prec)
            out = {"D": ctx.image(BS_IMG_INTENSITY, f64=True), "Di": ctx.image(BS_IMG_INCIDENT, f64=True),
                   "Absorbance": ctx.image(BS_IMG_ABSORBANCE, f64=True)}
        e = errors(out, rec)
        if rec["build"] == "f64" and prec == BS_PREC_FP64:
            assert max(e.values()) <= 1e-10, e
        elif rec["build"] == "f64":
            assert max(e.values()) <= 1e-5, e
        else:
            assert all(e[k] <= TOL_F32[k] for k in e), (prec, e)


@pytest.mark.parametrize("name", rg.source_scenes())
def test_gpu_extended_source_matches_the_references_driver(name):
    """bs_simulate_sources over the point sources the reference loaded from the scene's image, against
    its SimulateExtendedSource (shipped single-precision build run on the CPU)."""
    rec = rg.load()[name]
    for prec in (BS_PREC_FP64, BS_PREC_MIXED):
        with Context(rg.params(rec)) as ctx:
            ctx.set_spheres(rg.spheres(rec))
            ctx.set_waves(rg.waves(rec))
            ctx.simulate_sources(rg.sources(rec), prec)
            out = {"D": ctx.image(BS_IMG_INTENSITY, f64=True), "Di": ctx.image(BS_IMG_INCIDENT, f64=True),
                   "Absorbance": ctx.image(BS_IMG_ABSORBANCE, f64=True)}
        e = errors(out, rec)
        assert all(e[k] <= TOL_F32[k] for k in e), (prec, e)


@pytest.mark.parametrize("name", rg.ring_scenes())
def test_gpu_ring_drivers_match_the_shipped_references_run(name):
    """bs_simulate_ring_detector / _line / _interp against the reference's own --interpolate 1, 2, 3
    drivers (shipped single-precision build run on the CPU)."""
    rec = rg.load()[name]
    mode, points, rings = rg.rings(rec)
    run = {1: "simulate_ring_detector", 2: "simulate_ring_line", 3: "simulate_ring_interp"}.get(mode)
    for prec in (BS_PREC_FP64, BS_PREC_MIXED):
        with Context(rg.params(rec)) as ctx:
            ctx.set_spheres(rg.spheres(rec))
            ctx.set_waves(rg.waves(rec))
            if run:
                getattr(ctx, run)(points, rings, prec)
            else:  # --interpolate 0 with no rings: the central source alone
                ctx.simulate(prec)
            out = {"D": ctx.image(BS_IMG_INTENSITY, f64=True), "Di": ctx.image(BS_IMG_INCIDENT, f64=True),
                   "Absorbance": ctx.image(BS_IMG_ABSORBANCE, f64=True)}
        e = errors(out, rec)
        assert all(e[k] <= TOL_F32[k] for k in e), (prec, e)


CLI_FILES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cli_files.json")


@pytest.mark.parametrize("name", ["nu_append", "lambda_overwrite"])
def test_cli_writes_the_references_output_files(name, tmp_path):
    """The files the reference's executable writes (its main() and fileoutStruct::Save run on the CPU,
    golden ref_cli_files.json): this CLI run with the same flags in the same order gives the same ENVI
    headers (band values of --nu or --lambda, --append or overwrite) and absorbance-spectrum text, and
    each band's data within the single-precision bounds."""
    import base64
    import json
    g = json.load(open(CLI_FILES))[name]
    for flags in g["runs"]:
        r = subprocess.run([EXE] + [f.replace("{dir}", str(tmp_path)) for f in flags], capture_output=True,
                           text=True, cwd=str(tmp_path))
        assert r.returncode == 0, r.stdout + r.stderr
    tol = {"i": TOL_F32["D"], "inc": TOL_F32["Di"], "a": TOL_F32["Absorbance"], "t": TOL_F32["Absorbance"]}
    for f, ref in g["files"].items():
        assert (tmp_path / (f + ".hdr")).read_text() == ref["hdr"], f
        mine = np.fromfile(tmp_path / f, dtype="<f4")
        theirs = np.frombuffer(base64.b64decode(ref["data"]), dtype="<f4")
        assert mine.shape == theirs.shape, f
        bands = mine.size // 144
        for b in range(bands):
            e = rel_finite(mine[b * 144:(b + 1) * 144].astype(np.float64), theirs[b * 144:(b + 1) * 144].astype(np.float64))
            assert e <= tol[f], (f, b, e)
    assert (tmp_path / "as.txt").read_text() == g["as.txt"]


@pytest.mark.parametrize("name", rg.scenes("f32") + rg.ring_scenes() + rg.source_scenes())
def test_cli_with_the_references_flags_matches_its_run(name, tmp_path):
    rec = rg.load()[name]
    outs = {k: str(tmp_path / k) for k in ("D", "Di", "Absorbance")}
    flags = list(rec["flags"])
    if "{image}" in flags:  # the extended-source image the reference read
        (tmp_path / "source.pgm").write_bytes(bytes.fromhex(rec["image_pgm"]))
        flags = [str(tmp_path / "source.pgm") if f == "{image}" else f for f in flags]
    cmd = [EXE] + flags + ["--intensity", outs["D"], "--incident", outs["Di"], "--absorbance",
                           outs["Absorbance"], "--absorbance-spec", ""]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    res = int(rec["dims"][2])
    for key, path in outs.items():
        img = np.fromfile(path, dtype=np.float32).reshape(res, res)
        e = rel_finite(img, rg.image(rec, key))
        assert e <= TOL_F32[key], (key, e)
