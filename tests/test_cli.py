"""The `bimsim` command line: flag grammar and derived parameters (CPU), and an
end-to-end run writing ENVI files (GPU)."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import BS_IMG_ABSORBANCE, BS_IMG_INCIDENT, BS_IMG_INTENSITY, BS_PREC_FP64, Context, abi, lib

EXE = os.path.join(os.path.dirname(lib.library_path()), "bimsim")


def run(*args, check=True):
    if not os.path.exists(EXE):
        from bimsim_gb300 import build
        build.build()
    r = subprocess.run([EXE] + [str(a) for a in args], capture_output=True, text=True)
    if check:
        assert r.returncode == 0, r.stdout + r.stderr
    return r


def dry(*args):
    return json.loads(run("--dry-run", *args).stdout.strip().splitlines()[-1])


def test_defaults_match_reference():
    d = dry()
    assert d["lambda"] == 1 and d["resolution"] == 256 and d["padding"] == 1
    assert d["condenser"] == [0, 1] and d["objective"] == [0, 1]
    assert d["field_order"] == 10 and d["samples"] == 400
    assert d["lut_us"] == 1 and d["lut_uf"] == 0 and d["scalar"] == 1
    assert d["plane_min"] == [-5, 0, -5] and d["plane_max"] == [5, 0, 5] and d["normal"] == [0, 1, 0]
    assert d["outputs"]["intensity"] == "out_i.bmp" and d["outputs"]["transmittance"] == ""


def test_config1_flags():
    d = dry("--spheres", 0, 0, 0, 5, 0, "--materials", 1.4, 0.05, "--lambda", 2.5, "--condenser", 0, 0.5,
            "--objective", 0, 0.5, "--samples", 400, "--resolution", 256, "--xy", 20, 0, "--padding", 2,
            "--recursive")
    assert d["lut_us"] == 0 and d["lut_uf"] == 0 and d["padding"] == 2 and d["supersample"] == 1
    assert d["plane_min"] == [-10, -10, 0] and d["normal"] == [0, 0, 1]
    assert d["spheres"] == [[0, 0, 0, 5, pytest.approx(1.4, rel=1e-7), pytest.approx(0.05, rel=1e-6)]]


def test_mode_flags_precedence():
    # arguments.h:99-111: --recursive wins over --recursive-us over --lut-uf
    assert dry("--recursive", "--lut-uf")["lut_uf"] == 0
    d = dry("--recursive-us", "--lut-uf")
    assert d["lut_us"] == 0 and d["lut_uf"] == 0
    d = dry("--lut-uf")
    assert d["lut_us"] == 1 and d["lut_uf"] == 1


def test_spheres_groups_and_materials():
    d = dry("--spheres", 1, 2, 3, 1.5, 1, -3, 0, 0, 2, 0, "--materials", 1.4, 0.05, 1.3, 0.0)
    assert len(d["spheres"]) == 2
    assert d["spheres"][0][:4] == [1, 2, 3, 1.5] and d["spheres"][0][4] == pytest.approx(1.3)
    assert d["spheres"][1][4] == pytest.approx(1.4)


def test_bad_sphere_count_and_missing_material():
    r = run("--dry-run", "--spheres", 1, 2, 3, 4, 5, 6, check=False)
    assert r.returncode == 1 and "Invalid number of sphere parameters" in r.stdout
    r = run("--dry-run", "--spheres", 0, 0, 0, 1, 3, check=False)
    assert r.returncode == 1 and "A material is not loaded for sphere 1" in r.stdout
    r = run("--dry-run", "--materials", 1.4, 0.05, 1.3, check=False)
    assert r.returncode == 1 and "n, k pairs" in r.stdout


def test_supersampling_rule():
    # dx = s/res > lambda/2 -> ss = ceil(2 s / (res lambda)); only --xy changes s
    assert dry("--xy", 40, "--resolution", 64, "--lambda", 0.5)["supersample"] == 3
    assert dry("--xz", 400, "--resolution", 64, "--lambda", 1)["supersample"] == 2  # s stays 40


def test_wavenumber_and_k():
    d = dry("--nu", 2000, "--k", 0.5, 0.3)
    assert d["lambda"] == pytest.approx(5.0) and d["wavenumber"] == 1
    assert d["k"] == pytest.approx([np.cos(0.5) * np.sin(0.3), np.sin(0.5) * np.sin(0.3), np.cos(0.3)], rel=1e-6)


def test_sphere_file(tmp_path):
    f = tmp_path / "s.txt"
    f.write_text("-3 0 0 1 0\n0 3 0 1 1\n")
    d = dry("--sphere-file", f, "--materials", 1.4, 0.05, 1.5, 0.0)
    assert [s[:4] for s in d["spheres"]] == [[-3, 0, 0, 1], [0, 3, 0, 1]]


def test_help_exits_1_like_reference():
    r = run("--help", check=False)
    assert r.returncode == 1 and "--spheres" in r.stdout


@pytest.mark.gpu
def test_cli_end_to_end_envi(tmp_path):
    """The CLI's ENVI files equal the C ABI's images and the oracle's, and --append adds bands."""
    wfile = tmp_path / "w.txt"
    from bimsim_gb300 import scenes
    waves = scenes.mc_waves(24, 0, 0.5, seed=21)
    np.savetxt(wfile, waves)
    common = ["--spheres", 0.5, 0, 0, 2, 0, "--materials", 1.4, 0.05, "--lambda", 3, "--condenser", 0, 0.5,
              "--objective", 0, 0.5, "--resolution", 16, "--xy", 12, 0, "--waves-file", wfile,
              "--precision", "fp64", "--lut-res", 96, 128]
    out = tmp_path / "I"
    absf = tmp_path / "A"
    run(*common, "--intensity", out, "--absorbance", absf, "--incident", "", "--absorbance-spec", "")
    I = np.fromfile(out, dtype=np.float32).reshape(16, 16)
    hdr = open(str(out) + ".hdr").read()
    assert "bands = 1" in hdr and "wavelength = {\n3}" in hdr
    p = abi.make_params(lam=3, condenser=(0, 0.5), objective=(0, 0.5), xy=(12, 0), resolution=16, us_lut_r=96,
                        us_lut_theta=128)
    arr, ns = abi.sphere_array([(0.5, 0, 0, 2, np.float32(1.4), np.float32(0.05))])
    _, _, D, Di = oracle_lib.simulate(p, arr, ns, np.loadtxt(wfile))
    assert np.linalg.norm(I - D) / np.linalg.norm(D) < 1e-6
    A = np.fromfile(absf, dtype=np.float32).reshape(16, 16)
    assert np.linalg.norm(A + np.log10(D / Di)) / np.linalg.norm(np.log10(D / Di)) < 1e-5
    run(*common, "--intensity", out, "--absorbance", "", "--incident", "", "--absorbance-spec", "", "--append")
    assert "bands = 2" in open(str(out) + ".hdr").read()
    assert np.fromfile(out, dtype=np.float32).size == 2 * 256
