"""The `bimsim` command line: flag grammar and derived parameters, source-image
reading and the image writers (CPU), and end-to-end runs writing ENVI and image
files (GPU)."""
import json
import os
import struct
import subprocess
import tempfile
import zlib

import numpy as np
import pytest

import oracle_lib
from bimsim_gb300 import BS_IMG_ABSORBANCE, BS_IMG_INCIDENT, BS_IMG_INTENSITY, BS_PREC_FP64, Context, abi, lib

EXE = os.path.join(os.path.dirname(lib.library_path()), "bimsim")


def run(*args, check=True, cwd=None):
    if not os.path.exists(EXE):
        from bimsim_gb300 import build
        build.build()
    # the reference's default outputs (out_*.bmp) land in cwd: keep them out of the repository
    r = subprocess.run([EXE] + [str(a) for a in args], capture_output=True, text=True,
                       cwd=cwd or tempfile.gettempdir())
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
    run(*common, "--intensity", out, "--absorbance", absf, "--incident", "", "--absorbance-spec", "", cwd=tmp_path)
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
    run(*common, "--intensity", out, "--absorbance", "", "--incident", "", "--absorbance-spec", "", "--append",
        cwd=tmp_path)
    assert "bands = 2" in open(str(out) + ".hdr").read()
    assert np.fromfile(out, dtype=np.float32).size == 2 * 256


def test_material_files_give_sphere_indices(tmp_path):
    m1 = tmp_path / "m1.txt"
    m1.write_text("2.0 1.40 0.00\n4.0 1.50 0.02\n")
    m2 = tmp_path / "m2.txt"
    m2.write_text("# [wavenumber,n,k]\n5000 1.30 0.1\n2000 1.60 0.3\n")
    d = dry("--material-file", m1, m2, "--lambda", 2.5, "--spheres", 0, 0, 0, 1, 0, 3, 0, 0, 1, 1)
    s0, s1 = d["spheres"]
    # lambda 2.5 lies a quarter into [2, 4]: the reference weights give 1.40 * 0.25 + 1.50 * 0.75
    assert s0[4] == pytest.approx(1.475, rel=1e-6) and s0[5] == pytest.approx(0.015, rel=1e-5)
    n = lib.material_eval(m2, [np.float32(2.5)])[0]
    assert s1[4] == pytest.approx(n.real, rel=1e-7) and s1[5] == pytest.approx(n.imag, rel=1e-6)
    r = run("--material-file", tmp_path / "missing.txt", "--dry-run", check=False)
    assert r.returncode == 1 and "not found" in r.stdout


# ---------------------------------------------------------------------------
# source images (--extended-source) and image outputs
# ---------------------------------------------------------------------------
def write_bmp(path, rows, bpp):
    """rows: list of lists of (r, g, b) (bpp 24) or palette indices (bpp 8, grey palette), top row first."""
    h, w = len(rows), len(rows[0])
    stride = (w * bpp // 8 + 3) & ~3
    pal = b"".join(bytes((i, i, i, 0)) for i in range(256)) if bpp == 8 else b""
    off = 54 + len(pal)
    data = b""
    for r in reversed(rows):
        line = b"".join(bytes((px[2], px[1], px[0])) for px in r) if bpp == 24 else bytes(r)
        data += line + b"\0" * (stride - len(line))
    hdr = b"BM" + struct.pack("<IHHI", off + len(data), 0, 0, off)
    hdr += struct.pack("<IiiHHIIiiII", 40, w, h, 1, bpp, 0, len(data), 2835, 2835, 256 if bpp == 8 else 0, 0)
    open(path, "wb").write(hdr + pal + data)


def test_extended_source_images_give_one_source_per_nonzero_pixel(tmp_path):
    pgm = tmp_path / "s.pgm"
    pgm.write_text("P2\n# comment\n3 2\n255\n0 128 255\n10 0 0\n")
    assert dry("--extended-source", pgm, "--xy", 10, 0)["point_sources"] == 3
    bmp24 = tmp_path / "s24.bmp"
    write_bmp(bmp24, [[(0, 9, 9), (200, 0, 0)], [(1, 0, 0), (0, 0, 0)]], 24)  # first channel = red
    assert dry("--extended-source", bmp24, "--xy", 10, 0)["point_sources"] == 2
    bmp8 = tmp_path / "s8.bmp"
    write_bmp(bmp8, [[0, 3, 0, 7], [5, 0, 0, 0]], 8)
    assert dry("--extended-source", bmp8, "--xy", 10, 0)["point_sources"] == 3
    r = run("--extended-source", tmp_path / "missing.pgm", "--dry-run", check=False)
    assert r.returncode == 1 and "cannot open" in r.stdout
    for mode in (1, 2, 3):
        d = dry("--interpolate", mode, "--points-rings", 6, 3)
        assert d["interpolate"] == mode and d["points_rings"] == [6, 3]
    # modes 1 and 3 with fewer than two rings: the central source only
    assert dry("--interpolate", 3, "--points-rings", 0, 0)["points_rings"] == [1, 1]
    # mode 0's ring loop never advances in the reference: refused with rings, the central source without
    r = run("--interpolate", 0, "--dry-run", check=False)
    assert r.returncode == 1 and "does not terminate" in r.stdout
    assert dry("--interpolate", 0, "--points-rings", 2, 0)["interpolate"] == 0
    r = run("--interpolate", 4, "--dry-run", check=False)
    assert r.returncode == 1 and "not a mode" in r.stdout


def brewer_rgb(values, vmin, vmax):
    """Restatement of the Brewer map (rts/visualization/colormap.h:92-110): a = (v - vmin) / (vmax - vmin)
    in float32, the normalised texture coordinate a + 1/22 (float32), linear filtering with exact
    weights and clamping between the 11 control points, 255 * colour truncated to 8 bits."""
    ctrl = np.array([[49, 54, 149], [69, 117, 180], [116, 173, 209], [171, 217, 233], [224, 243, 248],
                     [255, 255, 191], [254, 224, 144], [253, 174, 97], [244, 109, 67], [215, 48, 39],
                     [165, 0, 38]], dtype=np.float64)
    ctrl = (np.round(ctrl / 255.0 * 1e6) / 1e6).astype(np.float32).astype(np.float64)
    v = np.asarray(values, np.float64).astype(np.float32)
    a = (v - np.float32(vmin)) / (np.float32(vmax) - np.float32(vmin))
    t = (a + np.float32(1.0 / 22)).astype(np.float32)
    xb = t.astype(np.float64) * 11 - 0.5
    fl = np.floor(xb)
    fr = xb - fl
    i0 = np.clip(fl.astype(int), 0, 10)
    i1 = np.clip(fl.astype(int) + 1, 0, 10)
    c = ((1 - fr)[:, None] * ctrl[i0] + fr[:, None] * ctrl[i1]).astype(np.float32)
    return (np.float32(255) * c).astype(np.uint8)


def read_bmp24(path):
    b = open(path, "rb").read()
    off, = struct.unpack("<I", b[10:14])
    w, h = struct.unpack("<ii", b[18:26])
    stride = (w * 3 + 3) & ~3
    img = np.zeros((h, w, 3), np.uint8)
    for y in range(h):
        row = b[off + (h - 1 - y) * stride: off + (h - 1 - y) * stride + 3 * w]
        img[y] = np.frombuffer(row, np.uint8).reshape(w, 3)[:, ::-1]
    return img


def read_png_rgb(path):
    b = open(path, "rb").read()
    assert b[:8] == bytes([137, 80, 78, 71, 13, 10, 26, 10])
    pos, idat, w = 8, b"", 0
    while pos < len(b):
        n, = struct.unpack(">I", b[pos:pos + 4])
        typ, data = b[pos + 4:pos + 8], b[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", b[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + data) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h = struct.unpack(">II", data[:8])
            assert data[8:10] == bytes([8, 2])
        elif typ == b"IDAT":
            idat += data
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[y * (3 * w + 1): (y + 1) * (3 * w + 1)] for y in range(h)]
    assert all(r[0] == 0 for r in rows)
    return np.stack([np.frombuffer(r[1:], np.uint8).reshape(w, 3) for r in rows])


@pytest.fixture(scope="module")
def image_writer(tmp_path_factory):
    """A small driver of cli/image_io.cpp: writes colour-mapped values read from stdin."""
    d = tmp_path_factory.mktemp("imgw")
    src = d / "drv.cpp"
    src.write_text(r'''
#include "image_io.h"
#include <iostream>
int main(int argc, char** argv) {
    int w, h, pos, cm; std::cin >> w >> h >> pos >> cm;
    std::vector<double> v((size_t)w * h);
    for (auto& x : v) std::cin >> x;
    std::string err;
    if (!bsio::write_scalar_image(argv[1], w, h, v, pos != 0, (bsio::Colormap)cm, err)) { std::cout << err; return 1; }
    return 0;
}''')
    cli = os.path.join(os.path.dirname(os.path.dirname(lib.library_path())), "cli")
    exe = d / "drv"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", cli, str(src), os.path.join(cli, "image_io.cpp"),
                           "-o", str(exe)])

    def write(path, vals, positive=True, cm=0):
        h, w = vals.shape
        inp = f"{w} {h} {int(positive)} {cm}\n" + " ".join(repr(float(x)) for x in vals.ravel())
        r = subprocess.run([str(exe), str(path)], input=inp, capture_output=True, text=True)
        return r
    return write


def test_brewer_bmp_and_png_match_the_reference_colormap(image_writer, tmp_path):
    rng = np.random.default_rng(7)
    vals = rng.uniform(0, 3, (5, 7))
    vals[2, 3] = 3.5                                  # the maximum: range [0, 3.5]
    for ext, reader in ((".bmp", read_bmp24), (".png", read_png_rgb)):
        path = tmp_path / ("a" + ext)
        assert image_writer(path, vals).returncode == 0
        img = reader(path)
        assert img.shape == (5, 7, 3)
        exp = brewer_rgb(vals.ravel(), 0.0, 3.5).reshape(5, 7, 3)
        assert np.array_equal(img, exp)
    # the six-decimal control points: (69, 117, 180) of the second point render as (68, 117, 179)
    ctrl = (np.round(np.array([69, 117, 180]) / 255.0 * 1e6) / 1e6).astype(np.float32)
    assert (np.float32(255) * ctrl).astype(np.uint8).tolist() == [68, 117, 179]


def test_colour_maps_are_the_references(image_writer, tmp_path):
    """The image writer's Brewer and gray maps give the bytes of the reference's own rts::gpu2cpu
    (rts/visualization/colormap.h; golden ref_colormap.json from its kernels run on the CPU with exact
    texture weights) for 2204 values on [0, 3.5]; and the numpy restatement agrees."""
    import json
    g = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_colormap.json")))
    vals = np.array(g["values"])
    n = vals.size
    grid = vals.reshape(19, n // 19) if n % 19 == 0 else np.concatenate([vals, np.full(-n % 29, 0.0)]).reshape(-1, 29)
    for cm, name in ((0, "brewer"), (1, "gray")):
        ref = np.frombuffer(bytes.fromhex(g[name]), np.uint8).reshape(-1, 3)
        path = tmp_path / f"{name}.bmp"
        assert image_writer(path, grid, cm=cm).returncode == 0
        img = read_bmp24(path).reshape(-1, 3)[:n]
        assert np.array_equal(img, ref), np.argwhere(np.any(img != ref, axis=1))[:5].ravel()
    assert np.array_equal(brewer_rgb(vals, 0.0, 3.5), np.frombuffer(bytes.fromhex(g["brewer"]), np.uint8).reshape(-1, 3))


def test_gray_and_signed_range(image_writer, tmp_path):
    vals = np.array([[-2.0, -1.0, 0.0, 1.0]])
    path = tmp_path / "g.bmp"
    assert image_writer(path, vals, positive=False, cm=1).returncode == 0
    img = read_bmp24(path)
    expect = (np.float32(255) * np.clip(((vals.ravel() + 2) / 4).astype(np.float32), 0, 1)).astype(np.uint8)
    assert np.array_equal(img[0, :, 0], expect) and np.array_equal(img[0, :, 1], expect)
    r = image_writer(tmp_path / "x.jpg", vals)
    assert r.returncode == 1 and "not supported" in r.stdout


@pytest.mark.gpu
def test_cli_extended_source_and_image_outputs(tmp_path):
    """--extended-source sums point sources exactly like bs_simulate_sources; image outputs are the
    colour-mapped detector images; near- and far-field images are written by default."""
    from bimsim_gb300 import BS_PREC_MIXED, lib as L, scenes
    src = tmp_path / "s.pgm"
    src.write_text("P2\n2 2\n255\n0 255\n128 0\n")
    waves = scenes.mc_waves(24, 0, 0.5, seed=22)
    wfile = tmp_path / "w.txt"
    np.savetxt(wfile, waves)
    common = ["--spheres", 0.5, 0, 0, 2, 0, "--materials", 1.4, 0.05, "--lambda", 3, "--condenser", 0, 0.5,
              "--objective", 0, 0.5, "--resolution", 16, "--xy", 12, 0, "--waves-file", wfile, "--lut-res", 96, 128,
              "--extended-source", src]
    run(*common, "--intensity", tmp_path / "I", "--incident", "", "--absorbance", "", "--absorbance-spec", "",
        cwd=tmp_path)
    I = np.fromfile(tmp_path / "I", dtype=np.float32).reshape(16, 16)
    p = abi.make_params(lam=3, condenser=(0, 0.5), objective=(0, 0.5), xy=(12, 0), resolution=16, us_lut_r=96,
                        us_lut_theta=128)
    srcs = []
    for x, y, v in ((1, 0, 255), (0, 1, 128)):   # x outer, y inner, non-zero pixels only
        f = L.plane_point(p, np.float32(x / 2), np.float32(y / 2))
        srcs.append([*f, float(np.float32(v) / np.float32(255))])
    with Context(p) as ctx:
        ctx.set_spheres([(0.5, 0, 0, 2, float(np.float32(1.4)), float(np.float32(0.05)))])
        ctx.set_waves(waves)
        ctx.simulate_sources(np.array(srcs), BS_PREC_MIXED)
        ref = ctx.image(BS_IMG_INTENSITY)
    assert np.array_equal(I, ref)
    # default outputs: detector images as BMP (Brewer), near and far field magnitude images
    d2 = tmp_path / "run2"
    d2.mkdir()
    run(*common[:-2], "--absorbance-spec", "", cwd=d2)
    for name, n in (("out_i.bmp", 16), ("out_inc.bmp", 16), ("out_a.bmp", 16), ("out_n.bmp", 48), ("out_f.bmp", 16)):
        img = read_bmp24(d2 / name)
        assert img.shape == (n, n, 3), name
    run(*common[:-2], "--intensity", d2 / "I", "--absorbance-spec", "", "--near-field", "", "--far-field", "",
        cwd=d2)
    Ie = np.fromfile(d2 / "I", dtype=np.float32).astype(np.float64).reshape(16, 16)
    img = read_bmp24(d2 / "out_i.bmp")
    m = Ie.ravel()[np.argmax(np.abs(Ie.ravel()))]
    exp = brewer_rgb(Ie.ravel(), 0.0, m).reshape(16, 16, 3)
    # the image is mapped from the double image, the expectation from its float32 ENVI copy
    assert np.mean(np.abs(img.astype(int) - exp.astype(int)) <= 1) == 1.0
