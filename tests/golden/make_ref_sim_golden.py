"""Record golden near fields and detector images from the reference's own path run on the CPU.

    make -C oracle ref-sim REF_DIR=<reference checkout>
    python tests/golden/make_ref_sim_golden.py

oracle/_ref/libref_sim_f32.so and libref_sim_f64.so are the reference's sources (host .cpp and
device .cu alike) compiled in place for the host with the CUDA stand-ins of oracle/ref_cuda
(oracle/Makefile, target ref-sim; entry points in oracle/ref_run.cpp).  f32 is the reference as it
ships (ptype float); f64 is the same sources with ptype double, which runs every path except the
LUT apply and the incident-field LUT, whose texture copies are hard-coded for float
(nfScalarUpLut.cu:414-415, nfScalarUfLut.cu:159).  For each scene below, a list of the reference's
own flags, this writes into tests/golden/ref_sim.json the inputs as the reference holds them after
parsing (wavelength, apertures, spheres, the near-field plane), its Monte Carlo directions, Mie
coefficients, per-sphere tables (sampled rows), near fields U and Uf after sumUf, and the detector
images D, Di and absorbance; for the ring scenes (stop = 2: the driver of --interpolate 1, 2 or 3,
as fileout.cu:219-243 calls it) the inputs, directions, coefficients and the detector images the
driver leaves.  Arrays are little-endian float64, base64-encoded.  tests/golden/ref_colormap.json
holds the reference's colour map (rts::gpu2cpu of rts/visualization/colormap.h, Brewer and gray) of a
set of values, from oracle/ref_colormap.cpp in the same library; tests/golden/ref_cli_files.json the
files its executable writes (ENVI intensity, incident, absorbance and transmittance with their headers,
the absorbance-spectrum text) for runs with --append and --nu and runs that overwrite.
"""
import base64
import contextlib
import ctypes as C
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

TWO = ["--spheres", "0.3", "-0.2", "0", "2.2", "0", "5", "4", "1", "1", "1", "--materials", "1.5", "0.04", "1.3", "0"]

# a 4 x 3 source image: four nonzero pixels of different brightness
EXT_PGM = b"P5\n4 3\n255\n" + bytes([0, 255, 0, 128, 64, 0, 0, 0, 0, 0, 200, 0])

RING_OPTICS = ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6", "--resolution", "12", "--xy",
               "16", "0", "--samples", "20"]

# name: (build, stop: 0 the whole path, 1 after the tables, 2 the ring-source driver, 3 the whole path with
# the near field back-propagated, 4 the extended-source driver, 5 the near fields only; flags; 6, the parse
# only, is the PARSE table below)
SCENES = {
    # ptype double: direct (recursive) order sums, the whole path
    "rec_two_spheres": ("f64", 0, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                        "--resolution", "12", "--xy", "16", "0", "--samples", "20", "--recursive"]),
    "rec_large_ka": ("f64", 0, ["--spheres", "0.1", "-0.05", "0", "5", "0", "--materials", "1.4", "0.05",
                                "--lambda", "2.5", "--condenser", "0", "0.5", "--objective", "0", "0.5",
                                "--resolution", "8", "--xy", "10", "0", "--padding", "2", "--samples", "16",
                                "--recursive"]),
    "rec_xz_focus": ("f64", 0, ["--spheres", "0.5", "1", "-0.5", "1.6", "0", "-2", "-1.5", "2", "1.1", "1",
                                "--materials", "1.35", "0.02", "1.5", "0", "--lambda", "7", "--condenser", "0.1",
                                "0.45", "--objective", "0", "0.5", "--xz", "12", "0.4", "--resolution", "12",
                                "--focus", "0.5", "0", "0.3", "--amplitude", "2", "--samples", "16",
                                "--field-order", "14", "--recursive"]),
    "rec_supersample": ("f64", 0, ["--spheres", "0.23", "0.11", "0", "1.03", "0", "--materials", "1.4", "0.05",
                                   "--lambda", "1.5", "--condenser", "0", "0.5", "--objective", "0", "0.5",
                                   "--resolution", "6", "--xy", "6", "0", "--samples", "16", "--recursive"]),
    # --vector: the reference's vector stub (nfVectorUf.cu's incident field, no scattered field); stop = 5,
    # the near fields only: past sumUf the reference writes the crop's y and z components through null
    # pointers (fieldslice.cu:340-361)
    "vec_direct": ("f64", 5, TWO + ["--lambda", "3", "--condenser", "0.1", "0.6", "--objective", "0", "0.6",
                                   "--resolution", "12", "--xy", "16", "0", "--samples", "20", "--focus", "0.5",
                                   "-0.25", "0", "--vector"]),
    # --plane-wave: one incident plane wave along k instead of the focused field (nfScalarUf.cu:187,
    # nfScalarUs.cu:541, nfScalarUpLut.cu:365)
    "rec_plane_wave": ("f64", 0, TWO + ["--lambda", "3", "--objective", "0", "0.6", "--resolution", "12", "--xy",
                                       "16", "0", "--amplitude", "1.5", "--plane-wave", "--recursive"]),
    # a yz plane (it contains the beam axis, so the objective passes little of the incident field and the
    # float build's rounding of Di grows: double build only)
    "rec_yz_plane": ("f64", 0, ["--spheres", "0.3", "0.2", "-0.4", "1.8", "0", "-0.5", "3", "3", "1.2", "1",
                                "--materials", "1.42", "0.03", "1.33", "0.01", "--lambda", "2.8", "--condenser", "0",
                                "0.5", "--objective", "0", "0.55", "--yz", "14", "1.9", "--resolution", "10",
                                "--samples", "24", "--field-order", "16", "--recursive"]),
    # ptype double: the per-sphere tables of the LUT mode (sphere::calcUp and sphere.cu's sums)
    "tables_two_spheres": ("f64", 1, TWO + ["--lambda", "3", "--resolution", "12", "--xy", "16", "0",
                                           "--samples", "8"]),
    # ptype float, as the reference ships: the default LUT path with its texture fetches
    "lut_two_spheres": ("f32", 0, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                        "--resolution", "12", "--xy", "16", "0", "--samples", "20"]),
    "lut_uf_lut": ("f32", 0, ["--spheres", "1", "0.5", "0", "2", "0", "-4", "-3.5", "0.2", "1.3", "1",
                              "--materials", "1.45", "0.03", "1.3", "0.02", "--lambda", "3", "--condenser", "0.1",
                              "0.5", "--objective", "0.05", "0.45", "--resolution", "12", "--xy", "14", "0.5",
                              "--samples", "24", "--lut-uf"]),
    "lut_supersample_nu": ("f32", 0, ["--spheres", "0.23", "0.11", "0", "1.03", "0", "--materials", "1.4", "0.05",
                                      "--nu", "6666.667", "--condenser", "0", "0.5", "--objective", "0", "0.5",
                                      "--resolution", "6", "--xy", "6", "0", "--samples", "16"]),
    "vec_lut_uf_f32": ("f32", 5, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                       "--resolution", "12", "--xy", "16", "0", "--samples", "20", "--vector",
                                       "--lut-uf"]),
    "lut_plane_wave": ("f32", 0, TWO + ["--lambda", "3", "--objective", "0", "0.6", "--resolution", "12", "--xy",
                                       "16", "0", "--amplitude", "1.5", "--plane-wave"]),
    "lut_padding0": ("f32", 0, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                     "--resolution", "20", "--xy", "16", "0", "--samples", "20", "--padding", "0"]),
    "vec_direct_f32": ("f32", 5, TWO + ["--lambda", "3", "--condenser", "0.1", "0.6", "--objective", "0", "0.6",
                                       "--resolution", "12", "--xy", "16", "0", "--samples", "20", "--focus", "0.5",
                                       "-0.25", "0", "--vector"]),
    "rec_two_spheres_f32": ("f32", 0, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                            "--resolution", "12", "--xy", "16", "0", "--samples", "20",
                                            "--recursive"]),
    # stop = 3: applyBackpropagation over the plane position (z = 1.5) before the band-pass
    "rec_backprop": ("f64", 3, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                     "--resolution", "12", "--xy", "16", "1.5", "--samples", "20", "--recursive"]),
    "lut_backprop": ("f32", 3, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                     "--resolution", "12", "--xy", "16", "-2.5", "--samples", "20"]),
    # stop = 4: --extended-source, the reference's point-source driver over the nonzero pixels of an
    # 8-bit image (EXT_PGM, written to a temporary file that replaces "{image}")
    "ext_source": ("f32", 4, TWO + ["--lambda", "3", "--condenser", "0", "0.6", "--objective", "0", "0.6",
                                   "--resolution", "12", "--xy", "16", "0", "--samples", "20",
                                   "--extended-source", "{image}"]),
    # ptype float: the ring-source drivers of --interpolate 1, 2, 3 (stop = 2), their shared-memory
    # ring sums run as cooperative blocks
    "ring1_detector": ("f32", 2, TWO + RING_OPTICS + ["--focus", "0.5", "-0.25", "0", "--amplitude", "0.75",
                                                     "--interpolate", "1", "--points-rings", "5", "4"]),
    "ring2_line": ("f32", 2, TWO + RING_OPTICS + ["--interpolate", "2", "--points-rings", "7", "5"]),
    "ring2_line_pow2": ("f32", 2, TWO + RING_OPTICS + ["--focus", "0.5", "-0.25", "0", "--amplitude", "0.75",
                                                      "--interpolate", "2", "--points-rings", "8", "3"]),
    "ring0_no_rings": ("f32", 2, TWO + RING_OPTICS + ["--focus", "0.5", "-0.25", "0", "--amplitude", "0.75",
                                                     "--interpolate", "0", "--points-rings", "3", "0"]),
    "ring3_nearfield": ("f32", 2, TWO + RING_OPTICS + ["--focus", "0.5", "-0.25", "0", "--amplitude", "0.75",
                                                      "--recursive", "--interpolate", "3", "--points-rings", "4",
                                                      "3"]),
}
# stop = 6: the reference's parse of its own flags only (LoadParameters and init; nothing simulated), for
# the CLI grammar: "{dir}/name" is a file of PARSE_FILES written to a temporary directory
PARSE_FILES = {"s.txt": "1 2 0 1.5 1\n-3 0.5 0.2 2\n0 -4 -1 1.2 0\n",
               "m1.txt": "3.0 1.40 0.01\n4.0 1.45 0.03\n5.0 1.50 0.02\n",
               "m2.txt": "# [wavenumber,n,k]\n3000 1.30 0.00\n2000 1.35 0.05\n1500 1.32 0.01\n"}
PARSE = {
    "p_defaults": [],
    "p_k_direction": ["--k", "0.3", "0.5", "--xy", "20", "0", "--resolution", "16"],
    "p_explicit_plane": ["--plane-lower-left", "-4", "-3", "1", "--plane-upper-right", "4", "5", "1",
                         "--plane-normal", "0", "0", "1", "--resolution", "16"],
    "p_single_na": ["--condenser", "0.45", "--objective", "0.7", "--lambda", "2", "--resolution", "16", "--xy", "10"],
    "p_supersample_rule": ["--xy", "10", "0", "--resolution", "20", "--lambda", "0.3"],
    "p_sphere_file": ["--sphere-file", "{dir}/s.txt", "--materials", "1.4", "0.05", "1.5", "0.01", "--resolution",
                      "16", "--xy", "20", "0"],
    "p_material_files": ["--material-file", "{dir}/m1.txt", "{dir}/m2.txt", "--lambda", "4.2", "--spheres", "0", "0",
                         "0", "2", "1", "3", "3", "0", "1", "0", "--resolution", "16", "--xy", "20", "0"],
    "p_nu_xz": ["--nu", "2500", "--xz", "30", "2", "--resolution", "32"],
    "p_single_n": ["--materials", "1.33", "--spheres", "0", "0", "0", "2", "--resolution", "16"],
    "p_flags": ["--recursive-us", "--lut-uf", "--plane-wave", "--samples", "123", "--field-order", "17", "--padding",
                "2", "--amplitude", "0.5", "--focus", "1", "2", "3", "--resolution", "16", "--xy", "12", "1"],
}
TABLE_THETA_ROWS = list(range(0, 1000, 37)) + [999]


def enc(a):
    return base64.b64encode(np.ascontiguousarray(a, dtype="<f8").tobytes()).decode()


@contextlib.contextmanager
def quiet():
    """The reference prints progress to stdout and stderr; keep it out of this script's output."""
    sys.stdout.flush()
    sys.stderr.flush()
    fds = [os.dup(1), os.dup(2)]
    null = os.open(os.devnull, os.O_WRONLY)
    os.dup2(null, 1)
    os.dup2(null, 2)
    try:
        yield
    finally:
        C.CDLL(None).fflush(None)  # the reference's buffered printf output
        sys.stdout.flush()
        sys.stderr.flush()
        os.dup2(fds[0], 1)
        os.dup2(fds[1], 2)
        for fd in fds + [null]:
            os.close(fd)


def main(out_dir=HERE):
    libs = {}
    for b in ("f32", "f64"):
        path = os.path.join(REPO, "oracle", "_ref", f"libref_sim_{b}.so")
        if not os.path.exists(path):
            sys.exit("build the host-run reference first: make -C oracle ref-sim REF_DIR=<checkout>")
        lib = C.CDLL(path)
        lib.ref_sim_run.argtypes = [C.c_int, C.c_void_p, C.c_int]
        lib.ref_sim_size.restype = C.c_long
        lib.ref_sim_size.argtypes = [C.c_char_p]
        lib.ref_sim_get.argtypes = [C.c_char_p, C.c_void_p]
        libs[b] = lib
    out = {}
    tmp = tempfile.mkdtemp()
    image = os.path.join(tmp, "source.pgm")
    with open(image, "wb") as fh:
        fh.write(EXT_PGM)
    for name, (b, stop, flags) in SCENES.items():
        lib = libs[b]
        argv = ["bimsim"] + [image if f == "{image}" else f for f in flags]
        arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        with quiet():
            rc = lib.ref_sim_run(len(argv), arr, stop)
        assert rc == 0, name

        def get(key):
            n = lib.ref_sim_size(key.encode())
            if n < 0:
                return None
            v = np.zeros(n)
            lib.ref_sim_get(key.encode(), v.ctypes.data_as(C.c_void_p))
            return v

        dims = get("dims")
        # no near-field pixel within 1e-4 um of a sphere surface: there the single-precision
        # inside test (d < a) of the float build and the double-precision one could disagree
        q = get("nf_quad")
        R0, R1 = int(dims[0]), int(dims[1])
        u = np.arange(R0)[None, :, None] / R0
        v = np.arange(R1)[:, None, None] / R1
        pts = q[0:3] + q[3:6] * u + q[6:9] * v
        for s in range(int(dims[4])):
            sin = get(f"sphere{s}.in")
            gap = np.abs(np.linalg.norm(pts - sin[:3], axis=2) - sin[3]).min()
            assert gap > 1e-4, (name, s, gap)
        rec = {"build": b, "flags": flags, "stop": stop, "dims": dims.tolist(), "scene": get("scene").tolist(),
               "nf_quad": get("nf_quad").tolist(), "waves": enc(get("waves")), "spheres": []}
        for s in range(int(dims[4])):
            sp = {"in": get(f"sphere{s}.in").tolist(), "geom": get(f"sphere{s}.geom").tolist(),
                  "A": enc(get(f"sphere{s}.A")), "B": enc(get(f"sphere{s}.B"))}
            usp = get(f"sphere{s}.Usp")
            if stop == 1 and usp is not None:
                g = sp["geom"]
                dR, thetaR, aR = int(g[3]), int(g[4]), int(g[5])
                usp = usp.view(np.complex128).reshape(thetaR, dR)[TABLE_THETA_ROWS]
                uip = get(f"sphere{s}.Uip").view(np.complex128).reshape(thetaR, aR)[TABLE_THETA_ROWS]
                sp.update(theta_rows=TABLE_THETA_ROWS, Usp=enc(usp.view(np.float64)), Uip=enc(uip.view(np.float64)))
            rec["spheres"].append(sp)
        if stop in (0, 3):
            for key in ("U", "Uf", "D", "Di", "Absorbance"):
                rec[key] = enc(get(key))
        if stop == 5:
            for key in ("U", "Uf"):
                rec[key] = enc(get(key))
        if stop == 2:
            rec["rings"] = get("rings").tolist()  # mode, points, rings
            for key in ("D", "Di", "Absorbance"):
                rec[key] = enc(get(key))
        if stop == 4:
            rec["image_pgm"] = EXT_PGM.hex()
            rec["sources"] = get("sources").tolist()  # x, y, z, amplitude per source, in load order
            for key in ("D", "Di", "Absorbance"):
                rec[key] = enc(get(key))
        out[name] = rec
        print(name, b, "R =", int(dims[0]), "res =", int(dims[2]), "ss =", int(dims[3]), "waves =", int(dims[5]))
    for f, text in PARSE_FILES.items():
        with open(os.path.join(tmp, f), "w") as fh:
            fh.write(text)
    for name, flags in PARSE.items():
        lib = libs["f32"]
        argv = ["bimsim"] + [f.replace("{dir}", tmp) for f in flags]
        arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        with quiet():
            assert lib.ref_sim_run(len(argv), arr, 6) == 0, name

        def get(key):
            n = lib.ref_sim_size(key.encode())
            v = np.zeros(n)
            lib.ref_sim_get(key.encode(), v.ctypes.data_as(C.c_void_p))
            return v

        dims = get("dims")
        out[name] = {"build": "f32", "flags": flags, "stop": 6, "dims": dims.tolist(), "scene": get("scene").tolist(),
                     "nf_quad": get("nf_quad").tolist(), "files": {f: PARSE_FILES[f] for f in PARSE_FILES
                                                                   if "{dir}/" + f in flags},
                     "spheres": [{"in": get(f"sphere{s}.in").tolist()} for s in range(int(dims[4]))]}
        print(name, "parsed: R =", int(dims[0]), "spheres =", int(dims[4]))
    with open(os.path.join(out_dir, "ref_sim.json"), "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote ref_sim.json", os.path.getsize(os.path.join(out_dir, "ref_sim.json")), "bytes")

    # the reference's executable end to end (ref_sim_save: main.cpp's steps, then fileoutStruct::Save): the
    # ENVI files and the absorbance-spectrum text it writes, one run per entry of "runs" in the same
    # directory ("{dir}" in the flags)
    lib.ref_sim_save.argtypes = [C.c_int, C.c_void_p]
    optics = ["--condenser", "0", "0.6", "--objective", "0", "0.6", "--resolution", "12", "--xy", "16", "0",
              "--samples", "20"]
    outs = ["--intensity", "{dir}/i", "--incident", "{dir}/inc", "--absorbance", "{dir}/a", "--transmittance",
            "{dir}/t", "--absorbance-spec", "{dir}/as.txt"]
    cli_cases = {"nu_append": [TWO + ["--nu", nu] + optics + outs + ["--append"] for nu in ("3333.3333", "3500")],
                 "lambda_overwrite": [TWO + ["--lambda", lam] + optics + outs for lam in ("3", "3.25")]}
    files = {}
    for name, runs in cli_cases.items():
        d = tempfile.mkdtemp()
        for flags in runs:
            argv = ["bimsim"] + [f.replace("{dir}", d) for f in flags]
            arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
            with quiet():
                assert lib.ref_sim_save(len(argv), arr) == 0, name
        rec = {"runs": runs, "files": {}}
        for f in ("i", "inc", "a", "t"):
            rec["files"][f] = {"hdr": open(os.path.join(d, f + ".hdr")).read(),
                               "data": base64.b64encode(open(os.path.join(d, f), "rb").read()).decode()}
        rec["as.txt"] = open(os.path.join(d, "as.txt")).read()
        files[name] = rec
    with open(os.path.join(out_dir, "ref_cli_files.json"), "w") as fh:
        json.dump(files, fh, separators=(",", ":"))
    print("wrote ref_cli_files.json")

    # the colour map of image outputs: rts::gpu2cpu (rts/visualization/colormap.h), Brewer and gray,
    # on [0, max] as scalarslice::toImage maps a positive image (scalarslice.cu:93-138)
    lib = libs["f32"]
    lib.ref_colormap.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_int, C.c_void_p]
    rng = np.random.default_rng(11)
    vals = np.concatenate([rng.uniform(0, 3.5, 1500), np.linspace(0, 3.5, 701), [3.5, 0.0, 1.75]])
    vals = vals.astype(np.float32)
    cmap = {"values": vals.astype(np.float64).tolist(), "vmin": 0.0, "vmax": 3.5}
    for cm, name in ((0, "brewer"), (1, "gray")):
        rgb = np.zeros(3 * vals.size, np.uint8)
        lib.ref_colormap(vals.ctypes.data_as(C.c_void_p), vals.size, 0.0, 3.5, cm, rgb.ctypes.data_as(C.c_void_p))
        cmap[name] = rgb.tobytes().hex()
    with open(os.path.join(out_dir, "ref_colormap.json"), "w") as fh:
        json.dump(cmap, fh, separators=(",", ":"))
    print("wrote ref_colormap.json")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
