"""Reader of tests/golden/ref_sim.json: golden outputs of the reference's own path run on the CPU
(recorded by tests/golden/make_ref_sim_golden.py from the host-run build of the reference's
sources).  Rebuilds each scene's bs_params and spheres from the inputs as the reference held them
after parsing its flags."""
import base64
import json
import os

import numpy as np

from bimsim_gb300 import abi

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_sim.json")
_cache = None


def load():
    global _cache
    if _cache is None:
        with open(PATH) as fh:
            _cache = json.load(fh)
    return _cache


def arr(b64):
    return np.frombuffer(base64.b64decode(b64), dtype="<f8").copy()


def values(flags, name):
    """The single-precision values that follow --name, up to the next flag."""
    i = flags.index("--" + name) + 1
    out = []
    while i < len(flags) and not flags[i].startswith("--"):
        out.append(float(np.float32(flags[i])))
        i += 1
    return out


def flag(flags, name, n):
    return values(flags, name)[:n]


def plane(flags):
    """(pmin, pmax, normal) as lImagePlane builds them in single precision (arguments.h:340-407): an
    axis-aligned plane of size s (default 40) at a position (default 0), else the explicit corners and
    normal (defaults (-5, 0, -5), (5, 0, 5), (0, 1, 0))."""
    f = np.float32
    for name in ("xy", "xz", "yz"):
        if "--" + name in flags:
            v = values(flags, name)
            s = v[0] if v else 40.0
            pos = v[1] if len(v) > 1 else 0.0
            h = float(f(s) / f(2))
            if name == "xy":
                return (-h, -h, pos), (h, h, pos), (0.0, 0.0, 1.0)
            if name == "xz":
                return (-h, pos, -h), (h, pos, h), (0.0, -1.0, 0.0)
            return (pos, -h, -h), (pos, h, h), (1.0, 0.0, 0.0)

    def vec(name, default):
        return tuple(values(flags, name)) if "--" + name in flags else tuple(float(f(v)) for v in default)
    return vec("plane-lower-left", (-5, 0, -5)), vec("plane-upper-right", (5, 0, 5)), vec("plane-normal", (0, 1, 0))


def plane_size(flags):
    """s of the supersampling rule: the --xy size, else 40 (arguments.h:346-418)."""
    if "--xy" in flags:
        v = values(flags, "xy")
        return v[0] if v else 40.0
    return 40.0


def params(rec):
    sc, dims = rec["scene"], rec["dims"]
    pmin, pmax, nrm = plane(rec["flags"])
    p = abi.make_params(lam=sc[0], amplitude=sc[1], k_dir=tuple(sc[2:5]), focus=tuple(sc[5:8]),
                        condenser=tuple(sc[8:10]), objective=tuple(sc[10:12]), plane=(pmin, pmax, nrm),
                        resolution=int(dims[2]), padding=int(sc[12]), supersample=int(sc[13]),
                        field_order=int(sc[14]), lut_us=bool(sc[15]), lut_uf=bool(sc[16]), plane_wave=bool(sc[17]),
                        scalar="--vector" not in rec["flags"])
    return p


def spheres(rec):
    return [tuple(s["in"]) for s in rec["spheres"]]


def waves(rec):
    return arr(rec["waves"]).reshape(-1, 3)


def field(rec, key):
    R0, R1 = int(rec["dims"][0]), int(rec["dims"][1])
    return arr(rec[key]).view(np.complex128).reshape(R1, R0)


def image(rec, key):
    res = int(rec["dims"][2])
    return arr(rec[key]).reshape(res, res)


def scenes(build=None, full=True):
    """Single-source scenes: the whole path (full) or the tables only."""
    d = load()
    return sorted(n for n, r in d.items()
                  if r["stop"] in (0, 1) and (build is None or r["build"] == build) and (r["stop"] == 0) == full)


def nearfield_scenes(build=None):
    """Scenes recorded up to sumUf (the near fields U and Uf only)."""
    return sorted(n for n, r in load().items() if r["stop"] == 5 and (build is None or r["build"] == build))


def backprop_scenes(build=None):
    """Whole-path scenes with applyBackpropagation before the band-pass."""
    return sorted(n for n, r in load().items() if r["stop"] == 3 and (build is None or r["build"] == build))


def plane_position(rec):
    """z_d, the propagation distance: the plane position of --xy/--xz/--yz as a float (arguments.h:346-409)."""
    for name in ("xy", "xz", "yz"):
        if "--" + name in rec["flags"]:
            v = values(rec["flags"], name)
            return v[1] if len(v) > 1 else 0.0
    return 0.0


def parse_scenes():
    """The reference's parse of its own flags, nothing simulated (CLI grammar cases)."""
    return sorted(n for n, r in load().items() if r["stop"] == 6)


def flags_with_files(rec, directory):
    """The record's flags with its files written into `directory` ("{dir}" replaced)."""
    for name, text in rec.get("files", {}).items():
        with open(os.path.join(str(directory), name), "w") as fh:
            fh.write(text)
    return [f.replace("{dir}", str(directory)) for f in rec["flags"]]


def source_scenes():
    """Scenes run through the reference's extended-source driver (--extended-source)."""
    return sorted(n for n, r in load().items() if r["stop"] == 4)


def sources(rec):
    """The point sources (x, y, z, amplitude) the reference loaded from the scene's image."""
    return np.array(rec["sources"]).reshape(-1, 4)


def ring_scenes():
    """Scenes run through the reference's ring-source drivers (--interpolate 1, 2, 3)."""
    return sorted(n for n, r in load().items() if r["stop"] == 2)


def rings(rec):
    """(mode, points, rings) of a ring scene."""
    return tuple(int(v) for v in rec["rings"])
