"""Every golden file under tests/golden is what its generator writes from the reference's own
sources: both reference builds are made from the checkout that BIMSIM_REF_DIR names (make -C oracle
ref ref-sim), both generators write into a temporary directory, and each file must equal the
committed one byte for byte.  Skipped where the checkout is not available (it is not on the GPU
host); about a minute with it."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
REF_DIR = os.environ.get("BIMSIM_REF_DIR", "")

pytestmark = pytest.mark.skipif(not (REF_DIR and os.path.isdir(REF_DIR)),
                                reason="set BIMSIM_REF_DIR to the reference checkout")


def test_goldens_regenerate_byte_for_byte(tmp_path):
    jobs = "-j%d" % max(1, min(8, os.cpu_count() or 1))
    subprocess.check_call(["make", "-s", jobs, "-C", os.path.join(REPO, "oracle"), "ref", "ref-sim",
                           "REF_DIR=" + REF_DIR])
    for gen in ("make_golden.py", "make_ref_sim_golden.py"):
        r = subprocess.run([sys.executable, os.path.join(GOLDEN, gen), str(tmp_path)], capture_output=True,
                           text=True, timeout=900)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    made = sorted(f for f in os.listdir(tmp_path) if f.endswith(".json"))
    committed = sorted(f for f in os.listdir(GOLDEN) if f.endswith(".json"))
    assert made == committed
    for f in made:
        with open(os.path.join(tmp_path, f), "rb") as a, open(os.path.join(GOLDEN, f), "rb") as b:
            assert a.read() == b.read(), f
