"""Material files (bs_material_eval, the CLI's --material-file) against golden
vectors recorded from the reference's own rts::material<float> (see
tests/golden/make_golden.py): column formats, sorting, the swapped
interpolation weights, clamping, dropped signs.  Host code, no GPU."""
import json
import os

import numpy as np
import pytest

from bimsim_gb300 import BimsimError, lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "material.json")


@pytest.mark.parametrize("case", sorted(json.load(open(GOLDEN))))
def test_material_file_matches_reference(case, tmp_path):
    g = json.load(open(GOLDEN))[case]
    path = tmp_path / "m.txt"
    path.write_text(g["text"])
    n = lib.material_eval(path, g["lambda"])
    ref = np.array(g["n"]).view(np.complex128)
    assert np.array_equal(n, ref), (case, n, ref)


def test_weights_are_swapped_like_the_reference(tmp_path):
    path = tmp_path / "m.txt"
    path.write_text("2.0 1.0 0.0\n4.0 2.0 0.0\n")
    # at 2.5 (a quarter of the way) the reference returns 1.0*0.25 + 2.0*0.75
    assert lib.material_eval(path, [2.5])[0] == pytest.approx(1.75)


def test_missing_file_and_short_lines(tmp_path):
    with pytest.raises(BimsimError):
        lib.material_eval(tmp_path / "none.txt", [1.0])
    bad = tmp_path / "bad.txt"
    bad.write_text("2.0 1.4\n")
    with pytest.raises(BimsimError):
        lib.material_eval(bad, [2.0])
    blank = tmp_path / "blank.txt"
    blank.write_text("2.0 1.4 0.1\n\n3.0 1.5 0.2\n")  # the reference never returns on the blank line
    assert lib.material_eval(blank, [3.0])[0] == pytest.approx(1.5 + 0.2j)
