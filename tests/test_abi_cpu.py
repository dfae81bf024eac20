"""C ABI checks that need no GPU: the library loads, exports every entry point
that include/bimsim_gb300.h declares, the ctypes mirror matches the C layout,
and argument validation fails with BS_ERR_ARG before touching CUDA."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from bimsim_gb300 import abi, lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "bimsim_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(?:bs_status|const char\*)\s+(bs_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def so():
    path = lib.library_path()
    if not os.path.exists(path):
        from bimsim_gb300 import build
        build.build()
    return lib.library()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "bs_create" in names and "bs_simulate" in names and "bs_write_envi" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(so):
    missing = [n for n in declared_functions() if not hasattr(so, n)]
    assert not missing, missing


def test_struct_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "bimsim_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(bs_params), sizeof(bs_sphere), sizeof(bs_info),
         sizeof(bs_stats), offsetof(bs_params, resolution), offsetof(bs_params, reserved),
         sizeof(bs_server_config), sizeof(bs_request), offsetof(bs_request, waves), sizeof(bs_result_info),
         sizeof(bs_server_stats));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "t.c")
        exe = os.path.join(td, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe])
        vals = list(map(int, subprocess.check_output([exe]).split()))
    assert vals == [C.sizeof(abi.Params), C.sizeof(abi.Sphere), C.sizeof(abi.Info), C.sizeof(abi.Stats),
                    abi.Params.resolution.offset, abi.Params.reserved.offset, C.sizeof(abi.ServerConfig),
                    C.sizeof(abi.Request), abi.Request.waves.offset, C.sizeof(abi.ResultInfo),
                    C.sizeof(abi.ServerStats)]


def test_version_and_error_strings(so):
    assert b"sm_103a" in so.bs_version()
    assert isinstance(so.bs_last_error(), bytes)


@pytest.mark.parametrize("field,value", [("lambda_", 0.0), ("resolution", 0), ("padding", -1), ("supersample", 0),
                                         ("field_order", -2), ("us_lut_theta", 1)])
def test_bad_parameters_rejected_before_cuda(so, field, value):
    p = abi.make_params()
    setattr(p, field, value)
    h = C.c_void_p()
    st = so.bs_create(C.byref(p), C.byref(h))
    assert st == 1  # BS_ERR_ARG
    assert so.bs_last_error()


def test_condenser_order_rejected(so):
    p = abi.make_params(condenser=(0.6, 0.5))
    h = C.c_void_p()
    assert so.bs_create(C.byref(p), C.byref(h)) == 1


def test_null_arguments(so):
    assert so.bs_create(None, None) == 1
    assert so.bs_destroy(None) == 0
    assert so.bs_simulate(None, 0) == 1


def test_make_params_supersample_rule():
    # arguments.h:411-418: ss = ceil(2 s / (res lambda)) when s/res > lambda/2
    assert abi.make_params(lam=1.0, xy=(40, 0), resolution=256).supersample == 1
    assert abi.make_params(lam=0.1, xy=(40, 0), resolution=256).supersample == 4


def test_envi_writer_bytes_match_the_references_envifile(so, golden):
    """bs_envi_add_band (the writer behind bs_write_envi) against the bytes the reference's own
    EnviFile::addBand + close wrote (golden envi.json): header text and data, write then append."""
    import numpy as np
    e = golden("envi")
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "band")
        b1 = np.array(e["b1"], dtype=np.float32).reshape(e["lines"], e["samples"])
        b2 = np.array(e["b2"], dtype=np.float32).reshape(e["lines"], e["samples"])
        lib.envi_add_band(path, b1, e["wl"][0], append=False)
        assert open(path + ".hdr").read() == e["hdr_1"]
        assert open(path, "rb").read().hex() == e["dat_1"]
        lib.envi_add_band(path, b2, e["wl"][1], append=True)
        assert open(path + ".hdr").read() == e["hdr_2"]
        assert open(path, "rb").read().hex() == e["dat_2"]
        with pytest.raises(lib.BimsimError):  # a band of another size is refused (envi.h:66-89)
            lib.envi_add_band(path, np.zeros((2, 2), np.float32), 1.0, append=True)
