"""bs_mie_noalloc: Mie coefficients for callers that cannot allocate device
memory (inside CUDA stream capture, allocation-free serving loops, frameworks
owning device memory through their own pool).  Checked through the C ABI
against the context path (bs_simulate + bs_get_mie) at the double-precision
tolerance of the other parity tests, on two calls in a row."""
import ctypes as C

import numpy as np
import pytest

from bimsim_gb300 import BS_PREC_FP64, Context, abi, lib, scenes

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same bound as test_gpu_parity.test_mie_coefficients_fp64


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_mie_noalloc_matches_context_path_twice():
    import torch

    so = lib.library()
    lam = 2.5
    spheres = [(0.0, 0.0, 0.0, 5.0, 1.4, 0.05),      # k a = 12.57: the cbessjy.cpp:541 branch
               (6.0, -4.0, 0.5, 1.3, 1.55, 0.01),
               (-5.0, 5.0, -1.0, 2.7, 1.25, 0.0)]
    p = abi.make_params(lam=lam, condenser=(0, 0.5), objective=(0, 0.5), xy=(24, 0), resolution=12, padding=1,
                        lut_us=False)
    with Context(p) as ctx:
        ctx.set_spheres(spheres)
        ctx.set_waves(scenes.mc_waves(8, 0, 0.5, seed=3))
        ctx.simulate(BS_PREC_FP64)
        ref = []
        for i, s in enumerate(spheres):
            nl = abi_nl(s[3], lam)
            ref.append(ctx.mie(i, nl))
    nl_max = max(len(a) - 1 for a, _ in ref)
    k = 2 * float(np.float32(3.14159)) / lam
    dev = torch.device("cuda")
    sph = torch.tensor([[s[3], s[4], s[5]] for s in spheres], dtype=torch.float64, device=dev)
    A = torch.zeros((len(spheres), nl_max + 1, 2), dtype=torch.float64, device=dev)
    B = torch.zeros_like(A)
    for call in range(2):
        A.fill_(np.nan)
        B.fill_(np.nan)
        torch.cuda.synchronize()
        st = so.bs_mie_noalloc(C.c_void_p(sph.data_ptr()), len(spheres), nl_max, k, C.c_void_p(A.data_ptr()),
                               C.c_void_p(B.data_ptr()), None)
        assert st == 0, so.bs_last_error()
        torch.cuda.synchronize()
        a = A.cpu().numpy()
        b = B.cpu().numpy()
        for i, (ra, rb) in enumerate(ref):
            n = len(ra)
            ga = a[i, :n, 0] + 1j * a[i, :n, 1]
            gb = b[i, :n, 0] + 1j * b[i, :n, 1]
            assert rel(ga, ra) <= TOL, (call, i, rel(ga, ra))
            assert rel(gb, rb) <= TOL, (call, i, rel(gb, rb))


def test_mie_noalloc_rejects_sizes_beyond_the_work_space():
    so = lib.library()
    dummy = C.c_void_p(1)
    assert so.bs_mie_noalloc(dummy, 257, 10, 2.0, dummy, dummy, None) == 1
    assert b"256" in so.bs_last_error()
    assert so.bs_mie_noalloc(dummy, 1, 128, 2.0, dummy, dummy, None) == 1
    assert b"127" in so.bs_last_error()


def abi_nl(a, lam):
    import oracle_lib
    return oracle_lib.load().bso_calc_nl(a, lam)
