"""bs_mie_noalloc: Mie coefficients for callers that cannot allocate device
memory (inside CUDA stream capture, allocation-free serving loops, frameworks
owning device memory through their own pool).  Checked through the C ABI
against the context path (bs_simulate + bs_get_mie) and the oracle at the
double-precision tolerance of the other parity tests, on two calls in a row."""
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
            oa, ob = oracle_mie(k, spheres[i], n - 1)
            assert rel(ga, oa) <= TOL and rel(gb, ob) <= TOL, (call, i, rel(ga, oa), rel(gb, ob))
            assert not np.any(a[i, n:]) and not np.any(b[i, n:])  # orders above the sphere's own Nl


def test_mie_noalloc_small_sphere_beside_a_large_one_at_the_order_limit():
    """k a from 0.25 to 63 in one call with nl = 127: every entry finite, each sphere's orders up to its
    own Nl equal to the oracle's, zeros above."""
    import torch

    so = lib.library()
    lam = 2.0
    k = 2 * float(np.float32(3.14159)) / lam
    spheres = [(0.08, 1.4, 0.05), (20.0, 1.4, 0.02), (0.5, 1.6, 0.0), (7.3, 1.2, 0.04)]
    dev = torch.device("cuda")
    sph = torch.tensor(spheres, dtype=torch.float64, device=dev)
    A = torch.full((len(spheres), 128, 2), np.nan, dtype=torch.float64, device=dev)
    B = torch.full_like(A, np.nan)
    st = so.bs_mie_noalloc(C.c_void_p(sph.data_ptr()), len(spheres), 127, k, C.c_void_p(A.data_ptr()),
                           C.c_void_p(B.data_ptr()), None)
    assert st == 0, so.bs_last_error()
    torch.cuda.synchronize()
    a, b = A.cpu().numpy(), B.cpu().numpy()
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    for i, (rad, nre, nim) in enumerate(spheres):
        nl = abi_nl(rad, lam)
        oa, ob = oracle_mie(k, (0, 0, 0, rad, nre, nim), nl)
        assert rel(a[i, :nl + 1, 0] + 1j * a[i, :nl + 1, 1], oa) <= TOL
        assert rel(b[i, :nl + 1, 0] + 1j * b[i, :nl + 1, 1], ob) <= TOL
        assert not np.any(a[i, nl + 1:]) and not np.any(b[i, nl + 1:])


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


def oracle_mie(k, sphere, nl):
    import oracle_lib
    A = np.zeros(2 * nl + 2)
    B = np.zeros(2 * nl + 2)
    oracle_lib.load().bso_mie(k, sphere[3], sphere[4], sphere[5], nl, oracle_lib.P(A), oracle_lib.P(B))
    return A.view(np.complex128), B.view(np.complex128)
