"""Serving front end on the GPU: results are bit-identical alone and in a
concurrent mix, tables are reused for a repeated scene with identical
results, and the device-memory budget holds."""
import numpy as np
import pytest

from bimsim_gb300 import (BS_IMG_ABSORBANCE, BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED, Context, Server, abi,
                          estimate_bytes, scenes)

pytestmark = pytest.mark.gpu


def request(i):
    """A seeded mix of the served workload's shapes, scaled down (config 4 uses 128^2..2048^2)."""
    rng = np.random.default_rng(100 + i)
    res = int(rng.choice([32, 48, 64]))
    ns = int(rng.integers(1, 5))
    lam = float(rng.uniform(2.5, 12.5))
    nk = int(rng.choice([64, 128, 200]))
    fov = 100.0 * res / 1024 * 4
    p = abi.make_params(lam=lam, condenser=(0, 0.5), objective=(0, 0.5), xy=(fov, 0), resolution=res, padding=1,
                        lut_uf=True, us_lut_r=256, us_lut_theta=256, uf_lut_r=256)
    s = scenes.random_spheres(ns, fov, 0.5, 2.0, seed=200 + i)
    w = scenes.mc_waves(nk, 0.0, 0.5, seed=300 + i)
    prec = BS_PREC_FP64 if i % 4 == 3 else BS_PREC_MIXED
    kind = BS_IMG_ABSORBANCE if i % 3 == 2 else BS_IMG_INTENSITY
    return p, s, w, prec, kind


def alone(p, s, w, prec, kind):
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(prec)
        return ctx.image(kind)


def test_results_identical_alone_and_in_the_mix():
    reqs = [request(i) for i in range(10)]
    ref = [alone(*r) for r in reqs]
    with Server(workers=4) as srv:
        tickets = [srv.submit(p, s, waves=w, precision=prec, image=kind) for p, s, w, prec, kind in reqs]
        for t in tickets:
            srv.wait(t, 120.0)
        workers = set()
        for t, r in zip(tickets, ref):
            img, info = srv.fetch(t)
            workers.add(info.worker)
            assert np.array_equal(img, r, equal_nan=True)
        st = srv.stats()
        assert st.completed == 10 and st.failed == 0
        assert st.bytes_peak <= st.hbm_budget
        assert st.p50_ms > 0 and st.p99_ms >= st.p50_ms
    assert len(workers) > 1  # the mix ran on several contexts


def test_repeated_scene_reuses_tables_with_identical_results():
    p, s, w, _, _ = request(1)
    w2 = scenes.mc_waves(len(w), 0.0, 0.5, seed=999)
    with Server(workers=2) as srv:
        a = srv.submit(p, s, waves=w)
        srv.wait(a, 60.0)
        img_a, info_a = srv.fetch(a)
        b = srv.submit(p, s, waves=w2)       # same scene, other directions: same tables
        srv.wait(b, 60.0)
        img_b, info_b = srv.fetch(b)
        assert info_a.lut_reused == 0 and info_b.lut_reused == 1
        assert info_b.worker == info_a.worker
        assert srv.stats().lut_reuses == 1
    assert np.array_equal(img_a, alone(p, s, w, BS_PREC_MIXED, BS_IMG_INTENSITY))
    assert np.array_equal(img_b, alone(p, s, w2, BS_PREC_MIXED, BS_IMG_INTENSITY))


def test_tight_budget_runs_requests_one_at_a_time():
    reqs = [request(i) for i in range(4)]
    need = max(estimate_bytes(p, s, len(w), prec) for p, s, w, prec, _ in reqs)
    budget = need + need // 4
    ref = [alone(*r) for r in reqs]
    with Server(workers=3, hbm_budget=budget) as srv:
        tickets = [srv.submit(p, s, waves=w, precision=prec, image=kind) for p, s, w, prec, kind in reqs]
        for t in tickets:
            srv.wait(t, 120.0)
        for t, r in zip(tickets, ref):
            img, _ = srv.fetch(t)
            assert np.array_equal(img, r, equal_nan=True)
        assert srv.stats().bytes_peak <= budget


@pytest.mark.parametrize("i", range(6))
def test_estimate_covers_what_a_context_allocates(i):
    p, s, w, prec, kind = request(i)
    est = estimate_bytes(p, s, len(w), prec)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(prec)
        ctx.image(kind)
        held = ctx.info().device_bytes
    assert held <= est <= held * 1.05 + 4096, (held, est)


def test_a_failing_request_leaves_the_others_intact():
    """A request the library rejects at run time (mixed-precision tables taller than the GPU's
    gather-texture limit) fails alone: its fetch raises with the message, the rest complete."""
    from bimsim_gb300 import BimsimError
    good = [request(i) for i in range(3)]
    ref = [alone(*r) for r in good]
    bad_p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(16, 0), resolution=16, padding=1,
                            us_lut_r=70000, us_lut_theta=16)
    with Server(workers=2) as srv:
        tickets = [srv.submit(p, s, waves=w, precision=prec, image=kind) for p, s, w, prec, kind in good[:2]]
        bad = srv.submit(bad_p, [(0, 0, 0, 2.0, 1.4, 0.05)], waves=scenes.mc_waves(8, 0, 0.5, seed=1))
        p, s, w, prec, kind = good[2]
        tickets.append(srv.submit(p, s, waves=w, precision=prec, image=kind))
        for t in tickets + [bad]:
            srv.wait(t, 120.0)
        with pytest.raises(BimsimError) as e:
            srv.fetch(bad)
        assert "texture limit" in str(e.value)
        for t, r in zip(tickets, ref):
            img, info = srv.fetch(t)
            assert np.array_equal(img, r, equal_nan=True)
        st = srv.stats()
        assert st.completed == 3 and st.failed == 1


def test_stream_priority_keeps_results_identical():
    """bs_set_stream_priority moves the context to a new stream of that priority (the server gives
    cheap requests the higher ones); the slice's bits do not change."""
    p, s, w, prec, kind = request(2)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(BS_PREC_MIXED)
        a = ctx.image(BS_IMG_INTENSITY)
        assert ctx.lib.bs_set_stream_priority(ctx.h, -1000) == 0  # clamped to the device's greatest
        ctx.simulate(BS_PREC_MIXED)
        b = ctx.image(BS_IMG_INTENSITY)
        assert ctx.lib.bs_set_stream_priority(ctx.h, 0) == 0
        ctx.simulate(BS_PREC_MIXED)
        c = ctx.image(BS_IMG_INTENSITY)
    assert np.array_equal(a, b) and np.array_equal(a, c)
