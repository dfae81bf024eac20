"""Serving front end without a GPU: the host-only memory estimate, and the
scheduler in dry-run mode (admission under the device-memory budget, arrival
order with bounded passing, ticket life cycle, latency percentiles)."""
import time

import numpy as np
import pytest

from bimsim_gb300 import BS_PREC_FP64, BS_PREC_MIXED, BimsimError, Server, abi, estimate_bytes, scenes


def scene(res=64, ns=3, nk=64, lut_r=256, seed=4):
    p = abi.make_params(lam=3.0, condenser=(0, 0.5), objective=(0, 0.5), xy=(100.0 * res / 1024, 0),
                        resolution=res, padding=1, lut_uf=True, us_lut_r=lut_r, us_lut_theta=256, uf_lut_r=lut_r)
    s = scenes.random_spheres(ns, 100.0 * res / 1024, 0.5, 1.5, seed=seed)
    return p, s, scenes.mc_waves(nk, 0.0, 0.5, seed=seed)


def test_estimate_counts_fields_and_tables():
    p, s, w = scene()
    R = 3 * 64
    mixed = estimate_bytes(p, s, len(w), BS_PREC_MIXED)
    fp64 = estimate_bytes(p, s, len(w), BS_PREC_FP64)
    assert mixed >= 2 * R * R * 8                      # U and Uf in complex float
    assert fp64 >= 2 * R * R * 16
    # one Usp table alone: 256 rows x 256 angles x 8 B (linear) x 2 (texture copy)
    assert mixed > 256 * 256 * 8 * 2
    # more spheres -> more table bytes
    p2, s2, _ = scene(ns=6)
    assert estimate_bytes(p2, s2, len(w), BS_PREC_MIXED) > mixed


def test_estimate_with_table_budget_is_smaller_and_rejects_too_small():
    p, s, w = scene(ns=4)
    full = estimate_bytes(p, s, len(w), BS_PREC_MIXED)
    one = 300 * 258 * 8 * 2  # a little more than one sphere's tables (rows dR + aR <= 300)
    capped = estimate_bytes(p, s, len(w), BS_PREC_MIXED, lut_budget=one)
    assert capped < full
    with pytest.raises(BimsimError):
        estimate_bytes(p, s, len(w), BS_PREC_MIXED, lut_budget=1000)


def test_dry_run_completes_every_request_with_its_own_result():
    p, s, w = scene()
    est = estimate_bytes(p, s, len(w))
    with Server(workers=3, hbm_budget=4 * est, dry_run=True) as srv:
        tickets = [srv.submit(p, s, waves=w) for _ in range(12)]
        for t in tickets:
            srv.wait(t, 10.0)
        for t in tickets:
            img, info = srv.fetch(t)
            assert img.shape == (64, 64)
            assert np.all(img == t)           # dry run: an image of the ticket number
            assert info.status == 0 and info.ms_total >= info.ms_queued >= 0
        st = srv.stats()
        assert st.completed == 12 and st.failed == 0 and st.queued == 0
        assert 0 < st.p50_ms <= st.p99_ms <= st.max_ms
        assert st.bytes_peak <= st.hbm_budget
        with pytest.raises(BimsimError):       # a fetched ticket is released
            srv.poll(tickets[0])


def test_dry_run_budget_limits_concurrency():
    p, s, w = scene()
    est = estimate_bytes(p, s, len(w))
    with Server(workers=4, hbm_budget=est + est // 2, dry_run=True) as srv:  # room for one at a time
        tickets = [srv.submit(p, s, waves=w) for _ in range(6)]
        for t in tickets:
            srv.wait(t, 10.0)
        st = srv.stats()
        assert st.completed == 6
        assert st.bytes_peak <= est + est // 2


def test_requests_of_another_shape_count_held_plus_new_bytes():
    # a context's buffers only grow, so after a request of another shape it may hold the union of
    # both allocations: with a budget below the sum, the worker gives its buffers back first
    a = scene(res=64, ns=3, nk=64)
    b = scene(res=48, ns=4, nk=128, seed=5)
    ea, eb = estimate_bytes(*a[:2], len(a[2])), estimate_bytes(*b[:2], len(b[2]))
    budget = max(ea, eb) + min(ea, eb) // 2
    with Server(workers=1, hbm_budget=budget, dry_run=True) as srv:
        tickets = [srv.submit(*(a if i % 2 == 0 else b)[:2], waves=(a if i % 2 == 0 else b)[2]) for i in range(6)]
        for t in tickets:
            srv.wait(t, 10.0)
        assert srv.stats().completed == 6 and srv.stats().bytes_peak <= budget
    with Server(workers=1, hbm_budget=ea + eb, dry_run=True) as srv:
        tickets = [srv.submit(*(a if i % 2 == 0 else b)[:2], waves=(a if i % 2 == 0 else b)[2]) for i in range(4)]
        for t in tickets:
            srv.wait(t, 10.0)
        assert srv.stats().bytes_peak > max(ea, eb)  # room for both: the buffers stay and grow


def test_request_larger_than_budget_is_rejected_or_chunked():
    p, s, w = scene(ns=4)
    full = estimate_bytes(p, s, len(w))
    with Server(workers=2, hbm_budget=1 << 20, dry_run=True) as srv:  # 1 MiB: not even the fields fit
        with pytest.raises(BimsimError) as e:
            srv.submit(p, s, waves=w)
        assert e.value.status == 3  # BS_ERR_NOMEM
    # a budget below the all-tables estimate but above one sphere at a time: admitted with chunked tables
    with Server(workers=1, hbm_budget=full - full // 8, dry_run=True) as srv:
        t = srv.submit(p, s, waves=w)
        srv.wait(t, 10.0)
        img, info = srv.fetch(t)
        assert info.status == 0


def test_small_requests_pass_a_blocked_head_a_bounded_number_of_times():
    big_p, big_s, w = scene(res=128, ns=6)
    small_p, small_s, _ = scene(res=32, ns=1)
    big = estimate_bytes(big_p, big_s, len(w))
    small = estimate_bytes(small_p, small_s, len(w))
    assert small * 4 < big
    with Server(workers=2, hbm_budget=big + small, dry_run=True) as srv:
        sub = {}
        first = srv.submit(big_p, big_s, waves=w)   # occupies most of the budget
        head = srv.submit(big_p, big_s, waves=w)    # must wait for the first
        sub[head] = time.perf_counter()
        smalls = []
        for _ in range(20):
            t = srv.submit(small_p, small_s, waves=w)
            sub[t] = time.perf_counter()
            smalls.append(t)
        for t in [first, head] + smalls:
            srv.wait(t, 20.0)
        start = {}
        for t in [first, head] + smalls:
            _, info = srv.fetch(t)
            if t in sub:
                start[t] = sub[t] + info.ms_queued * 1e-3
        assert srv.stats().completed == 22
        passed = sum(1 for t in smalls if start[t] < start[head] - 2e-4)
        assert passed <= 8, passed


def test_wait_times_out_and_bad_tickets():
    p, s, w = scene()
    est = estimate_bytes(p, s, len(w))
    with Server(workers=1, hbm_budget=2 * est, dry_run=True) as srv:
        with pytest.raises(BimsimError):
            srv.poll(12345)
        with pytest.raises(BimsimError):
            srv.submit(p, s, waves=None, n_waves=0)   # no waves
        t = srv.submit(p, s, waves=w)
        srv.wait(t, 10.0)
        assert srv.poll(t)
        srv.fetch(t)


def test_dry_run_needs_a_budget():
    with pytest.raises(BimsimError):
        Server(workers=1, hbm_budget=0, dry_run=True)


def test_fast_lane_takes_only_short_requests():
    """With 3 workers the last is a fast lane: requests above 1e11 (pixel, sphere, wave)
    interactions never run on it (short ones may run on any worker)."""
    big_p, big_s, _ = scene(res=256, ns=40)        # (768^2 px) x 40 spheres x 5000 waves = 1.2e11
    big_w = scenes.mc_waves(5000, 0.0, 0.5, seed=5)
    small_p, small_s, small_w = scene(res=32, ns=1, nk=16)
    budget = 50 * estimate_bytes(big_p, big_s, len(big_w))
    runs = []
    with Server(workers=3, hbm_budget=budget, dry_run=True) as srv:
        for i in range(12):
            big = i % 2 == 0
            p, s, w = (big_p, big_s, big_w) if big else (small_p, small_s, small_w)
            runs.append((srv.submit(p, s, waves=w), big))
        for t, _ in runs:
            srv.wait(t, 20.0)
        workers = {t: srv.fetch(t)[1].worker for t, _ in runs}
    assert len(workers) == 12
    assert all(workers[t] != 2 for t, big in runs if big)


def test_cheapest_queued_request_starts_first():
    """One worker, held by the first request; of the requests queued behind it the cheaper start
    first, whatever their arrival order (each passes the older, dearer ones at most 8 times)."""
    sizes = [(128, 8), (128, 8), (16, 1), (128, 8), (16, 1), (16, 1)]
    reqs = [scene(res=r, ns=n, nk=32) for r, n in sizes]
    budget = 10 * max(estimate_bytes(p, s, len(w)) for p, s, w in reqs)
    with Server(workers=1, hbm_budget=budget, dry_run=True) as srv:
        sub = []
        for p, s, w in reqs:
            sub.append((srv.submit(p, s, waves=w), time.perf_counter()))
        start = {}
        for t, t_sub in sub:
            srv.wait(t, 20.0)
            start[t] = t_sub + srv.fetch(t)[1].ms_queued * 1e-3
    order = sorted(range(len(sub)), key=lambda i: start[sub[i][0]])
    # after whichever request started first, the three small ones precede the remaining large ones
    rest = [i for i in order if i != order[0]]
    small = [i for i in rest if sizes[i][0] == 16]
    large = [i for i in rest if sizes[i][0] == 128]
    assert max(rest.index(i) for i in small) < min(rest.index(i) for i in large), order
