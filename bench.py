"""Benchmark: field-slice pixels/s of the near-field-to-detector path.

Workload (one "step" = one full slice): the 1024^2-detector scene with 50
spheres over 100 um, lambda 3 um, 1000 Monte Carlo plane waves, scalar LUT
mode with the incident-field LUT, LUTs of 4096 radial x 1024 angular samples,
padding 1 (near field 3072^2), mixed precision.  Seeded synthetic scene
(bimsim_gb300.scenes.config2); the reference publishes no dataset.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs under torch.distributed.run as independent replicas (one slice per
rank per step, no collective in the data path; weak scaling).  `--impl
reference` times the CPU implementation of the path (the double-precision
restatement in oracle/; the reference's own GPU code cannot be built: it is a
CMake project that needs the STIM library, OpenCV and FFTW, and four of its
.cu files use texture references that CUDA 12 removed) on a bounded band of
near-field rows and extrapolates.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "bimsim-cuda_gb300"))

METRIC = "field-slice pixels/s (1024², 50 spheres) & served p50/p99, mixed vs FP64 at 1e-5"
FLOP_PER_LOOKUP = 30  # (pixel, sphere, wave) interaction of the Us LUT stage


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def profile_record():
    """Per-launch DRAM bytes and shared-memory wavefronts of the dominant kernel, from the ncu
    capture recorded in profiles/us_lut_tex_config2.json (written beside its summary)."""
    try:
        return json.load(open(os.path.join(REPO, "profiles", "us_lut_tex_config2.json")))
    except (OSError, ValueError):
        return {}


def profile_traffic():
    return profile_record().get("traffic_bytes_per_launch")


def profile_wavefronts():
    return profile_record().get("shared_wavefronts_per_launch")


def measured_peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def cpu_reference(p, spheres, waves, rows, threads):
    """Time the CPU implementation of the path (the oracle, all host cores) on
    `rows` near-field rows of the slice through all spheres and waves.  The
    scene set-up and the complete lookup tables are timed once, as a whole
    slice would pay them; only the per-pixel band is scaled to the slice.
    Returns (seconds for the whole slice, R, breakdown, the band's near field
    U as complex (rows, R), its first row)."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import numpy as np

    import oracle_lib
    from bimsim_gb300 import abi
    lib = oracle_lib.load()
    g = oracle_lib.geom(p)
    R = g.R
    row0 = R // 2 - rows // 2
    arr, ns = abi.sphere_array(spheres)
    w = np.ascontiguousarray(waves, dtype=np.float64).reshape(-1)
    out = np.zeros(2 * rows * R)
    t = np.zeros(3)
    t0 = time.perf_counter()
    lib.bso_nearfield_rows_timed(oracle_lib.C.byref(p), arr, ns, oracle_lib.P(w), len(w) // 3, threads, row0,
                                 row0 + rows, oracle_lib.P(out), oracle_lib.P(t))
    wall = time.perf_counter() - t0
    total = t[0] + t[1] + t[2] * R / rows
    parts = {"setup_s": float(t[0]), "tables_s": float(t[1]), "band_s": float(t[2]), "band_rows": rows,
             "scale": R / rows, "measured_s": wall}
    return total, R, parts, out.view(np.complex128).reshape(rows, R), row0


def fp64_subset(trace, max_lookups=1e11, total_lookups=4e11):
    """Requests of the served trace that the sequential plain-FP64 comparison runs: in trace order,
    each of at most `max_lookups` (pixel, sphere, wave) lookups, until `total_lookups` are taken (a
    bounded sample of every resolution the trace holds below that size)."""
    out, acc = [], 0.0
    for i, (_, p, s, w) in enumerate(trace):
        lk = (p.resolution * p.supersample * (2 * p.padding + 1)) ** 2 * len(s) * len(w)
        if lk <= max_lookups and acc + lk <= total_lookups:
            out.append(i)
            acc += lk
    return out


def nf_pixels(p):
    return (p.resolution * p.supersample * (2 * p.padding + 1)) ** 2


def run_served(args):
    """Served workload (config 4): Poisson arrivals of seeded requests of all five resolutions
    (128^2 to 2048^2, scenes.served_trace) into the serving front end; latencies are submit -> image
    ready.  Then the same-requests comparison against sequential plain FP64: the requests of
    fp64_subset() are served mixed (all submitted at once) and run one after another in FP64, each
    on a fresh context as the reference runs one process per slice."""
    import numpy as np

    from bimsim_gb300 import BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED, Context, Server, scenes
    trace = scenes.served_trace(args.serve_requests, seed=4, resolutions=(128, 256, 512, 1024, 2048),
                                rate_hz=args.serve_rate)
    out = serve_trace(trace, args.serve_workers, args.serve_rate)
    if args.serve_light_requests > 0:
        light = scenes.served_trace(args.serve_light_requests, seed=4, resolutions=(128, 256, 512, 1024, 2048),
                                    rate_hz=args.serve_light_rate)
        out["light_load"] = serve_trace(light, args.serve_workers, args.serve_light_rate)
    if args.no_fp64:
        return out
    # ---- the same requests: served mixed (closed loop) vs sequential plain FP64 ----
    idx = fp64_subset(trace)
    sub = [trace[i] for i in idx]
    sub_pixels = sum(nf_pixels(p) for _, p, _, _ in sub)
    with Server(workers=args.serve_workers) as srv:
        t0 = time.perf_counter()
        tk = [srv.submit(p, s, waves=w, precision=BS_PREC_MIXED) for _, p, s, w in sub]
        for t in tk:
            srv.wait(t, 900.0)
            srv.fetch(t)
        wall_mixed = time.perf_counter() - t0
    def sequential(prec):
        t0 = time.perf_counter()
        for _, p, s, w in sub:
            with Context(p) as c:
                c.set_spheres(s)
                c.set_waves(w)
                c.simulate(prec)
                c.image(BS_IMG_INTENSITY)
        return time.perf_counter() - t0
    wall_mixed_seq = sequential(BS_PREC_MIXED)
    wall_fp64 = sequential(BS_PREC_FP64)
    out["same_requests_vs_fp64"] = {
        "requests": idx, "resolutions": sorted({p.resolution for _, p, _, _ in sub}),
        "nf_pixels": sub_pixels, "served_mixed_wall_s": wall_mixed, "fp64_sequential_wall_s": wall_fp64,
        "served_mixed_pixels_per_s": sub_pixels / wall_mixed, "fp64_sequential_pixels_per_s": sub_pixels / wall_fp64,
        "speedup": wall_fp64 / wall_mixed, "target": 10.0,
        "mixed_sequential_wall_s": wall_mixed_seq, "served_vs_sequential_mixed": wall_mixed_seq / wall_mixed,
        "note": "measured: the requests of the trace of at most 1e11 lookups, in trace order up to 4e11 in all; "
                "mixed through the server (all submitted at once), FP64 one fresh context per request in turn; "
                "mixed_sequential_wall_s: the same mixed requests one fresh context at a time, so "
                "served_vs_sequential_mixed is what running them side by side on the workers' streams gains"}
    return out


def serve_trace(trace, workers, rate):
    """Submit `trace` (scenes.served_trace) at its arrival times to a server of `workers` contexts;
    latencies are submit -> image ready."""
    import numpy as np

    from bimsim_gb300 import BS_PREC_MIXED, Server
    lookups = sum(nf_pixels(p) * len(s) * len(w) for _, p, s, w in trace)
    pixels = sum(nf_pixels(p) for _, p, _, _ in trace)
    by_res = {}
    with Server(workers=workers) as srv:
        t0 = time.perf_counter()
        tickets = []
        for t_arr, p, s, w in trace:
            dt = t_arr - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets.append((srv.submit(p, s, waves=w, precision=BS_PREC_MIXED), p.resolution))
        gpu_ms = 0.0
        for t, res in tickets:
            srv.wait(t, 900.0)
            _, info = srv.fetch(t)
            gpu_ms += info.ms_gpu
            by_res.setdefault(res, []).append(info.ms_total)
        wall = time.perf_counter() - t0
        st = srv.stats()
    return {"p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms, "max_ms": st.max_ms,
            "p50_ms_by_resolution": {f"{r}^2": float(np.median(v)) for r, v in sorted(by_res.items())},
            "requests": st.completed, "failed": st.failed, "lut_reuses": st.lut_reuses,
            "workers": workers, "arrival_rate_hz": rate, "wall_s": wall,
            "requests_per_s": st.completed / wall, "served_pixels_per_s": pixels / wall,
            "served_lookups_per_s": lookups / wall, "lookups": lookups, "sum_gpu_ms": gpu_ms,
            "peak_bytes": st.bytes_peak, "budget_bytes": st.hbm_budget,
            "trace": f"{len(trace)} requests, Poisson arrivals at {rate}/s; res in "
                     "{128,256,512,1024,2048}^2, S ~ U{1..200}, lambda ~ U(2.5,12.5) um, nk in {200,1000,2000}, "
                     "config-2 scene family, 25% repeat an earlier scene with new directions; mixed precision"}


def reference_host_timings():
    """Single-threaded timings of the reference's own host special-function code (oracle/_ref, built
    only where the reference checkout exists), recorded by oracle/time_reference_host.py."""
    try:
        return json.load(open(os.path.join(REPO, "profiles", "reference_host_timings.json")))
    except (OSError, ValueError):
        return None


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from bimsim_gb300 import scenes
    p, spheres, waves = scenes.config2()
    threads = os.cpu_count() or 1
    rows = args.ref_rows
    per, meas = [], []
    for i in range(args.warmup + args.steps):
        dt, R, parts, _, _ = cpu_reference(p, spheres, waves, rows, threads)
        if i >= args.warmup:
            per.append(dt)
            meas.append(parts["measured_s"])
    t_slice = statistics.median(per)
    value = R * R / t_slice
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pixels/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(meas) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "extrapolated": True,
        "config": {"workload": "config2: 1024^2 detector, 50 spheres, 1000 waves, LUT 4096x1024, near field 3072^2",
                   "sample": f"each step: scene set-up, full tables, then {rows} of {R} near-field rows through all "
                             f"spheres and waves; value = R^2 / (set-up + tables + band x {R}/{rows})"},
        "band_s": parts["band_s"], "band_rows": rows, "scale": R / rows, "setup_s": parts["setup_s"],
        "tables_s": parts["tables_s"], "slice_s_extrapolated": t_slice,
        "cpu_baseline": {"value": value, "unit": "pixels/s", "cores": threads, "kind": "port",
                         "sample": f"scene set-up and full tables once, then {rows} of {R} near-field rows x 50 "
                                   f"spheres x 1000 waves scaled by {R}/{rows} (extrapolated)"},
        "e2e": {"value": value, "unit": "pixels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_host_special_functions": reference_host_timings(),
    }
    print(json.dumps(line))


def secondary_workloads(args, flush):
    """Configs 1, 3 and a reduced config 5, timed on the device (CUDA events of the library's stream,
    summed over the slices of a step) after one warm-up run each."""
    import numpy as np
    import torch

    from bimsim_gb300 import BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED, Context, scenes
    out = {}
    # config 1: the plain method, FP64, direct order sums
    p, s, w = scenes.config1()
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(BS_PREC_FP64)
        ms = []
        for _ in range(5):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ctx.simulate(BS_PREC_FP64)
            ctx.image(BS_IMG_INTENSITY)
            ms.append(ctx.stats().ms_total)
        R = ctx.info().nf_res
        st = ctx.stats()
    out["config1"] = {"workload": "256^2 over 20 um, padding 2 (near field 1280^2), one sphere a=5 um n=1.4+0.05i, "
                                  "lambda 2.5 um, 400 waves, direct order sums, FP64",
                      "ms_per_slice": statistics.median(ms), "pixels_per_s": R * R / (statistics.median(ms) * 1e-3),
                      "ms_us": st.ms_us, "ms_uf": st.ms_uf, "ms_detector": st.ms_detector, "runs": len(ms)}
    # config 3: 16 of the 512 bands of the sweep through bs_sweep
    p, s, w, lambdas, table = scenes.config3(n_lambda=512)
    idx = np.linspace(0, 511, 16).round().astype(int)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.sweep(lambdas[idx[:2]], table[idx[:2]], precision=BS_PREC_MIXED)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.sweep(lambdas[idx], table[idx], precision=BS_PREC_MIXED)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        st = ctx.stats()
        R = ctx.info().nf_res
    out["config3"] = {"workload": "512^2 over 100 um (near field 1536^2), 50 spheres of 3 Lorentzian materials, "
                                  "1000 waves, 16 of the 512 wavelengths in 2.5-12.5 um, mixed, bs_sweep",
                      "bands": len(idx), "bands_per_s": len(idx) / wall, "ms_per_band": wall / len(idx) * 1e3,
                      "pixels_per_s": len(idx) * R * R / wall, "full_sweep_s_at_this_rate": 512 * wall / len(idx),
                      "last_band_ms_us": st.ms_us, "last_band_wave_chunk": st.lut_wave_chunk,
                      "timing": "host clock around the sweep with a device synchronize on both sides"}
    # config 5 at 512^2 (the full 4096^2 slice takes minutes): 1000 spheres, 81 orders, 2000 waves
    p, s, w = scenes.config5(resolution=512)
    with Context(p) as ctx:
        ctx.set_spheres(s)
        ctx.set_waves(w)
        ctx.simulate(BS_PREC_MIXED)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ctx.simulate(BS_PREC_MIXED)
        ctx.image(BS_IMG_INTENSITY)
        st = ctx.stats()
        R = ctx.info().nf_res
    out["config5_reduced"] = {"workload": "REDUCED config 5: 512^2 over 400 um (near field 1536^2; the benchmark "
                                          "scene is 4096^2), 1000 spheres a~U(2,20) in |z|<60 um, lambda 2 um, "
                                          "2000 waves, LUT 4096x1024, mixed",
                              "ms_per_slice": st.ms_total, "pixels_per_s": R * R / (st.ms_total * 1e-3),
                              "ms_us": st.ms_us, "ms_lut": st.ms_lut, "lookups": st.us_interactions,
                              "lookups_per_s": st.us_interactions / (st.ms_us * 1e-3)}
    return out


def run_gb300(args):
    import numpy as np
    import torch

    from bimsim_gb300 import (BS_FIELD_TOTAL, BS_IMG_ABSORBANCE, BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED,
                              Context, scenes)
    from bimsim_gb300.lib import measure_fma_peak

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    if args.small:
        # profiling case: the same pixel density and table sampling per micrometre at 256^2 (near field 768^2)
        p, spheres, waves = scenes.config2(resolution=256, fov=25.0, n_spheres=10, samples=1000, lut_r=1024)
    else:
        p, spheres, waves = scenes.config2()
    ctx = Context(p)
    ctx.set_spheres(spheres)
    ctx.set_waves(waves)
    R = ctx.info().nf_res
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (126 MB)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        ctx.simulate(BS_PREC_MIXED)
    # ---- device-resident timing (inputs already in HBM); the step time is the library's CUDA-event
    # time of the slice on its own stream (bs_stats.ms_total), the host clock is kept beside it ----
    sampler = ClockSampler(local)
    sampler.start()
    dev_ms, host_s, us_ms, launches = [], [], [], 0
    for _ in range(args.steps):
        flush.fill_(1.0)  # L2 flushed between timed steps
        barrier()
        t0 = time.perf_counter()
        ctx.simulate(BS_PREC_MIXED)
        torch.cuda.synchronize()
        host_s.append(time.perf_counter() - t0)
        st = ctx.stats()
        dev_ms.append(st.ms_total)
        us_ms.append(st.ms_us)
        launches += st.kernel_launches
    clocks = sampler.stop()
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    staged = st.lut_chunks_staged / st.lut_chunks_total if st.lut_chunks_total else 0.0
    wave_chunk = st.lut_wave_chunk
    total = sum(dev_ms) * 1e-3
    host_total = sum(host_s)
    if dist:
        t = torch.tensor([total, host_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total, host_total = float(t[0].item()), float(t[1].item())
    value = ws * args.steps * R * R / total
    # ---- end to end through the C ABI with host buffers ----
    pinned_waves = torch.from_numpy(np.ascontiguousarray(waves)).pin_memory()
    img = torch.empty((p.resolution, p.resolution), dtype=torch.float32).pin_memory()
    e2e_times = []
    d2h = 2 * p.resolution * p.resolution * 4
    h2d = len(spheres) * 48 + waves.size * 8
    for _ in range(max(1, args.steps)):
        flush.fill_(1.0)
        barrier()
        t0 = time.perf_counter()
        ctx.set_spheres(spheres)
        ctx.set_waves(pinned_waves.numpy())
        ctx.simulate(BS_PREC_MIXED)
        a = ctx.image(BS_IMG_INTENSITY)
        b = ctx.image(BS_IMG_ABSORBANCE)
        img.copy_(torch.from_numpy(a))
        e2e_times.append(time.perf_counter() - t0)
    e2e_total = sum(e2e_times)
    if dist:
        t = torch.tensor([e2e_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = ws * len(e2e_times) * R * R / e2e_total
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    # ---- roofline of the dominant kernel (Us LUT apply) ----
    fp32_tf, fp64_tf = measure_fma_peak()
    ns, nk = len(spheres), waves.shape[0]
    lookups = R * R * ns * nk
    us_s = statistics.median(us_ms) * 1e-3
    achieved = FLOP_PER_LOOKUP * lookups / us_s / 1e12
    # ---- the plain FP64 path on the same slice: its speed, and the mixed result's error against it ----
    fp64 = None
    mix_i = ctx.image(BS_IMG_INTENSITY, f64=True)  # the last end-to-end step's slice
    mix_a = ctx.image(BS_IMG_ABSORBANCE, f64=True)
    rows = args.ref_rows
    r0 = R // 2 - rows // 2
    mix_rows = ctx.field(BS_FIELD_TOTAL)[r0:r0 + rows].copy()
    f64_rows = None
    if not args.no_fp64:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.simulate(BS_PREC_FP64)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        ref_i = ctx.image(BS_IMG_INTENSITY, f64=True)
        ref_a = ctx.image(BS_IMG_ABSORBANCE, f64=True)
        f64_rows = ctx.field(BS_FIELD_TOTAL)[r0:r0 + rows].copy()
        fp64 = {"pixels_per_s": R * R / t64, "ms_per_slice": t64 * 1e3, "device_ms": ctx.stats().ms_total,
                "runs": 1, "mixed_speedup": (R * R / (total / args.steps)) / (R * R / t64),
                "note": "one FP64 slice of the same scene on the same context (no warm-up run), host-timed "
                        "with a device synchronize on both sides"}
        rel = float(np.linalg.norm(mix_i - ref_i) / np.linalg.norm(ref_i))
        rel_a = float(np.linalg.norm(mix_a - ref_a) / np.linalg.norm(ref_a))
        case = "intensity and absorbance images of this slice, mixed vs the plain FP64 GPU path"
    else:
        ps, ss, wv = scenes.config2(resolution=256, fov=25.0, n_spheres=8, samples=200)
        with Context(ps) as c2:
            c2.set_spheres(ss)
            c2.set_waves(wv)
            c2.simulate(BS_PREC_FP64)
            ref = c2.image(BS_IMG_INTENSITY, f64=True)
            ref_a = c2.image(BS_IMG_ABSORBANCE, f64=True)
            c2.simulate(BS_PREC_MIXED)
            mix = c2.image(BS_IMG_INTENSITY, f64=True)
            mix_a = c2.image(BS_IMG_ABSORBANCE, f64=True)
        rel = float(np.linalg.norm(mix - ref) / np.linalg.norm(ref))
        rel_a = float(np.linalg.norm(mix_a - ref_a) / np.linalg.norm(ref_a))
        case = "intensity and absorbance, same scene family at 256^2, 8 spheres, 200 waves"
    ctx.close()
    # ---- configs 1, 3 and a reduced config 5 (after the timed regions) ----
    extra = None if args.small or args.no_extra else secondary_workloads(args, flush)
    # ---- served latency and the same-requests FP64 comparison ----
    served = None if args.no_serve or args.small or ws > 1 else run_served(args)
    # ---- CPU baseline (oracle on a bounded band of rows) and the band's error against it ----
    cpu = None
    vs_oracle = None
    if not args.no_cpu and not args.small:
        dt, Rr, parts, band, _ = cpu_reference(p, spheres, waves, rows, os.cpu_count() or 1)
        cpu = {"value": Rr * Rr / dt, "unit": "pixels/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"double precision: scene set-up and the full lookup tables once, then {rows} of {Rr} "
                         f"near-field rows x 50 spheres x 1000 waves scaled by {Rr}/{rows} (extrapolated)",
               "parts": parts,
               # the reference's own host Bessel/Mie/table code, single-threaded as it runs it, measured
               # where its checkout exists (oracle/time_reference_host.py), with the host named
               "reference_host_special_functions": reference_host_timings()}
        nb = np.linalg.norm(band)
        vs_oracle = {"mixed": float(np.linalg.norm(mix_rows - band) / nb),
                     "fp64": None if f64_rows is None else float(np.linalg.norm(f64_rows - band) / nb),
                     "tolerance": {"mixed": 1e-4, "fp64": 1e-10},
                     "case": f"near field U of rows [{r0}, {r0 + rows}) of the full config-2 slice (all 3072 "
                             "columns, 50 spheres, 1000 waves) vs the oracle's same rows"}
    peaks = measured_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": "pixels/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "host_ms_per_step": host_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 tables and geometry)",
        "data": "synthetic (seeded Philox scene and waves)",
        "config": {"workload": ("PROFILING CASE (not the benchmark): 256^2 over 25 um, 10 spheres, LUT 1024x1024, "
                                "near field 768^2" if args.small else
                                "config2: 1024^2 detector over 100 um, 50 spheres a~U(1,5) n~U(1.2,1.6)+iU(0,.05), "
                                "lambda 3 um, 1000 MC waves, scalar LUT + Uf LUT, LUT 4096x1024, near field 3072^2"),
                   "precision": "mixed", "l2": "flushed between timed steps (256 MB write); LUTs 1.6 GB > L2",
                   "timing": "CUDA events on the library's stream around each slice (bs_stats.ms_total)",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e_value, "unit": "pixels/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "kernel": "us_lut_tex_kernel", "achieved": achieved,
                     "peak": fp32_tf, "unit": "TFLOP/s", "frac": achieved / fp32_tf,
                     "traffic": profile_traffic(),
                     "peak_source": "measured FP32 FMA loop on this GPU (bs_measure_fma_peak)",
                     "work": f"{FLOP_PER_LOOKUP} flop x {lookups} (pixel, sphere, wave) lookups per launch",
                     "launch_ms": us_s * 1e3, "lookups_per_s": lookups / us_s,
                     "staged_fraction": staged, "wave_chunk": wave_chunk,
                     "hbm_peak_gbs": peaks.get("hbm_gbs"), "fp64_peak_tflops": fp64_tf,
                     "why_not_hbm_or_tensor": "no step is a dense contraction (no tensor-core use) and the kernel "
                                              "reads ~0.14 TB/s of DRAM: it is bound by the shared-memory (L1TEX) "
                                              "pipe feeding its FP32 arithmetic, so the roofline is the measured "
                                              "FP32 FMA peak; the DRAM view is roofline_hbm, the shared-memory "
                                              "pipe roofline_l1"},
        "roofline_hbm": (None if not (profile_traffic() and peaks.get("hbm_gbs")) else
                         {"bound": "hbm", "kernel": "us_lut_tex_kernel", "unit": "GB/s",
                          "achieved": profile_traffic() / us_s / 1e9, "peak": peaks["hbm_gbs"],
                          "frac": profile_traffic() / us_s / 1e9 / peaks["hbm_gbs"],
                          "traffic": profile_traffic(), "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                          "note": "DRAM bytes of one full launch (ncu, profiles/us_lut_tex_config2.json) over this "
                                  "run's launch time"}),
        # the shared-memory (L1TEX data) pipe retires one 128-byte wavefront per SM per cycle
        "roofline_l1": (None if not (profile_wavefronts() and not args.small and clocks.get("sm_mhz")) else
                        {"bound": "shared-memory wavefronts", "kernel": "us_lut_tex_kernel",
                         "unit": "wavefronts per SM per cycle",
                         "achieved": profile_wavefronts() / (us_s * clocks["sm_mhz"] * 1e6 * n_sm),
                         "peak": 1.0,
                         "frac": profile_wavefronts() / (us_s * clocks["sm_mhz"] * 1e6 * n_sm),
                         "wavefronts": profile_wavefronts(),
                         "wavefronts_per_warp_lookup": profile_wavefronts() / (lookups / 32),
                         "note": "shared wavefronts of one full launch (ncu, profiles/us_lut_tex_config2.json) "
                                 "over this run's launch time at the sampled SM clock"}),
        "mixed_vs_fp64_rel_l2": {"value": rel, "absorbance": rel_a, "tolerance": 1e-5, "case": case},
        "mixed_vs_oracle_rows_rel_l2": vs_oracle,
        "fp64_plain": fp64,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "served": served,
        "secondary": extra,
    }
    print(json.dumps(line))


def run_workload(args):
    """Secondary workloads, one JSON line each (not the headline line):
      sweep    config 3: 512^2 config-2 scene, 50 spheres (3 Lorentzian materials), 1000 waves,
               --sweep-bands wavelengths evenly spaced in 2.5-12.5 um through bs_sweep
      config1  the plain method: 256^2 over 20 um, padding 2, one sphere a = 5 um, 400 waves,
               direct order sums, FP64
      config5  the large scene: 4096^2 over 400 um (near field 12288^2), 1000 spheres a ~ U(2, 20) in
               a slab |z| < 60 um, lambda 2 um, 2000 waves, LUT mode, mixed precision (one slice is
               about 11 minutes: run it with --warmup 0 --steps 1); --c5-resolution / --c5-samples
               shrink it for a quick check, and the JSON line then says so
    Steps: --warmup untimed and --steps timed runs of the whole workload, L2 flushed between."""
    import numpy as np
    import torch

    from bimsim_gb300 import BS_IMG_INTENSITY, BS_PREC_FP64, BS_PREC_MIXED, Context, scenes
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    if args.workload == "sweep":
        from bimsim_gb300 import dist as bdist
        p, s, w, lambdas, table = scenes.config3(n_lambda=512)
        idx = np.linspace(0, 511, args.sweep_bands).round().astype(int)
        idx = np.array(bdist.shard(list(idx), rank, ws), dtype=int)  # whole bands per rank, no collective
        lambdas, table = lambdas[idx], table[idx]
        prec = BS_PREC_MIXED
        work = f"config3: 512^2 detector over 100 um (near field 1536^2), 50 spheres, 1000 waves, " \
               f"{len(lambdas)} of the 512 wavelengths in 2.5-12.5 um, LUT 4096x1024"
    elif args.workload == "config5":
        p, s, w = scenes.config5(resolution=args.c5_resolution, samples=args.c5_samples)
        lambdas = table = None
        prec = BS_PREC_MIXED
        full = args.c5_resolution == 4096 and args.c5_samples == 2000
        work = ("config5" if full else "REDUCED config5") + \
            f": {args.c5_resolution}^2 over 400 um, 1000 spheres a~U(2,20) in |z|<60 um, lambda 2 um, " \
            f"{args.c5_samples} waves, LUT 4096x1024, mixed"
    else:
        p, s, w = scenes.config1()
        lambdas = table = None
        prec = BS_PREC_FP64
        work = "config1: 256^2 over 20 um, padding 2 (near field 1280^2), one sphere a=5 um n=1.4+0.05i, " \
               "lambda 2.5 um, 400 waves, direct order sums (--recursive)"
    torch.cuda.set_device(local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ctx = Context(p)
    ctx.set_spheres(s)
    ctx.set_waves(w)
    R = ctx.info().nf_res

    def step():
        if lambdas is not None:
            ctx.sweep(lambdas, table, precision=prec, images=True)
        else:
            ctx.simulate(prec)
            ctx.image(BS_IMG_INTENSITY)

    for _ in range(args.warmup):
        step()
    sampler = ClockSampler(local)
    sampler.start()
    times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        if ws > 1:
            tdist.barrier()
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    st = ctx.stats()
    per = statistics.median(times)
    nb = len(lambdas) if lambdas is not None else 1
    if ws > 1:
        # every rank's bands (a sweep) or one replica slice per rank, over the slowest rank's time
        from bimsim_gb300 import dist as bdist
        per = bdist.max_over_ranks(per, device="cuda")
        nb = args.sweep_bands if lambdas is not None else ws
        tdist.destroy_process_group()
        if rank != 0:
            return
    metric = ("sweep bands/s" if lambdas is not None else
              "field-slice pixels/s (plain FP64 direct)" if args.workload == "config1" else
              "field-slice pixels/s (config 5, mixed)")
    line = {"metric": metric,
            "value": nb / per if lambdas is not None else nb * R * R / per,
            "unit": "bands/s" if lambdas is not None else "pixels/s",
            "field_slice_pixels_per_s": nb * R * R / per, "n_gpus": ws, "steps": args.steps,
            "scaling": "weak" if lambdas is None else "strong (bands sharded over ranks)",
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "dtype": "f32 (FP64 tables and geometry)" if prec == BS_PREC_MIXED else "f64",
            "data": "synthetic (seeded)", "config": {"workload": work, "l2": "flushed between steps"},
            "last_band_stats": {"ms_us": st.ms_us, "ms_lut": st.ms_lut, "ms_uf": st.ms_uf, "ms_detector": st.ms_detector,
                                "ms_total": st.ms_total, "interactions": st.us_interactions},
            "clocks": clocks}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-rows", type=int, default=int(os.environ.get("BS_REF_ROWS", "12")))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip configs 1, 3 and the reduced config 5")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 slice (about 40 s on config 2)")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: config-2 scene family at 256^2 over 25 um, 10 spheres, LUT 1024 x 1024")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-rate", type=float, default=4.0)
    ap.add_argument("--serve-workers", type=int, default=6)
    ap.add_argument("--serve-light-requests", type=int, default=16,
                    help="a second served run below saturation (0 skips it)")
    ap.add_argument("--serve-light-rate", type=float, default=0.5)
    ap.add_argument("--workload", default="slice", choices=["slice", "sweep", "config1", "config5"])
    ap.add_argument("--c5-resolution", type=int, default=4096)
    ap.add_argument("--c5-samples", type=int, default=2000)
    ap.add_argument("--sweep-bands", type=int, default=64)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "slice":
        run_workload(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
