"""Workloads of the benchmark configurations other than the headline one
(used by bench.py --config N).

  1  plain FP64 integral + update, 10,368 cells x 200 directions (Thomson)
  3  multigroup HG: 300,000 cells x 590 directions x 8 groups, g = 0.7,
     lambda_g = 0.3 + 0.08 g, split-precision paths against FP64
  4  64 uneven problems in one persistent launch per step, replayed from a
     CUDA graph (N log-uniform in [5k, 200k], M in {146, 302, 590}, Thomson
     or HG with g ~ U[0, 0.8], lambda ~ U[0.2, 0.95], seed 3)
  5  serving: Poisson arrivals at 10-120 % of measured saturation, requests
     with N lognormal (median 50,000, clipped to [2,000, 500,000]), M in
     {110, 302, 590, 1202}, HG g ~ U[0, 0.8], 5-40 iterations, 120 GB cap

All inputs are synthetic and seeded; FP64 references for the accuracy
columns are computed here with numpy on a sample of cells.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

M64 = (1 << 64) - 1


# ---------------------------------------------------------------- counter hash (as the library's)
def _mix64(z):
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(M64)
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(M64)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(M64)
    return z ^ (z >> np.uint64(31))


def _key(seed: int, stream: int):
    with np.errstate(over="ignore"):
        return _mix64(np.uint64((seed * 0x632BE59BD9B4E019 + stream) & M64))


def hash_uniform(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        r = _mix64(_key(seed, stream) ^ _mix64(idx.astype(np.uint64)))
    return ((r >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def hash_lognormal(seed: int, stream: int, idx: np.ndarray, mu: float, sigma: float) -> np.ndarray:
    idx = idx.astype(np.uint64)
    u1 = hash_uniform(seed, stream, 2 * idx)
    u2 = hash_uniform(seed, stream, 2 * idx + 1)
    return np.exp(mu + sigma * (np.sqrt(-2.0 * np.log(u1)) * np.cos(2 * math.pi * u2)))


# ---------------------------------------------------------------- direction sets and weights
def fibonacci(M: int):
    i = np.arange(M, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / M
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = math.pi * (3.0 - math.sqrt(5.0)) * i
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1), np.full(M, 4 * math.pi / M), 4 * math.pi


def weights(M: int, phase: int, g: float) -> np.ndarray:
    xyz, area, fa = fibonacci(M)
    mu = xyz @ xyz.T  # [j][k]
    if phase == 0:
        return (3.0 * (1.0 + mu * mu) / 4.0) * area[:, None] / fa
    den = 1.0 + g * g - 2.0 * g * mu
    w = area[:, None] * (1.0 - g * g) / (4.0 * math.pi * den * np.sqrt(den))
    return w / w.sum(axis=0, keepdims=True)


def batch_reference(N, M, G, phase, g, seed, lam, cells, mu=0.0, sigma=1.0):
    """FP64 S [G][M][len(cells)] of one step for the device-generated inputs."""
    W = weights(M, phase, g)
    out = np.empty((G, M, len(cells)))
    for gi in range(G):
        idx = ((gi * M + np.arange(M))[:, None] * N + cells[None, :]).ravel()
        ibar = hash_lognormal(seed, 1, idx, mu, sigma).astype(np.float32).astype(np.float64).reshape(M, len(cells))
        B = (0.1 + 0.9 * hash_uniform(seed, 2, gi * N + cells)).astype(np.float32).astype(np.float64)
        out[gi] = (1.0 - lam[gi]) * B[None, :] + lam[gi] * (W.T @ ibar)
    return out


def rel_stats(a, b):
    r = np.abs(a - b) / np.abs(b)
    return float(r.max()), float(r.mean())


# ---------------------------------------------------------------- timing helper
def timed_steps(ctx, fn, steps, torch, stream_handle):
    stream = torch.cuda.ExternalStream(stream_handle)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


# ---------------------------------------------------------------- configurations
def config3(pkg, native, ctx, torch, steps, warmup, precision):
    N, M, G, g = 300_000, 590, 8, 0.7
    # schedule for M = 590 at this cell count (not timed)
    best, tried = ctx.autotune_schedule(M, precision, cells=N * G)
    lam = np.array([0.3 + 0.08 * i for i in range(G)])
    desc = native.problem_desc(N, M, G, 1, g, precision)
    b = native.Batch(ctx)
    pid = b.add_synthetic(desc, 2, 0.0, 1.0, 0.1, 1.0, lam)
    for _ in range(warmup):
        b.step(False)
    ctx.kernel_timing(True)
    t = timed_steps(ctx, lambda: b.step(False), steps, torch, ctx.stream_handle(pkg.STREAM_SCATTERING_1))
    kms, kn = ctx.kernel_timing(False)
    S, _ = b.read(pid)
    cells = np.arange(0, N, N // 64)[:64]
    ref = batch_reference(N, M, G, 1, g, 2, lam, cells)
    mx, mean = rel_stats(S[:, :, cells].astype(np.float64), ref)
    b.close()
    units = N * M * G
    return {"value": units * steps / t / 1e9, "ms_per_step": t / steps * 1e3, "kernel_ms": kms / max(kn, 1),
            "tflops_alg": 2.0 * N * G * M * M / (kms / max(kn, 1) / 1e3) / 1e12,
            "max_rel_err": mx, "mean_rel_err": mean, "precision": precision,
            "workload": "300,000 cells x 590 directions x 8 groups, HG g=0.7 row-normalised, lognormal(0,1) FP32, "
                        "lambda_g=0.3+0.08g",
            "autotuned": {x: best[x] for x in ("flush", "bn", "order", "ms")}, "schedules_timed": len(tried)}


def moments_pass(pkg, native, ctx, torch, steps, warmup, N=663_552):
    """The FP64 moment kernels on the config 2 Illum (663,552 cells x 1000
    directions, 21.2 GB resident): energy + flux (rts_moments), and energy,
    flux, impulse tensor and both divergences in one pass (rts_illum_params,
    synthetic cell geometry).  Kernel times from CUDA events on the kernels'
    stream; FP64 flops per (cell, direction): 12 and 59."""
    M = 1000
    xyz, area, fa = native.synth_directions(M)
    ctx.init(xyz, area, fa, N)
    ctx.synth_illum(1, 0.0, 1.5)
    rng = np.random.default_rng(3)
    nrm = rng.normal(size=(N, 4, 3))
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    ctx.set_geometry(nrm, rng.uniform(0.5, 1.0, size=(N, 4)), rng.uniform(0.5, 1.0, size=N))
    out = {}
    for name, fn, flops in (("moments", lambda: ctx.moments(), 12),
                            ("illum_params", lambda: ctx.illum_params(), 59)):
        for _ in range(warmup):
            fn()
        ctx.kernel_timing(True)
        for _ in range(steps):
            fn()
        kms, kn = ctx.kernel_timing(False)
        sec = kms / max(kn, 1) / 1e3
        nbytes = N * M * 32 + N * (4 if name == "moments" else 17) * 8
        out[name] = {"kernel_ms": sec * 1e3, "fp64_tflops": flops * N * M / sec / 1e12,
                     "hbm_gbs": nbytes / sec / 1e9, "flops_per_cell_dir": flops, "bytes": nbytes}
    return out


def config4_problems(seed=3):
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(64):
        N = int(round(math.exp(rng.uniform(math.log(5000), math.log(200000)))))
        M = int(rng.choice([146, 302, 590]))
        hg = bool(rng.integers(0, 2))
        g = float(rng.uniform(0.0, 0.8)) if hg else 0.0
        lam = float(rng.uniform(0.2, 0.95))
        probs.append((N, M, 1 if hg else 0, g, lam, 1000 + i))
    return probs


def config4(pkg, native, ctx, torch, steps, warmup, precision):
    probs = config4_problems()
    # schedule per direction count (drain period, width, order), not timed
    tuned = {M: ctx.autotune_schedule(M, precision)[0] for M in sorted({p[1] for p in probs})}
    b = native.Batch(ctx)
    ids = []
    for (N, M, ph, g, lam, seed) in probs:
        desc = native.problem_desc(N, M, 1, ph, g, precision)
        ids.append(b.add_synthetic(desc, seed, 0.0, 1.0, 0.1, 1.0, [lam]))
    # accuracy after one step on sampled cells of a few problems
    b.step(False)
    errs = []
    for k in (0, 17, 42, 63):
        N, M, ph, g, lam, seed = probs[k]
        S, _ = b.read(ids[k])
        cells = np.linspace(0, N - 1, 16).astype(np.int64)
        ref = batch_reference(N, M, 1, ph, g, seed, [lam], cells)
        errs.append(rel_stats(S[:, :, cells].astype(np.float64), ref))
    per_graph = max(1, min(steps, 8))
    b.capture(per_graph, True)
    for _ in range(max(1, warmup // per_graph)):
        b.replay()
    replays = max(1, steps // per_graph)
    ctx.kernel_timing(True)
    launches0 = ctx.launch_count()
    t = timed_steps(ctx, b.replay, replays, torch, ctx.stream_handle(pkg.STREAM_SCATTERING_1))
    launches = ctx.launch_count() - launches0
    kms, kn = ctx.kernel_timing(False)
    nprob, tiles = b.size()
    b.close()
    units = sum(N * M for (N, M, *_r) in probs)
    flops = sum(2.0 * N * M * M for (N, M, *_r) in probs)
    nsteps = replays * per_graph
    return {"value": units * nsteps / t / 1e9, "ms_per_step": t / nsteps * 1e3, "problems": nprob, "tiles": tiles,
            "tflops_alg": flops * nsteps / t / 1e12, "graph_steps": per_graph, "gpu_launches": launches,
            "max_rel_err": max(e[0] for e in errs), "mean_rel_err": float(np.mean([e[1] for e in errs])),
            "precision": precision,
            "autotuned": {str(k): {x: v[x] for x in ("flush", "bn", "order", "ms")} for k, v in tuned.items()},
            "workload": "64 problems, N log-uniform [5k,200k], M in {146,302,590}, Thomson or HG g~U[0,0.8], "
                        "lambda~U[0.2,0.95], seed 3; one grouped launch per step, CUDA-graph replay"}


def config5_requests(rate, duration, seed, max_requests=4000):
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    while len(reqs) < max_requests:
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        if rate > 0 and t > duration:
            break
        N = int(np.clip(round(math.exp(rng.normal(math.log(50000), 1.0))), 2000, 500000))
        M = int(rng.choice([110, 302, 590, 1202]))
        g = float(rng.uniform(0.0, 0.8))
        iters = int(rng.integers(5, 41))
        reqs.append((t if rate > 0 else 0.0, N, M, g, iters))
    return reqs


def fifo_latencies(arrivals, service):
    """Latencies of requests served one at a time in arrival order, each for
    its service time (seconds)."""
    t, out = 0.0, []
    for a, s in zip(arrivals, service):
        t = max(t, a) + s
        out.append(t - a)
    return np.array(out)


def shared_latencies(arrivals, service, policy):
    """Latencies of requests on one server that runs at the isolated rate of
    whatever it serves, with preemption for free: "ps" shares it equally
    among the requests present (processor sharing), "srpt" gives it to the
    request with the least remaining service.  Idealised reference points
    for the measured p99 (seconds in, seconds out)."""
    order = np.argsort(arrivals, kind="stable")
    arr = np.asarray(arrivals, float)[order]
    rem = {}
    out = np.zeros(len(arr))
    t, i = 0.0, 0
    while i < len(arr) or rem:
        nxt = arr[i] if i < len(arr) else np.inf
        if not rem:
            t = nxt
        else:
            if policy == "ps":
                n = len(rem)
                k = min(rem, key=rem.get)
                done_t = t + rem[k] * n
                if done_t <= nxt:
                    dt = done_t - t
                    for j in rem:
                        rem[j] -= dt / n
                    t = done_t
                    del rem[k]
                    out[k] = t - arr[k]
                    continue
                for j in rem:
                    rem[j] -= (nxt - t) / n
                t = nxt
            else:
                k = min(rem, key=lambda j: (rem[j], j))
                if t + rem[k] <= nxt:
                    t += rem[k]
                    del rem[k]
                    out[k] = t - arr[k]
                    continue
                rem[k] -= nxt - t
                t = nxt
        while i < len(arr) and arr[i] <= t:
            rem[i] = float(np.asarray(service, float)[order][i])
            i += 1
    res = np.empty(len(arr))
    res[order] = out
    return res


def config5(pkg, native, ctx, torch, loads=(0.1, 0.5, 0.8, 1.0, 1.2), window_s=2.0, precision="fp16x3",
            policy=1, budget=0):
    cap = 120 * 10**9
    ctx.set_tuning(native.TUNE_SERVE_POLICY, policy)
    ctx.set_tuning(native.TUNE_SERVE_BUDGET, budget)
    # host input pool (pinned), generated on the device
    pool_n = 500000 * 1202
    pool = native.PinnedBuffer(pool_n * 4 + 500000 * 4)
    ibar_pool = pool.array(np.float32, pool_n)
    b_pool = pool.array(np.float32, 500000, offset_bytes=pool_n * 4)
    ctx.synth_host_f32(5, 1, True, 0.0, 1.0, pool_n, out=ibar_pool)
    ctx.synth_host_f32(5, 2, False, 0.1, 1.0, 500000, out=b_pool)
    lam = np.array([0.5])
    lam_p = lam.ctypes.data_as(native._dp)
    fp = C.POINTER(C.c_float)

    def build(specs):
        rng = np.random.default_rng(77)
        out = []
        for (t, N, M, g, iters) in specs:
            off = int(rng.integers(0, pool_n - N * M + 1))
            out.append(native.Request(t, native.problem_desc(N, M, 1, 1, g, precision), iters,
                                      ibar_pool[off:].ctypes.data_as(fp), b_pool.ctypes.data_as(fp), lam_p, None))
        return out

    # saturation: a backlog of requests all present at t = 0
    sat_specs = config5_requests(0.0, 0.0, seed=5, max_requests=96)
    st, _ = native.serve(ctx, build(sat_specs), cap)
    sat = st.throughput
    # mean work of the request distribution, from a large sample of it (the
    # heavy-tailed sizes make a small sample's mean unreliable)
    pop = config5_requests(0.0, 0.0, seed=999, max_requests=4000)
    mean_work = np.mean([N * M * it for (_, N, M, _, it) in pop])
    results = {"saturation_cell_dir_iter_per_s": sat, "saturation_requests": len(sat_specs),
               "policy": {0: "all resident", 1: "earliest deadline first within a tile budget",
                          2: "least remaining work first within a tile budget",
                          3: "first come first served within a tile budget"}[policy],
               "tile_budget": budget or "8 waves",
               "loads": []}
    for f in loads:
        rate = f * sat / mean_work
        specs = config5_requests(rate, window_s, seed=int(100 * f) + 7)
        # rescale the Poisson arrival times so that the offered work is
        # exactly f of the saturated throughput over the arrival span
        work = sum(N * M * it for (_, N, M, _, it) in specs)
        span = work / (f * sat)
        t_last = specs[-1][0] if specs and specs[-1][0] > 0 else 1.0
        specs = [(t * span / t_last, N, M, g, it) for (t, N, M, g, it) in specs]
        offered = work / span / sat
        reqs = build(specs)
        st, lat = native.serve(ctx, reqs, cap)
        ok = lat[lat >= 0]
        row = {"load": f, "offered_load": offered, "rate_per_s": rate, "requests": len(reqs), "completed": st.completed,
               "rejected": st.rejected, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms,
               "throughput_cell_dir_iter_per_s": st.throughput, "max_active": st.max_active,
               "makespan_s": st.makespan_s, "host_admit_s": st.admit_s, "device_step_s": st.step_s,
               "host_retire_s": st.retire_s, "steps": st.steps,
               "peak_gb": st.peak_bytes / 1e9}
        if abs(f - 0.8) < 1e-9:
            # isolated solve time of every request of this run, alone on the
            # device, one whole step per launch
            ctx.set_tuning(native.TUNE_SERVE_POLICY, 0)
            iso = []
            for r in reqs:
                s1, l1 = native.serve(ctx, [native.Request(0.0, r.desc, r.iterations, r.ibar, r.B, r.lambda_, None)],
                                      cap)
                iso.append(l1[0])
            ctx.set_tuning(native.TUNE_SERVE_POLICY, policy)
            iso = np.array(iso)
            ratio = ok / iso[: len(ok)] if len(ok) == len(iso) else lat / iso
            row["isolated_p50_ms"] = float(np.percentile(iso, 50))
            row["isolated_p99_ms"] = float(np.percentile(iso, 99))
            row["p99_latency_over_isolated"] = float(np.percentile(ratio, 99))
            row["p99_vs_isolated_p99"] = st.p99_ms / float(np.percentile(iso, 99))
            # the same arrivals through one server that runs each request alone
            # for its isolated time, first come first served: what queueing
            # alone costs at this load when requests gain nothing from sharing
            # the device (a reference point for the measured p99)
            arrivals = [r.arrival_s for r in reqs]
            fifo = fifo_latencies(arrivals, iso / 1e3) * 1e3
            row["fifo_alone_p99_ms"] = float(np.percentile(fifo, 99))
            row["fifo_alone_p99_vs_isolated_p99"] = row["fifo_alone_p99_ms"] / float(np.percentile(iso, 99))
            # ... and with free preemption: processor sharing and shortest
            # remaining service first, at the isolated rates
            for pol in ("ps", "srpt"):
                lat_p = shared_latencies(arrivals, iso / 1e3, pol) * 1e3
                row[f"{pol}_alone_p99_ms"] = float(np.percentile(lat_p, 99))
                row[f"{pol}_alone_p99_vs_isolated_p99"] = row[f"{pol}_alone_p99_ms"] / float(np.percentile(iso, 99))
        results["loads"].append(row)
    pool.close()
    ctx.set_tuning(native.TUNE_SERVE_POLICY, 1)
    return results


def config1(pkg, native, ctx, torch, steps, warmup):
    N, M, lam = 10368, 200, 0.5
    xyz, area, fa = native.synth_directions(M)
    B = native.synth_uniform(0, 2, 0.1, 1.0, N)
    ctx.init(xyz, area, fa, N)
    ctx.synth_illum(0, 0.0, 1.0)
    ctx.solve_setup("fp64", B, lam)
    for _ in range(warmup):
        ctx.solve_step_async(False)
    ctx.kernel_timing(True)
    t = timed_steps(ctx, lambda: ctx.solve_step_async(False), steps, torch, ctx.stream_handle(pkg.STREAM_SCATTERING_1))
    kms, kn = ctx.kernel_timing(False)
    return {"value": N * M * steps / t / 1e9, "ms_per_step": t / steps * 1e3, "kernel_ms": kms / max(kn, 1),
            "tflops_fp64": 2.0 * N * M * M / (kms / max(kn, 1) / 1e3) / 1e12, "precision": "fp64",
            "workload": "10,368 cells x 200 Fibonacci directions, Thomson, lognormal(0,1) seed 0, B~U(0.1,1), "
                        "lambda=0.5, one evaluation + update"}
