#!/usr/bin/env python3
"""Headline benchmark: electron-steps/s of the served FP32-compensated engine on
the diode-request mix (Poisson arrivals at 20/s, per-request diodes drawn from
the 128-diode batch distributions), against the plain FP64 one-diode-at-a-time
GPU form and the CPU restatement of the reference path.

A step is one serving iteration: admission of arrived requests, one time step
(emission, Beeman update, all-pair forces, velocities, absorption/compaction)
of every resident diode as one CUDA graph, per-diode counters back to the host
and retirement of completed simulations.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NM = 1e-9
METRIC = "electron-steps/s"
SEED = 20261203
WORKLOAD = ("serve: Poisson 20/s requests, each a planar diode with peak electrons log-U[256, 32768], "
            "V U[0.5, 5] kV, gap U[200, 2000] nm, work function U[2.5, 5.5] eV, emitter side "
            "U[100, 2000] nm, dt 0.25 fs, 1 image term, steps log-U[500, 20000]; pre-filled to peak N, "
            "MH 200 jumps, chains capped at capacity")


# ---------------------------------------------------------------------------------
# request stream: Poisson(20/s) arrivals; each request a planar diode with
# peak electrons log-U[256, 32768], V U[0.5, 5] kV, gap U[200, 2000] nm,
# work function U[2.5, 5.5] eV, square emitter side U[100, 2000] nm (centred),
# dt = 0.25 fs, one image-charge partner, steps log-U[500, 20000], own seed.
# Each is pre-filled with its peak electron count (x, y uniform over the
# emitter footprint, z uniform in [1 nm, gap - 1 nm]).
class RequestStream:
    def __init__(self, seed=SEED, rate=20.0, horizon=300.0, rank=0):
        self.rng = np.random.default_rng([seed, rank])
        self.rate, self.horizon = rate, horizon
        self.t = 0.0
        self.k = 0

    def next(self):
        self.t += self.rng.exponential(1.0 / self.rate)
        if self.t > self.horizon:
            return None
        r = self.rng
        cap = int(round(math.exp(r.uniform(math.log(256), math.log(32768)))))
        req = dict(arrival=self.t, index=self.k, capacity=cap,
                   V_s=float(r.uniform(500.0, 5000.0)), gap=float(r.uniform(200.0, 2000.0)) * NM,
                   phi=float(r.uniform(2.5, 5.5)), side=float(r.uniform(100.0, 2000.0)) * NM,
                   steps=int(round(math.exp(r.uniform(math.log(500), math.log(20000))))),
                   seed=int(r.integers(1, 2 ** 62)))
        self.k += 1
        return req


# Supply quadrature points of the largest emitter of the stream (2000 nm side: 100
# panels of 4 x 4 Gauss-Legendre nodes per side, nodes 5 nm apart), the per-diode
# bound for the quadrature tables of the serving engines.
MAX_SUPPLY_POINTS = 400 * 400


def diode_kwargs(req, max_chains=0):
    s = req["side"]
    return dict(V_s=req["V_s"], gap=req["gap"], time_step=0.25e-15, image_charge=True, N_ic_max=0,
                capacity=req["capacity"], emitter_pos=(-s / 2, -s / 2), emitter_dim=(s, s),
                work=[[req["phi"]]], emission=True, max_chains=max_chains, seed=req["seed"])


def prefill(req):
    rng = np.random.default_rng(req["seed"] % (2 ** 32))
    n, s, d = req["capacity"], req["side"], req["gap"]
    return np.column_stack([rng.uniform(-s / 2, s / 2, n), rng.uniform(-s / 2, s / 2, n),
                            rng.uniform(1 * NM, d - 1 * NM, n)])


# ---------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "rumdeed_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measure_fp32_peak():
    """FP32 FMA throughput of this GPU: cuBLAS SGEMM with TF32 disabled."""
    try:
        import torch
        torch.backends.cuda.matmul.allow_tf32 = False
        torch.set_float32_matmul_precision("highest")
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        for _ in range(2):
            a @ b
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(); a @ b; e1.record(); e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        return 2.0 * n ** 3 / best / 1e12
    except Exception as exc:  # torch missing: nominal figure
        print("fp32 peak probe failed: %s" % exc, file=sys.stderr)
        return None


class L2Flush:
    """Writes a 256 MB buffer (twice the 129 MB L2) between timed iterations."""

    def __init__(self):
        self.buf = None
        try:
            import torch
            self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        except Exception:
            pass

    def __call__(self):
        if self.buf is not None:
            self.buf.zero_()
            import torch
            torch.cuda.synchronize()


# ---------------------------------------------------------------------------------
def capacity_strata(reqs):
    """The requests by capacity octave (256-512, ..., 16384-32768): {octave: [requests]}."""
    out = {}
    for r in reqs:
        out.setdefault(min(6, int(math.log2(r["capacity"] / 256.0))), []).append(r)
    return out


def cpu_step_seconds(orc, r, steps, jumps=(1, 2)):
    """Seconds of one full time step of request r (pre-filled) in the oracle's
    OpenMP restatement: supply integral, MH chains, Beeman update with the
    all-pair forces, removal (the diode is full, so the emission test adds
    nothing).  The MH chains are timed at two short jump counts and
    extrapolated linearly to the step's 200 jumps (a step's MH cost is a start
    pass plus a fixed cost per jump), so that even the largest diodes take
    seconds.  Returns (seconds, electrons in flight)."""
    o = orc.OracleDiode(cap=r["capacity"], V_s=r["V_s"], d=r["gap"], time_step=0.25e-15,
                        image_charge=True, N_ic_max=0)
    s = r["side"]
    o.set_planar_emitter(-s / 2, -s / 2, s, s, [[r["phi"]]])
    o.set_emission(True, seed=r["seed"], mh_jumps=jumps[0], max_chains=r["capacity"])
    o.add_many(prefill(r), step=0)
    t0 = time.perf_counter()
    n_sup = o.supply()
    t_sup = time.perf_counter() - t0
    M = int(min(max(math.floor(n_sup + 0.5), 0), r["capacity"]))
    mh = []
    for j in jumps:
        o.s.mh_jumps = j
        t0 = time.perf_counter()
        o.mh_batch(1, M)
        mh.append(time.perf_counter() - t0)
    per_jump = max(0.0, (mh[1] - mh[0]) / (jumps[1] - jumps[0]))
    start = max(0.0, mh[0] - jumps[0] * per_jump)
    n = o.n
    t0 = time.perf_counter()
    o.verlet(1)
    o.remove(1)
    t_upd = time.perf_counter() - t0
    return t_sup + start + 200 * per_jump + t_upd, n


def cpu_sample(reqs_resident, rank=0):
    """The CPU restatement of the reference path (oracle, OpenMP, all host
    threads) on a capacity-stratified sample of the served window's resident
    set: per capacity octave, the resident request nearest the octave's median
    capacity runs one full time step (cpu_step_seconds), and the octave's
    electron-steps are charged at that request's per-electron time.  So the
    sample's per-electron cost follows the resident set's capacity mix.
    Returns (electron-steps/s, sample description, cores, seconds measured)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    orc.build()
    strata = capacity_strata(reqs_resident)
    tot_e, tot_t, t_meas, picked = 0.0, 0.0, 0.0, []
    for k in sorted(strata):
        group = sorted(strata[k], key=lambda q: q["capacity"])
        rep = group[len(group) // 2]
        w0 = time.perf_counter()
        secs, n = cpu_step_seconds(orc, rep, 1)
        t_meas += time.perf_counter() - w0
        per_e = secs / max(n, 1)
        e_group = sum(q["capacity"] for q in group)   # pre-filled to capacity
        tot_e += e_group
        tot_t += per_e * e_group
        picked.append((rep["capacity"], len(group)))
    cores = orc.lib().orc_omp_threads()
    desc = ("capacity-stratified sample of the %d resident requests of the served window: per capacity "
            "octave one request (capacity, requests in the octave) %s runs one full step with the "
            "oracle's OpenMP C restatement, MH timed at 1 and 2 jumps and extrapolated to 200; the "
            "octave's electron-steps are charged at its per-electron time" % (len(reqs_resident), picked))
    return (tot_e / tot_t if tot_t > 0 else 0.0), desc, cores, t_meas


def plain_fp64_all(rg, requests, budget_s=600.0):
    """The plain FP64 GPU form, one diode at a time (own engine per diode), on
    every resident request of the served window: one untimed step (graph
    capture), the chunking tuner for systems below 4096 electrons (a lone small
    system needs short chunks to fill 152 SMs; larger ones fill it at the
    default chunking), then one step timed with CUDA events (rd_run).  The
    requests are visited in a capacity-interleaved order, so that a budget cut
    leaves a sample spread over the capacities.  Returns (electron-steps/s,
    capacities covered, requests in all)."""
    order = sorted(requests, key=lambda q: q["capacity"])
    n = len(order)
    bits = max(1, (n - 1).bit_length())
    idx = sorted(range(1 << bits), key=lambda k: int(format(k, "0%db" % bits)[::-1], 2))
    order = [order[k] for k in idx if k < n]
    e_steps, dev_s, caps = 0, 0.0, []
    t_start = time.perf_counter()
    for r in order:
        if time.perf_counter() - t_start > budget_s:
            break
        kw = diode_kwargs(r)
        eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=1, particle_capacity=r["capacity"] + 64,
                        chain_capacity=r["capacity"] + 64, quad_capacity=rg.supply_points(**kw) + 64)
        d = eng.add_diode(**kw)
        d.add_particles(prefill(r), step=0)
        eng.run(1, 1)
        if r["capacity"] < 4096:
            eng.autotune()
        n0 = d.counters()["electron_steps"]
        eng.run(2, 1)
        ms, _ = eng.last_run_stats()
        e_steps += d.counters()["electron_steps"] - n0
        dev_s += ms / 1e3
        caps.append(r["capacity"])
        eng.close()
    return (e_steps / dev_s if dev_s > 0 else 0.0), caps, n


# ---------------------------------------------------------------------------------
def reduce_ranks(world, maxes, sums):
    """Max over ranks of the times, sum over ranks of the work counts."""
    if world <= 1:
        return list(maxes) + list(sums)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    mx = torch.tensor(maxes, dtype=torch.float64, device=dev)
    sm = torch.tensor(sums, dtype=torch.float64, device=dev)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return [float(x) for x in mx] + [float(x) for x in sm]


# DRAM bytes (read + write) of one planar MH jump, both halves of the plan, on the 128
# resident requests of the stream: the mean of jumps 2 and 3 of a one-pass ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum), profiles/k_mh_jump_planar_serve128.md.
MH_JUMP_DRAM_BYTES = 35.05e6


# Serving-iteration time of the 128-slot mix, used only to pace the stream's
# arrivals in the admission schedule below.
STEP_S_EST = 0.245
# The timed window starts at least this many serving iterations (~100 s) into the stream.
WINDOW_AFTER = 400


def fifo_schedule(reqs, S, step_s=STEP_S_EST):
    """Admission and completion iteration of each request of the stream when S
    slots serve it first come first served (rd_serve's order): a request is
    admitted at the first iteration when a slot is free and it has arrived,
    runs its steps, and frees its slot for the iteration after its last one.
    Returns [(admit, done)] with done = admit + steps."""
    import heapq
    free = [0] * S
    out = []
    for r in reqs:
        a = max(heapq.heappop(free), int(math.ceil(r["arrival"] / step_s)))
        heapq.heappush(free, a + r["steps"])
        out.append((a, a + r["steps"]))
    return out


def steady_window(reqs, S, lead):
    """A timed window of the saturated server that holds continuous batching:
    the first iteration T0 >= WINDOW_AFTER at which a resident request runs its
    last step (so it retires at the end of timed iteration 1 and the queue head
    is admitted at iteration 2).  Returns T0, the residents at T0 - lead as
    (request, remaining steps from T0 - lead on) in admission order, and the
    queue at that point (arrived, not admitted) in FIFO order."""
    sched = fifo_schedule(reqs, S)
    T0 = min(done - 1 for a, done in sched if done - 1 >= WINDOW_AFTER)
    ts = T0 - lead
    res = sorted([(a, r, done - ts) for r, (a, done) in zip(reqs, sched) if a <= ts < done], key=lambda x: x[0])
    queue = [r for r, (a, done) in zip(reqs, sched) if a > ts and r["arrival"] <= ts * STEP_S_EST]
    return T0, [(r, rem) for a, r, rem in res], queue


def run_ours(args, rank, world):
    import rumdeed_gb300 as rg
    rg.build()
    S = args.slots
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=S, particle_capacity=S * 32768 + 4096,
                    chain_capacity=S * 32768 + 4096, quad_capacity=S * MAX_SUPPLY_POINTS + 4096)
    stream = RequestStream(SEED, rank=rank)
    reqs = []
    while True:
        r = stream.next()
        if r is None:
            break
        reqs.append(r)
    # The saturated server's state at the window: the S resident requests with the steps
    # they still have to run, and the queue behind them (stream order).  The untimed
    # iterations before the window (warm-up, and one after the autotuner) are counted in.
    lead = args.warmup + 1
    T0, residents, queue = steady_window(reqs, S, lead)
    queue_pre, queue_later = queue[:2 * S], queue[2 * S:]
    submitted = {}

    def submit(r, steps):
        pos = prefill(r)
        rid = eng.submit(steps, pos=pos, **diode_kwargs(r))
        submitted[rid] = r
        return pos.nbytes

    for r, rem in residents:
        submit(r, rem)
    for r in queue_pre:
        submit(r, r["steps"])
    flush = L2Flush()
    for _ in range(args.warmup):
        eng.serve(1)
    # the autotuner picks the pair-sum chunking and the MH launch shape for the resident
    # mix; one more untimed iteration rebuilds the step graph under them
    tune = eng.autotune()
    eng.serve(1)
    # timed region: continuous batching on the saturated server.  The stream's later
    # requests keep arriving (submitted at their arrival rate, behind the queue);
    # residents retire and the queue head is admitted inside the window.
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clocks.start()
    dev_ms, wall_s, e_steps, h2d, d2h, admitted, retired = 0.0, 0.0, 0, 0, 0, 0, 0
    step_ms = []
    later = iter(queue_later)
    nxt = next(later, None)
    t_base = nxt["arrival"] if nxt is not None else 0.0
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush()
        w0 = time.perf_counter()
        now = t_base + (w0 - t0)
        while nxt is not None and nxt["arrival"] <= now:
            h2d += submit(nxt, nxt["steps"])
            nxt = next(later, None)
        st = eng.serve(1)
        wall_s += time.perf_counter() - w0
        dev_ms += st["device_ms"]
        step_ms.append(st["device_ms"])
        e_steps += st["electron_steps"]
        h2d += st["h2d_bytes"]
        d2h += st["d2h_bytes"]
        admitted += st["admitted"]
        retired += st["retired"]
    clk = clocks.stop()
    running = st["running"]
    queued = st["queued"]
    _, kps = eng.last_run_stats()
    # queueing delay of the requests admitted in the window (submitted before it)
    qd = []
    for rid in list(submitted):
        s = eng.poll(rid)
        if s["admit_s"] >= 0:
            qd.append(s["admit_s"] - s["submit_s"])
    resident_ids = [rid for rid in submitted if eng.poll(rid)["state"] == rg.REQ_RUNNING]
    resident = [submitted[rid] for rid in resident_ids]
    capped = sum(eng.poll(rid)["counters"]["chains_capped"] for rid in resident_ids)
    chains = sum(eng.poll(rid)["counters"]["chains"] for rid in resident_ids)
    # per-phase profile of one more step (dominant kernel: MH jump launches)
    prof = eng.profile_step(10 ** 6)

    # End to end through the public API (rd_submit / rd_serve, host buffers): every
    # request is cancelled, then the window's state -- the residents with the steps
    # they had left when it began, and the queue behind them -- is submitted again at
    # once from host memory, as new simulations.  The wall clock covers the
    # submissions, their admission (host -> device uploads through the engine's
    # pinned stage) and K serving iterations, each reading the per-diode counters
    # back to the host, with the same retirement and admission as the window.
    for rid in list(submitted):
        if eng.poll(rid)["state"] in (rg.REQ_QUEUED, rg.REQ_RUNNING):
            eng.cancel(rid)
    _, res_t0, queue_t0 = steady_window(reqs, S, 0)
    burst = [(r, rem, prefill(r)) for r, rem in res_t0] + [(r, r["steps"], prefill(r)) for r in queue_t0[:2 * S]]
    e2e_steps, e2e_h2d, e2e_d2h, e2e_adm, e2e_ret = 0, 0, 0, 0, 0
    w0 = time.perf_counter()
    for r, steps, pos in burst:
        eng.submit(steps, pos=pos, **diode_kwargs(r))
    for k in range(args.steps):
        st = eng.serve(1)
        e2e_steps += st["electron_steps"]
        e2e_h2d += st["h2d_bytes"]
        e2e_d2h += st["d2h_bytes"]
        e2e_adm += st["admitted"]
        e2e_ret += st["retired"]
    e2e_wall = time.perf_counter() - w0
    eng.close()

    tot_dev = dev_ms / 1e3
    tot_dev, wall_s, e2e_wall, e_all, e2e_all = reduce_ranks(
        world, [tot_dev, wall_s, e2e_wall], [float(e_steps), float(e2e_steps)])
    value = e_all / tot_dev if tot_dev > 0 else 0.0
    e2e = e2e_all / e2e_wall if e2e_wall > 0 else 0.0
    if rank != 0:
        return
    # dominant kernel roofline (FP32 pipe; 20 flops per Coulomb-like term).  The unit is one
    # MH jump: the mh_parts concurrent launches of k_mh_jump_planar<1> (one per part of the
    # plan, on their own streams), timed together by CUDA events that bracket the fork and
    # the join.
    jumps = max(prof["mh_jump_launches"], 1)
    avg_ms = prof["mh_jumps_ms"] / jumps
    flops_per_jump = 20.0 * prof["mh_pair_evals"] / jumps
    achieved = flops_per_jump / (avg_ms / 1e3) / 1e12 if avg_ms > 0 else 0.0
    peak = measure_fp32_peak()
    peak_src = "measured: cuBLAS SGEMM 8192^3, TF32 off"
    if peak is None:
        peak = 152 * 128 * 2 * 2.07e9 / 1e12
        peak_src = "nominal: 152 SMs x 128 lanes x 2 x 2.07 GHz"
    # the ncu figure was taken on the 128-slot resident set; other mixes report none
    traffic = MH_JUMP_DRAM_BYTES if args.slots == 128 else None
    plain_v, plain_caps, plain_n = plain_fp64_all(rg, resident, budget_s=args.plain_budget)
    cpu_v, cpu_desc, cores, cpu_t = cpu_sample(resident, rank=rank)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair sums (compensated) + f64 integration/FN",
        "data": "synthetic request stream (seeded PCG64; no dataset involved)",
        "config": {"workload": WORKLOAD,
                   "slots": S, "precision": "fp32c", "parallelism": "replicas" if world > 1 else "1 GPU",
                   "chunking": {"chunk_min": tune["chunk_min"], "chunk_count_max": tune["chunk_count_max"],
                                "mh_parts": tune["mh_parts"], "mh_form": tune["mh_form"],
                                "candidates": tune["candidates"],
                                "tuned_ms": tune["ms_chosen"], "default_ms": tune["ms_default"],
                                "fixed": "i-tile 128 (particles, points or chains per work item); force: 64 threads "
                                         "x 2 particles (one image partner), 128 x 1 otherwise"},
                   "l2": "256 MB buffer written between timed iterations",
                   "window": "the saturated server %d serving iterations into the stream (first-come-first-"
                             "served slot schedule of the stream): the %d resident requests with the steps they "
                             "have left, the queue behind them, later requests arriving at the stream's rate; "
                             "a resident retires at the end of the first timed iteration" % (T0, S),
                   "resident_diodes": running, "queued_requests": queued,
                   "admitted_in_timed": admitted, "retired_in_timed": retired,
                   "chains_in_last_step": chains, "chains_capped_in_last_step": capped},
        "latency": {"step_ms_p50": float(np.percentile(step_ms, 50)),
                    "step_ms_p99": float(np.percentile(step_ms, 99)),
                    "step_ms_max": float(max(step_ms)),
                    "queueing_delay_s_p50": float(np.percentile(qd, 50)) if qd else None,
                    "queueing_delay_s_p99": float(np.percentile(qd, 99)) if qd else None,
                    "simulation_latency": "a simulation lasts minutes (500-20000 steps at ~0.25 s): "
                                          "measured with step counts / 100 by --case serve-latency"},
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": e2e_h2d / max(args.steps, 1),
                "d2h_bytes_per_step": e2e_d2h / max(args.steps, 1),
                "window": "the window's state (%d resident requests with the steps they had left, %d queued) "
                          "submitted again from host memory at once, admitted (uploads through the pinned "
                          "stage) and served %d iterations with counter read-back, %d admitted and %d retired "
                          "after the first; wall clock; no L2 flush"
                          % (len(res_t0), len(burst) - len(res_t0), args.steps, e2e_adm - len(res_t0), e2e_ret),
                "steady_state": {"value": e_all / wall_s if wall_s > 0 else 0.0,
                                 "h2d_bytes_per_step": h2d / max(args.steps, 1),
                                 "d2h_bytes_per_step": d2h / max(args.steps, 1),
                                 "window": "the timed serving iterations, wall clock"}},
        "plain_fp64_one_diode_at_a_time": {"value": plain_v, "unit": METRIC,
                                           "covered": "%d of the %d resident requests" % (len(plain_caps), plain_n),
                                           "served_over_plain": value / plain_v if plain_v else None},
        "gpu_launches": 2 * args.steps * (kps + 1) + 3 * (admitted + len(burst)),
        "roofline": {"bound": "fp32", "kernel": "k_mh_jump_planar<1>",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "peak_source": peak_src,
                     "unit_of_work": "one MH jump of every chain: the %d concurrent launches "
                                     "(parts of the plan) of k_mh_jump_planar<1>" % tune["mh_parts"],
                     "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                        "launches of a jump on the burst case (the same 128 resident "
                                        "requests)" if traffic else "not captured for this mix"),
                     "flops_convention": "20 flops per Coulomb-like term (Nyland et al.); "
                                         "1 term per (chain, particle) at the cathode"},
        "phase_ms": {k: prof[k] for k in ("supply_ms", "mh_init_ms", "mh_jumps_ms", "emit_ms",
                                          "position_ms", "force_ms", "velocity_ms", "compact_ms",
                                          "total_ms")},
        "supply_TFLOPs": (20.0 * prof["supply_pair_evals"] / (prof["supply_ms"] / 1e3) / 1e12
                          if prof["supply_ms"] > 0 else None),
        "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": cpu_desc, "seconds": cpu_t},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    """The CPU restatement of the reference path (the Fortran reference cannot be
    built here) on the served window's resident set, capacity-stratified
    (cpu_sample): W + K repetitions, the median reported."""
    if rank != 0:
        return
    reqs = []
    st = RequestStream(SEED)
    while True:
        r = st.next()
        if r is None:
            break
        reqs.append(r)
    _, residents, _ = steady_window(reqs, args.slots, 0)
    resident = [r for r, rem in residents]
    vals, t_all = [], 0.0
    desc, cores = "", 0
    for k in range(args.warmup + args.steps):
        v, desc, cores, t = cpu_sample(resident, rank=0)
        if k >= args.warmup:
            vals.append(v)
            t_all += t
    value = statistics.median(vals) if vals else 0.0
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_all / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic request stream (seeded PCG64; no dataset involved)",
            "config": {"workload": WORKLOAD, "slots": args.slots,
                       "window": "the resident set of the served window (see the served line)"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                             "sample": desc + " (the Fortran reference cannot be built here: no "
                                              "Fortran compiler, Cuba 4.2.2 not vendored)"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------
# Secondary workloads (--case).  Each prints JSON lines of its own; none of them
# is the headline line above.

def micro_positions(n, seed):
    """n electrons, x, y uniform in a 1000 x 1000 nm box centred on the
    emitter centre, z uniform in [1, 999] nm (PCG64 seed per size)."""
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                            rng.uniform(1 * NM, 999 * NM, n)])


def cathode_grid(m=64):
    """m x m cell midpoints of the 1000 x 1000 nm cathode at z = 0."""
    c = (np.arange(m) + 0.5) / m * 1000 * NM - 500 * NM
    gx, gy = np.meshgrid(c, c, indexing="ij")
    return np.column_stack([gx.ravel(), gy.ravel(), np.zeros(m * m)])


def rel_err(got, ref):
    """Per-row norm-relative error |got - ref| / |ref|: (max, rms)."""
    e = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return float(e.max()), float(np.sqrt(np.mean(e * e)))


def case_micro(args):
    """Force/field kernel microbench: N uniform electrons (gap 1000 nm, V 2 kV,
    planar image series N_ic_max in {0, 7}, i.e. 1 or 29 image partners), the
    all-pair force of the FP32-compensated form against the FP64 form (max and
    RMS per-particle relative error) and the field at the 64 x 64 cathode
    midpoints.  Pair-interactions/s from device time (CUDA events)."""
    import rumdeed_gb300 as rg
    rg.build()
    peak = measure_fp32_peak()
    sizes = [int(s) for s in args.sizes.split(",")]
    nics = [int(s) for s in args.nics.split(",")]
    grid = cathode_grid(64)
    for N in sizes:
        pos = micro_positions(N, {4096: 1, 65536: 2, 262144: 3}.get(N, 4))
        for nic in nics:
            terms = 1 + 1 + 4 * nic
            pairs = float(N) * (N - 1)
            out = {"case": "micro", "N": N, "N_ic_max": nic, "terms_per_pair": terms}
            res = {}
            for prec, tag in ((rg.PREC_FP32C, "fp32c"), (rg.PREC_FP64, "fp64")):
                if prec == rg.PREC_FP64 and pairs * terms > args.fp64_budget:
                    out["fp64"] = "not run: %.2g pair-terms exceeds --fp64-budget" % (pairs * terms)
                    continue
                eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=N + 1024,
                                chain_capacity=4096, quad_capacity=4096)
                d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=N, image_charge=True, N_ic_max=nic)
                d.add_particles(pos)
                # chunking for this system size (the project's tuner); the FP64 form only where
                # its 45 timing passes stay short
                tune = eng.autotune() if (prec == rg.PREC_FP32C or pairs * terms < 2e9) else \
                    dict(zip(("chunk_min", "chunk_count_max"), eng.get_chunking()))
                acc = d.calculate_acceleration_particles()
                reps = 1 if pairs * terms > 2e11 else (3 if pairs > 1e9 else 20)
                ms = eng.time_accel(reps)
                fld = d.calc_field_at_batch(grid)
                fms = d.time_field_at(grid, reps=max(reps, 3))
                res[tag] = (acc, fld)
                out[tag] = {"force_ms": ms, "force_pairs_per_s": pairs / (ms / 1e3),
                            "force_tflops": 20.0 * terms * pairs / (ms / 1e3) / 1e12,
                            "field_ms": fms, "field_point_particle_per_s": grid.shape[0] * N / (fms / 1e3),
                            "chunking": {"chunk_min": tune["chunk_min"],
                                         "chunk_count_max": tune["chunk_count_max"]}}
                if prec == rg.PREC_FP32C and peak:
                    out[tag]["force_frac_of_measured_fp32"] = out[tag]["force_tflops"] / peak
                eng.close()
            if "fp64" in res:
                out["force_rel_err_max"], out["force_rel_err_rms"] = rel_err(res["fp32c"][0], res["fp64"][0])
                out["field_rel_err_max"], out["field_rel_err_rms"] = rel_err(res["fp32c"][1], res["fp64"][1])
                # the cathode field is the vacuum field minus the space-charge sum; where they
                # nearly cancel, |E| is small and its relative error large: also against |E_vac|
                dv = np.linalg.norm(res["fp32c"][1] - res["fp64"][1], axis=1) / (2.0e3 / (1000 * NM))
                out["field_err_max_over_vacuum"] = float(dv.max())
                out["field_min_over_vacuum"] = float(np.linalg.norm(res["fp64"][1], axis=1).min()
                                                     / (2.0e3 / (1000 * NM)))
            out["fp32_peak_tflops"] = peak
            print(json.dumps(out), flush=True)


def case_serve_latency(args):
    """Per-simulation latency of the serving loop, measured: the serving
    request stream (Poisson 20/s, the same diode distributions) with every
    request's step count divided by --step-scale so that simulations finish
    inside the window, served in real time for --window seconds.  Reports,
    over the requests that completed, the latency from submission to the
    last step (p50 / p99), its queueing part (submission to admission) and
    its service part, with the electron-steps/s of the window.  The full step
    counts (500-20000) make one simulation last minutes, so the headline run
    projects that latency instead."""
    import rumdeed_gb300 as rg
    rg.build()
    S = args.slots
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=S, particle_capacity=S * 32768 + 4096,
                    chain_capacity=S * 32768 + 4096, quad_capacity=S * MAX_SUPPLY_POINTS + 4096)
    stream = RequestStream(SEED)
    pending = stream.next()
    ids = []
    t0 = time.perf_counter()
    e_steps, dev_ms, iters, checks, violations = 0, 0.0, 0, 0, 0
    while time.perf_counter() - t0 < args.window:
        now = time.perf_counter() - t0
        while pending is not None and pending["arrival"] <= now:
            steps = max(1, int(round(pending["steps"] / args.step_scale)))
            ids.append(eng.submit(steps, pos=prefill(pending), **diode_kwargs(pending)))
            pending = stream.next()
        st = eng.serve(1)
        e_steps += st["electron_steps"]
        dev_ms += st["device_ms"]
        iters += 1
        if args.validate_every and iters % args.validate_every == 0:   # rd_validate self check
            violations += sum(eng.validate().values())
            checks += 1
    wall = time.perf_counter() - t0
    lat, queue, service = [], [], []
    states = {}
    for rid in ids:
        s = eng.poll(rid)
        states[s["state"]] = states.get(s["state"], 0) + 1
        if s["state"] == rg.REQ_DONE:
            lat.append(s["done_s"] - s["submit_s"])
            queue.append(s["admit_s"] - s["submit_s"])
            service.append(s["done_s"] - s["admit_s"])
    eng.close()
    pct = lambda v, q: float(np.percentile(v, q)) if v else None
    print(json.dumps({"case": "serve-latency", "window_s": wall, "step_scale": args.step_scale,
                      "submitted": len(ids), "completed": len(lat),
                      "running_or_queued": len(ids) - len(lat),
                      "latency_s_p50": pct(lat, 50), "latency_s_p99": pct(lat, 99),
                      "queueing_s_p50": pct(queue, 50), "queueing_s_p99": pct(queue, 99),
                      "service_s_p50": pct(service, 50), "service_s_p99": pct(service, 99),
                      "iterations": iters, "validate_checks": checks, "violations": violations,
                      "electron_steps_per_s_wall": e_steps / wall,
                      "electron_steps_per_s_device": e_steps / (dev_ms / 1e3) if dev_ms else None}),
          flush=True)


def hbm_peak_gbs():
    """Measured HBM copy bandwidth in GB/s (MEASURED_PEAKS.json), or None."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def case_verlet(args):
    """The HBM-bound per-particle kernels at a size that fills the GPU: 64
    planar diodes of --verlet-n / 64 electrons each (no emission), the Beeman
    position pass (k_position: boundary checks and FP32 packs included) and
    the velocity pass (k_velocity + the Ramo / mean-velocity reduction), timed
    with CUDA events (rd_time_verlet).  Algorithmic bytes per electron:
    position 268 B (reads species, x, v, a, a_prev, q = 108 B; writes x,
    a_prev2, a_prev, the cleared a and the four FP32 packs = 160 B), velocity
    132 B (reads species, v, a, a_prev, a_prev2, q = 108 B; writes v = 24 B;
    the Ramo / mean-velocity sums leave the kernel as 80 B per 128-electron
    item, under 1 B per electron, not counted).  Both kernels keep the state
    in FP64, and on this GPU the FP64 pipe, not HBM, is what they reach
    first."""
    import rumdeed_gb300 as rg
    rg.build()
    D, n = 64, max(1, args.verlet_n // 64)
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=D, particle_capacity=D * (n + 64),
                    chain_capacity=4096, quad_capacity=4096)
    rng = np.random.default_rng(7)
    for k in range(D):
        d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=n, image_charge=True, N_ic_max=0)
        d.add_particles(np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                                         rng.uniform(400 * NM, 600 * NM, n)]), step=0)
    pos_ms, vel_ms = eng.time_verlet(reps=20)
    eng.close()
    N = D * n
    peak = hbm_peak_gbs()
    out = {"case": "verlet", "electrons": N}
    for name, ms, b in (("position", pos_ms, 268), ("velocity", vel_ms, 132)):
        gbs = b * N / (ms / 1e3) / 1e9
        out[name] = {"ms": ms, "bytes_per_electron": b, "achieved_gbs": gbs,
                     "frac_of_measured_hbm": gbs / peak if peak else None}
    out["hbm_peak_gbs"] = peak
    print(json.dumps(out), flush=True)


def case_uncapped(args):
    """The chain cap.  The served engine runs at most `capacity` MH chains per
    diode and step (a step cannot add more electrons than the diode holds);
    the reference runs a chain for every one of the step's N_round candidates
    and lets Add_Particle drop what does not fit (src/mod_field_emission_v2.F90:
    283-330, src/mod_pair.F90:37-44).  The headline window's resident set runs
    W + K steps both ways: capped, then with each diode's chain bound raised to
    twice the N_round of its first capped step (chains_capped then counts what
    is still cut).  Reports emitted and dropped electrons, chains and
    electron-steps/s of both."""
    import rumdeed_gb300 as rg
    rg.build()
    reqs = []
    st = RequestStream(SEED)
    while True:
        r = st.next()
        if r is None:
            break
        reqs.append(r)
    _, residents, _ = steady_window(reqs, args.slots, 0)
    res = [r for r, rem in residents]

    def run(bounds):
        chcap = sum(bounds) + 4096
        eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=len(res), particle_capacity=len(res) * 32768 + 4096,
                        chain_capacity=chcap, quad_capacity=len(res) * MAX_SUPPLY_POINTS + 4096)
        ds = []
        for r, b in zip(res, bounds):
            d = eng.add_diode(**diode_kwargs(r, max_chains=b))
            d.add_particles(prefill(r), step=0)
            ds.append(d)
        eng.run(1, 1)
        first = [d.counters() for d in ds]
        c0 = [d.counters() for d in ds]
        eng.run(2, args.warmup + args.steps - 1)
        ms, _ = eng.last_run_stats()
        c1 = [d.counters() for d in ds]
        eng.close()
        steps = args.warmup + args.steps - 1
        return {"electron_steps_per_s": sum(b["electron_steps"] - a["electron_steps"] for a, b in zip(c0, c1))
                / (ms / 1e3),
                "ms_per_step": ms / steps, "emitted": sum(c["emitted_total"] for c in c1),
                "dropped": sum(c["dropped_total"] for c in c1),
                "chains_last_step": sum(c["chains"] for c in c1),
                "chains_capped_last_step": sum(c["chains_capped"] for c in c1)}, first
    capped, first = run([r["capacity"] for r in res])
    n_round = [c["chains"] + c["chains_capped"] for c in first]
    uncapped, _ = run([max(r["capacity"], 2 * n) for r, n in zip(res, n_round)])
    print(json.dumps({"case": "uncapped", "diodes": len(res), "steps": args.warmup + args.steps,
                      "n_round_first_step": sum(n_round),
                      "diodes_capped_first_step": sum(1 for c in first if c["chains_capped"] > 0),
                      "capped": capped, "uncapped": uncapped}), flush=True)


def case_compact(args):
    """Absorption and compaction at full size: 64 planar diodes of 262144
    electrons (16.8 M).  Two removal patterns: (a) three in four sit just below
    the anode moving up and cross it in the next position pass, the others
    (every fourth, so the survivors are spread over each diode) at mid-gap at
    rest; (b) 1 % of the electrons at random indices cross, the scattered
    removals of the reference's own compaction benchmark (Util/bench_compact.f90,
    1e6 particles with 1e4 removals).  One position pass marks the crossers;
    the removal that follows compacts each diode's survivors stably in place
    (rd_time_remove, CUDA events).  Algorithmic bytes: the survey's 2 x the
    moved survivors' state, 152 B of FP64 and int state per particle read and
    written once; the implementation also writes each moved survivor's 64 B of
    FP32 packs and reads and rewrites the 4 B removal mask of every particle
    behind the first removed one."""
    import rumdeed_gb300 as rg
    rg.build()
    D, n = 64, max(1024, args.verlet_n // 64)

    def fill(eng, D, n, pattern):
        rng = np.random.default_rng(11)
        for k in range(D):
            d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=n, image_charge=True, N_ic_max=0)
            if pattern == "three_in_four":
                keep = (np.arange(n) % 4) == 0
            else:
                keep = np.ones(n, dtype=bool)
                keep[rng.choice(n, n // 100, replace=False)] = False
            z = np.where(keep, 500 * NM, 999.9 * NM)
            vz = np.where(keep, 0.0, 1.0e8)
            d.add_particles(np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n), z]),
                            vel=np.column_stack([np.zeros(n), np.zeros(n), vz]), step=0)

    warm = rg.Engine(precision=rg.PREC_FP32C, max_diodes=2, particle_capacity=2 * 4096 + 64, chain_capacity=64,
                     quad_capacity=64)
    fill(warm, 2, 4096, "three_in_four")
    warm.time_remove()   # loads the kernels
    warm.close()
    peak = hbm_peak_gbs()
    for pattern in ("three_in_four", "scattered_1pct"):
        eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=D, particle_capacity=D * (n + 64), chain_capacity=4096,
                        quad_capacity=4096)
        fill(eng, D, n, pattern)
        pos_ms, rem_ms, moved, removed = eng.time_remove()
        left = sum(d.counters()["n"] for d in eng.diodes.values())
        eng.close()
        alg = 2.0 * moved * 152
        impl = moved * (2 * 152 + 64)
        print(json.dumps({"case": "compact", "pattern": pattern, "diodes": D, "electrons": D * n, "removed": removed,
                          "moved": moved, "survivors": left, "position_ms": pos_ms, "remove_ms": rem_ms,
                          "algorithmic_GBs": alg / (rem_ms / 1e3) / 1e9,
                          "implementation_GBs": impl / (rem_ms / 1e3) / 1e9,
                          "hbm_peak_GBs": peak, "frac_algorithmic": alg / (rem_ms / 1e3) / 1e9 / peak if peak else None,
                          "bytes": {"algorithmic_per_moved": 2 * 152, "implementation_per_moved": 2 * 152 + 64}}),
              flush=True)


def case_burst(args):
    """The first S requests of the serving stream admitted at once (no arrival
    pacing), then W + K serving iterations: the serving workload with a fixed
    resident set and a fixed launch order, for profiler captures."""
    import rumdeed_gb300 as rg
    rg.build()
    S = args.slots
    free0 = None
    try:
        import torch
        free0 = torch.cuda.mem_get_info()[0]
    except Exception:
        pass
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=S, particle_capacity=S * 32768 + 4096,
                    chain_capacity=S * 32768 + 4096, quad_capacity=S * MAX_SUPPLY_POINTS + 4096)
    stream = RequestStream(SEED)
    reqs = [stream.next() for _ in range(S)]
    for r in reqs:
        eng.submit(r["steps"], pos=prefill(r), **diode_kwargs(r))
    ms, es = [], 0
    for k in range(args.warmup + args.steps):
        st = eng.serve(1)
        if k >= args.warmup:
            ms.append(st["device_ms"])
            es += st["electron_steps"]
    used = None
    if free0 is not None:
        import torch
        used = (free0 - torch.cuda.mem_get_info()[0]) / 2 ** 30
    eng.close()
    print(json.dumps({"case": "burst", "slots": S, "steps": args.steps, "warmup": args.warmup,
                      "electron_steps_per_s": es / (sum(ms) / 1e3) if ms else 0.0,
                      "step_ms": ms, "device_gib_used": used}), flush=True)


def case_mh_small(args):
    """Small emission case for full profiler captures: 4 planar diodes of 6000
    electrons (1000 x 1000 nm emitter, 3 kV over 1000 nm, work function 3.5 eV,
    chains capped at 6000), one profiled step."""
    import rumdeed_gb300 as rg
    rg.build()
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=4, particle_capacity=4 * 8192,
                    chain_capacity=4 * 8192, quad_capacity=4 * 65536)
    rng = np.random.default_rng(1)
    n, side = 6000, 1000 * NM
    for k in range(4):
        d = eng.add_diode(V_s=3000.0, gap=1000 * NM, capacity=n, emitter_pos=(-side / 2, -side / 2),
                          emitter_dim=(side, side), work=[[3.5]], emission=True, max_chains=n, seed=10 + k)
        d.add_particles(np.column_stack([rng.uniform(-side / 2, side / 2, n), rng.uniform(-side / 2, side / 2, n),
                                         rng.uniform(1 * NM, 999 * NM, n)]), step=0)
    p = eng.profile_step(1)
    eng.close()
    print(json.dumps({"case": "mh-small", **p}), flush=True)


def case_one_diode(args):
    """One planar diode of the reference's one-diode configuration (1 um gap,
    2 kV, 1000 x 1000 nm emitter, dt 0.25 fs, one image term) at work function
    --phi and --jumps MH jumps per step, in --precision; no CPU leg and no
    tuner (--chunk-min / --chunk-count set the chunking by hand), so that a
    profiler sees only the engine's own launches.  Prints device ms per step
    and the kernels per step."""
    import rumdeed_gb300 as rg
    rg.build()
    side = 1000 * NM
    prec = rg.PREC_FP64 if args.precision == "fp64" else rg.PREC_FP32C
    eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=20064, chain_capacity=20064,
                    quad_capacity=65536)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, image_charge=True, N_ic_max=0,
                      capacity=20000, emitter_pos=(-side / 2, -side / 2), emitter_dim=(side, side),
                      emission=True, seed=SEED, work=[[args.phi]], mh_jumps=args.jumps)
    if args.chunk_min or args.chunk_count:
        eng.set_chunking(args.chunk_min, args.chunk_count)
    if args.uncaptured:
        # every step phase by phase from the host (rd_profile_step): plain stream launches, which a
        # profiler lists one by one (the step graph of a lone diode holds a conditional node)
        for k in range(args.warmup + args.steps):
            p = eng.profile_step(k + 1)
        ms, kps = p["total_ms"] * args.steps, 0
    else:
        eng.run(1, args.warmup)
        eng.run(args.warmup + 1, args.steps)
        ms, kps = eng.last_run_stats()
    c = d.counters()
    eng.close()
    print(json.dumps({"case": "one-diode", "precision": args.precision, "work_function_eV": args.phi,
                      "mh_jumps": args.jumps, "steps": args.steps, "ms_per_step": ms / args.steps,
                      "steps_per_s": args.steps / (ms / 1e3), "kernels_per_step": kps, "in_flight": c["n"],
                      "uncaptured": bool(args.uncaptured)}), flush=True)


def case_plain(args):
    """The plain single-diode deck (CPU-runnable size): gap 1000 nm, 2 kV, a
    1000 x 1000 nm emitter centred on the axis, work function 4.7 eV (and a
    populated 2.0 eV variant), dt 0.25 fs, one image partner, MH with 100 and
    with the reference's 200 jumps, Philox seed 20261203.  Steps/s of the GPU
    engine in FP64 and FP32-compensated form (device time, rd_run) beside the
    CPU restatement (FP64)."""
    import rumdeed_gb300 as rg
    rg.build()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    orc.build()
    side = 1000 * NM
    kw = dict(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, image_charge=True, N_ic_max=0, capacity=20000,
              emitter_pos=(-side / 2, -side / 2), emitter_dim=(side, side), emission=True, seed=SEED)
    for phi in (4.7, 2.0):
        for jumps in (100, 200):
            gpu = {}
            for prec, tag in ((rg.PREC_FP64, "fp64"), (rg.PREC_FP32C, "fp32c")):
                eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=20064,
                                chain_capacity=20064, quad_capacity=65536)
                d = eng.add_diode(work=[[phi]], mh_jumps=jumps, **kw)
                eng.run(1, args.warmup)
                tune = eng.autotune()   # a lone diode needs short chunks to fill the GPU
                eng.run(args.warmup + 1, args.steps)
                ms, kps = eng.last_run_stats()
                c = d.counters()
                eng.close()
                gpu[tag] = {"steps_per_s": args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                            "in_flight": c["n"], "emitted_total": c["emitted_total"], "N_sup": c["N_sup"],
                            "chunking": [tune["chunk_min"], tune["chunk_count_max"]]}
            o = orc.OracleDiode(cap=20000, V_s=2.0e3, d=1000 * NM, time_step=0.25e-15, image_charge=True,
                                N_ic_max=0)
            o.set_planar_emitter(-side / 2, -side / 2, side, side, [[phi]])
            o.set_emission(True, seed=SEED, mh_jumps=jumps, max_chains=20000)   # the default supply rule
            cpu_steps, t0 = 0, time.perf_counter()
            while cpu_steps < 3 and time.perf_counter() - t0 < 20.0:
                o.step(cpu_steps + 1)
                cpu_steps += 1
            cpu_t = time.perf_counter() - t0
            print(json.dumps({"case": "plain", "work_function_eV": phi, "mh_jumps": jumps,
                              "after_steps": args.warmup + args.steps, "kernels_per_step": kps,
                              "gpu": gpu, "cpu_steps_per_s": cpu_steps / cpu_t, "cpu_steps": cpu_steps,
                              "cpu_cores": orc.lib().orc_omp_threads()}), flush=True)


def case_tips(args):
    """16 hyperboloid tips in one engine: apex radius r U[10, 50] nm (base
    radius R = sqrt(r (h^2 + 2 d h) / d)), tip height h 500 nm, tip-anode gap
    d 1000 nm, V U[1, 5] kV, work function 4.5 eV, sphere image charge; each
    tip pre-filled with --tip-electrons electrons (x, y uniform over the base
    square, z uniform from 1 nm above the apex to 1 nm below the anode).
    FP32-compensated; electron-steps/s from device time."""
    import rumdeed_gb300 as rg
    rg.build()
    rng = np.random.default_rng([SEED, 4])
    ntip, n = 16, args.tip_electrons
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=ntip, particle_capacity=ntip * (n + 64),
                    chain_capacity=ntip * (n + 64), quad_capacity=ntip * 10000 + 4096)
    h, dd = 500 * NM, 1000 * NM
    tips = []
    for t in range(ntip):
        r = rng.uniform(10.0, 50.0) * NM
        R = math.sqrt(r * (h * h + 2.0 * dd * h) / dd)
        V = rng.uniform(1.0e3, 5.0e3)
        d = eng.add_diode(geometry=rg.GEOM_TIP, V_s=V, time_step=0.25e-15, image_charge=True, capacity=n,
                          tip_dim=(dd, R, h), tip_work_function=4.5, emission=True, max_chains=n,
                          seed=int(rng.integers(1, 2 ** 62)))
        pos = np.column_stack([rng.uniform(-R, R, n), rng.uniform(-R, R, n),
                               rng.uniform(h + 1 * NM, h + dd - 1 * NM, n)])
        d.add_particles(pos, step=0)
        tips.append((r, R, V))
    eng.run(1, args.warmup)
    e0 = sum(dio.counters()["electron_steps"] for dio in eng.diodes.values())
    eng.run(args.warmup + 1, args.steps)
    ms, kps = eng.last_run_stats()
    e1 = sum(dio.counters()["electron_steps"] for dio in eng.diodes.values())
    prof = eng.profile_step(args.warmup + args.steps + 1)
    cs = [dio.counters() for dio in eng.diodes.values()]
    eng.close()
    print(json.dumps({"case": "tips", "tips": ntip, "electrons_per_tip": n,
                      "electron_steps_per_s": (e1 - e0) / (ms / 1e3), "ms_per_step": ms / args.steps,
                      "kernels_per_step": kps, "phase_ms": prof,
                      "chains": [c["chains"] for c in cs], "emitted_step": [c["emitted_step"] for c in cs],
                      "in_flight": [c["n"] for c in cs]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--slots", type=int, default=128)
    ap.add_argument("--plain-budget", type=float, default=600.0,
                    help="seconds for the plain FP64 one-diode-at-a-time leg over the resident set")
    ap.add_argument("--case", default="serve",
                    choices=["serve", "micro", "burst", "mh-small", "plain", "tips", "serve-latency", "verlet",
                             "one-diode", "uncapped", "compact"],
                    help="serve: the headline serving benchmark; the others are secondary workloads")
    ap.add_argument("--sizes", default="4096,65536,262144", help="micro: electron counts")
    ap.add_argument("--nics", default="0,7,8", help="micro: N_ic_max values (K = 8 mirror terms read "
                    "as N_ic_max = 7, the series through n = 7, or as N_ic_max = 8)")
    ap.add_argument("--tip-electrons", type=int, default=100000, help="tips: electrons per tip")
    ap.add_argument("--step-scale", type=float, default=100.0,
                    help="serve-latency: every request's step count is divided by this")
    ap.add_argument("--window", type=float, default=60.0, help="serve-latency: seconds of real-time serving")
    ap.add_argument("--verlet-n", type=int, default=1 << 24, help="verlet: electrons in all (64 diodes)")
    ap.add_argument("--phi", type=float, default=4.7, help="one-diode: work function (eV)")
    ap.add_argument("--jumps", type=int, default=100, help="one-diode: MH jumps per step")
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"], help="one-diode: engine precision")
    ap.add_argument("--chunk-min", type=int, default=0, help="one-diode: j-chunk length (0: the default)")
    ap.add_argument("--chunk-count", type=int, default=0, help="one-diode: j-chunks per tile at most (0: the default)")
    ap.add_argument("--uncaptured", action="store_true",
                    help="one-diode: run the steps phase by phase (rd_profile_step) instead of the step graph")
    ap.add_argument("--validate-every", type=int, default=0,
                    help="serve-latency: run rd_validate every this many iterations (0: never)")
    ap.add_argument("--fp64-budget", type=float, default=2.0e11,
                    help="micro: largest N(N-1) x terms run in FP64 for the error check")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    if args.case != "serve":
        if rank == 0:
            {"micro": case_micro, "burst": case_burst, "mh-small": case_mh_small, "plain": case_plain,
             "serve-latency": case_serve_latency, "verlet": case_verlet, "one-diode": case_one_diode,
             "tips": case_tips, "uncapped": case_uncapped, "compact": case_compact}[args.case](args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
