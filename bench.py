#!/usr/bin/env python
"""bench.py -- micSA sweep throughput on GB300, in spin-flip attempts per ps.

Workload (one GPU): the plain micSA run at L=160, 2 disorder samples x 64
replicas, nc = 6 demons per site.  One step = one reference iteration
(Monte_Carlo flag=1, PROGRAM/src/main.cu:254-305): 6 x (even, odd)
half-sweeps plus the demon walk, on both samples, i.e.
V * 64 * 2 * 6 = 3.15e9 spin-flip attempts (timing.c:20-23 counts the same).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl micsa|reference]

--gpus N > 1 is launched by torchrun (one process per GPU): every rank runs
its own independent copy of the workload (the path has no exchange step;
replicas only) and the value is the total over ranks divided by the slowest
rank's time.  --impl reference times the CPU restatement of the reference's
algorithm (oracle/) on the host cores, on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "micsa-ea-mc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "spin-flips/ps at L=160"
UNIT = "spin-flip attempts/ps"
SEEDS = dict(seed_J=20260101, seed_u=1729, seed_MC0=0x5EED0000)
BETA = 0.90909090909090


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="micsa", choices=["micsa", "reference"])
    # smaller shapes for profiling captures (the headline is the default)
    ap.add_argument("--L", type=int, default=160)
    ap.add_argument("--nr", type=int, default=64)
    ap.add_argument("--nsamples", type=int, default=None,
                    help="samples (plain, default 2) or jobs (batched, default 512)")
    ap.add_argument("--nc", type=int, default=6)
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "served"],
                    help="plain: the headline run; batched: --nsamples jobs; served: a "
                         "Poisson request stream")
    ap.add_argument("--requests", type=int, default=200, help="served: requests in the trace")
    ap.add_argument("--hbm-gb", type=float, default=48.0, help="served: HBM budget (GiB)")
    ap.add_argument("--iterations", type=int, default=4096,
                    help="batched with --batch-L: iterations per job")
    ap.add_argument("--batch-L", type=int, default=None,
                    help="batched: one lattice size instead of the mixed-L stream")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    a = ap.parse_args()
    if a.nsamples is None:
        a.nsamples = 512 if a.workload == "batched" else 2
    return a


class Dist:
    """torch.distributed plumbing: barrier and max over ranks (nccl on GPUs,
    gloo where there is none)."""

    def __init__(self, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            import torch
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend)
            self.pg = dist
            self.backend = backend

    def barrier(self):
        if self.pg:
            if self.backend == "nccl":
                import torch
                self.pg.barrier(device_ids=[self.local])
            else:
                self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        dev = "cuda:%d" % self.local if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, device):
        self.device, self.proc, self.out = device, None, None

    def start(self):
        try:
            self.out = open(os.devnull, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=self.out, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            text, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            text, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        for line in text.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(self.NAMES, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes_per_attempt(nr):
    # per 64 attempts (one colour site-word x one replica word, one
    # half-sweep): own spin r+w 16 B, other-colour spin 8 B, demon r+w 32 B,
    # couplings 48/nr B (shared by the replicas)
    return (56.0 + 48.0 / nr) / 64.0


def traffic_per_launch(L, nr, ns, kernel="k_sweep"):
    """DRAM bytes of one half-sweep of all samples from the committed ncu
    summaries (profiles/*.md, lines 'traffic_bytes_per_launch[<kernel>] L nr
    ns: N'; no tag = k_sweep), scaled by the sites processed when only a
    smaller capture of that kernel exists."""
    import glob
    import re
    best = None
    for f in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for m in re.finditer(r"traffic_bytes_per_launch(?:\[(\w+)\])? L=(\d+) nr=(\d+) ns=(\d+): (\d+)",
                             open(f).read()):
            if (m.group(1) or "k_sweep") != kernel:
                continue
            cl, cn, cs, b = (int(x) for x in m.groups()[1:])
            if (cl, cn, cs) == (L, nr, ns):
                return float(b), "ncu capture of this shape (%s)" % kernel
            if cn == nr:
                best = (float(b) * (L ** 3 * ns) / (cl ** 3 * cs),
                        "ncu capture of %s at L=%d ns=%d scaled by sites" % (kernel, cl, cs))
    return best if best else (None, None)


def host_samples(L, nr, ns, nc):
    """Seeded reference initialisation of ns samples: one reference run
    (nbits = ns <= MAXNSAMPLES = 2), or, beyond that, one single-sample run
    per sample with its own spin seed; an object with per-sample J, spins,
    demon streams prc_C/xo_C and the thresholds thr."""
    import micsa
    mc = [SEEDS["seed_MC0"] + r for r in range(nr)]
    if ns <= micsa.HostModel.MAXNSAMPLES:
        return micsa.HostModel(L, nr, nc, SEEDS["seed_J"], SEEDS["seed_u"], mc, list(range(ns)),
                               beta=BETA, nthreads=os.cpu_count() or 8)
    runs = [micsa.HostModel(L, nr, nc, SEEDS["seed_J"], SEEDS["seed_u"] + 7919 * b, mc, [0],
                            beta=BETA, nthreads=os.cpu_count() or 8) for b in range(ns)]

    class Samples:
        J = [r.J[0] for r in runs]
        spins = [r.spins[0] for r in runs]
        prc_C = [r.prc_C[0] for r in runs]
        xo_C = [r.xo_C[0] for r in runs]
        thr = runs[0].thr
    return Samples()


def run_micsa(a, dist):
    import torch
    import micsa
    dev = dist.local
    torch.cuda.set_device(dev)
    L, nr, ns, nc = a.L, a.nr, a.nsamples, a.nc
    hm = host_samples(L, nr, ns, nc)
    ctx = micsa.Context(L, nr, ns, nc, device=dev)
    for b in range(ns):
        ctx.upload_couplings(b, hm.J[b])
        ctx.upload_spins(b, *hm.spins[b])
        ctx.refresh_demons(b, hm.prc_C[b], hm.xo_C[b], hm.thr)  # InitWalkers on the GPU
    demons = [ctx.download_demons(b) for b in range(ns)]  # for the upload-every-step variant
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    attempts = float(L ** 3) * nr * ns * nc
    # ---- device-resident throughput: the K steps in one call (graph replays,
    # or multi-iteration launches of the resident kernel at L <= 16)
    ctx.iterate(a.warmup)
    ctx.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    l0 = ctx.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.iterate(a.steps)
    e1.record(stream)
    e1.synchronize()
    ctx.synchronize()
    launches = ctx.kernel_launches() - l0
    torch.cuda.synchronize()
    dist.barrier()
    ck = clocks.stop()
    ms = dist.max(e0.elapsed_time(e1) / a.steps)
    value = attempts * dist.world / (ms * 1e9)
    # ---- dominant kernel: mean half-sweep launch time, CUDA events
    sweep_ms, iter_ms = ctx.profile(max(3, min(10, a.steps)))
    bpa = algorithmic_bytes_per_attempt(nr)
    per_launch = attempts / (2 * nc) * bpa
    achieved = per_launch / (sweep_ms * 1e-3) / 1e9
    peak, kind = peaks()
    traffic, tnote = traffic_per_launch(L, nr, ns, "k_sweep_dep" if "load=flow" in ctx.tuning()
                                        else "k_sweep")
    kernel = ("k_sweep_dep (dataflow sweep: the %d half-sweeps of an iteration in one launch; "
              "time per half-sweep)" % (2 * nc) if "load=flow" in ctx.tuning()
              else "k_sweep (micSA half-sweep)")
    roof = {"bound": "hbm", "kernel": kernel,
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": kind,
            "algorithmic_bytes_per_launch": int(per_launch),
            "launch_ms": round(sweep_ms, 5), "iteration_ms_profiled": round(iter_ms, 5),
            "autotune": ctx.tuning(),
            "traffic": traffic, "traffic_source": tnote}
    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not a.no_e2e:
        e2e = e2e_job(a, dist, ctx, hm, attempts)
        e2e["upload_every_step"] = e2e_upload_every_step(a, dist, ctx, demons, attempts)
    ctx.close()
    return dict(value=value, ms=ms, roof=roof, clocks=ck, e2e=e2e, launches=launches,
                attempts=attempts)


def _pinned(arr):
    import torch
    t = torch.empty(arr.size * arr.itemsize // 8, dtype=torch.int64, pin_memory=True)
    v = t.numpy().view(arr.dtype)
    v[:] = arr
    return t, v


def e2e_job(a, dist, ctx, hm, attempts):
    """The whole job of `steps` iterations through the C ABI, on the
    reference's schedule (main.cu:126-180): start state uploaded from pinned
    host memory, demon refresh and energy readback at t = 0, 1, 2, 4, ...
    (refresh_walkers + Measure_Energy_Spins/Clerics), iterations in between,
    and the final spins and demons read back (the checkpoint of
    copy_from_GPU_for_write).  h2d/d2h are the bytes of those copies per
    iteration."""
    import micsa
    L, nr, ns, nc = a.L, a.nr, a.nsamples, a.nc
    H = (L // 4) ** 3 // 2
    J = [_pinned(hm.J[b]) for b in range(ns)]
    sp = [(_pinned(hm.spins[b][0]), _pinned(hm.spins[b][1])) for b in range(ns)]
    start = [(bytes(hm.prc_C[b]), bytes(hm.xo_C[b])) for b in range(ns)]
    outs = [(_pinned(np.zeros(H * nr, np.uint64)), _pinned(np.zeros(H * nr, np.uint64)),
             _pinned(np.zeros(2 * H * nc * nr, np.uint64)),
             _pinned(np.zeros(2 * H * nc * nr, np.uint64))) for b in range(ns)]
    p64 = lambda v: v.ctypes.data_as(micsa.C.POINTER(micsa.C.c_uint64))
    lib = micsa.lib()

    def job():
        prc = (micsa.PRC * (ns * nr)).from_buffer_copy(b"".join(x[0] for x in start))
        xo = (micsa.Xoshiro * (ns * nr)).from_buffer_copy(b"".join(x[1] for x in start))
        for b in range(ns):
            micsa.check(ctx.h, lib.micsa_upload_couplings(ctx.h, b, p64(J[b][1])), "couplings")
            micsa.check(ctx.h, lib.micsa_upload_spins(ctx.h, b, p64(sp[b][0][1]), p64(sp[b][1][1])),
                        "spins")
        t, nref, nmeas = 0, 0, 0
        while t < a.steps:
            if t & (t - 1) == 0:
                # refresh t was drawn ahead (t > 0); draw the next one during
                # the iterations that follow (side stream)
                if t == 0:
                    ctx.refresh_demons_async(0, prc, xo, hm.thr)
                else:
                    ctx.refresh_commit()
                if (2 * t if t else 1) < a.steps:
                    ctx.refresh_demons_ahead(0, prc, xo, hm.thr)
                nref += 1
            nxt = 1
            while nxt <= t:
                nxt <<= 1
            nxt = min(nxt, a.steps)
            ctx.iterate(nxt - t)
            t = nxt
            if t & (t - 1) == 0 or t == a.steps:
                ctx.measure(spin=True, demon=True)
                nmeas += 1
        ctx.refresh_wait()
        for b in range(ns):
            o = outs[b]
            micsa.check(ctx.h, lib.micsa_download_spins(ctx.h, b, p64(o[0][1]), p64(o[1][1])), "spins")
            micsa.check(ctx.h, lib.micsa_download_demons(ctx.h, b, p64(o[2][1]), p64(o[3][1])),
                        "demons")
        return nref, nmeas

    job()  # warm-up: jump tables, graph capture
    ctx.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    nref, nmeas = job()
    ctx.synchronize()
    te = dist.max(time.perf_counter() - t0)
    h2d = ns * (12 * H * 8 + 2 * H * nr * 8) + nref * ns * nr * 120 * 8
    d2h = nmeas * ns * nr * (4 + 8) + ns * (2 * H * nr * 8 + 2 * 2 * H * nc * nr * 8)
    return {"value": round(attempts * a.steps * dist.world / (te * 1e12), 4), "unit": UNIT,
            "h2d_bytes_per_step": int(h2d // a.steps), "d2h_bytes_per_step": int(d2h // a.steps),
            "ms_per_step": round(te * 1e3 / a.steps, 4), "job_ms": round(te * 1e3, 2),
            "refreshes": nref, "measurements": nmeas,
            "step": "job of `steps` iterations: state upload, GPU demon refresh (drawn ahead on a "
                    "side stream) + energy readback at t=0,1,2,4,..., final spins+demons readback"}


def e2e_upload_every_step(a, dist, ctx, demons, attempts):
    """Worst case: every iteration re-uploads the whole demon set from
    pinned host memory (the reference's refresh upload, main.cu:355-362) and
    reads the energies back."""
    ns, nr = a.nsamples, a.nr
    pinned = [(_pinned(demons[b][0]), _pinned(demons[b][1])) for b in range(ns)]
    h2d = sum(p[1].nbytes for pair in pinned for p in pair)
    d2h = ns * nr * (4 + 8)

    def step():
        for b in range(ns):
            ctx.upload_demons(b, pinned[b][0][1], pinned[b][1][1])
        ctx.iterate(1)
        ctx.measure(spin=True, demon=True)

    for _ in range(max(1, a.warmup)):
        step()
    ke = max(3, min(20, a.steps // 2))
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        step()
    te = dist.max((time.perf_counter() - t0) / ke)
    return {"value": round(attempts * dist.world / (te * 1e12), 4), "unit": UNIT,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": round(te * 1e3, 4), "steps": ke}


def cpu_state(L, nr, ns, nc, seed=7):
    """Seeded random reference-layout state for the CPU arms (same shapes).
    Everything here comes from numpy and the oracle's own packer (packing_J,
    ini.c:521-578): the CPU arms never load the product library."""
    import oracle
    rng = np.random.default_rng(seed)
    H = (L // 4) ** 3 // 2
    out = []
    for _ in range(ns):
        J = oracle.pack_couplings(L, *(rng.integers(0, 2, size=L ** 3, dtype=np.uint8)
                                       for _ in range(3)))
        e = rng.integers(0, 2 ** 63, size=H * nr, dtype=np.uint64)
        o = rng.integers(0, 2 ** 63, size=H * nr, dtype=np.uint64)
        w0 = rng.integers(0, 2 ** 63, size=2 * H * nc * nr, dtype=np.uint64)
        w1 = rng.integers(0, 2 ** 63, size=2 * H * nc * nr, dtype=np.uint64) & w0
        out.append([J, e, o, w0, w1])
    return out


def cpu_iterations(L, nr, nc, states, n, threads):
    """n iterations of the oracle (the reference algorithm on its own layout,
    every replica range on its own thread); returns attempts/ps."""
    import oracle
    t0 = time.perf_counter()
    for _ in range(n):
        for J, e, o, w0, w1 in states:
            oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, threads)
    dt = time.perf_counter() - t0
    return float(L ** 3) * nr * nc * len(states) * n / (dt * 1e12), dt


def cpu_baseline(a, budget_s=10.0):
    """Bounded sample: oracle iterations of ONE sample of the workload on all
    host cores until ~budget_s of wall time."""
    threads = os.cpu_count() or 1
    st = cpu_state(a.L, a.nr, 1, a.nc)
    v, dt = cpu_iterations(a.L, a.nr, a.nc, st, 1, threads)
    n = max(1, int(budget_s / max(dt, 1e-3)))
    v, dt = cpu_iterations(a.L, a.nr, a.nc, st, n, threads)
    return {"value": round(v, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d oracle iteration(s) of 1 of %d samples (L=%d, %d replicas, nc=%d), %.1f s"
                      % (n, a.nsamples, a.L, a.nr, a.nc, dt)}


def run_reference(a):
    """CPU restatement of the reference (oracle/) on all host cores: each
    step is a bounded sample of the workload, one iteration of ONE of its
    samples (the samples are independent and identical in cost), so that the
    default --steps run ends in a couple of minutes."""
    threads = os.cpu_count() or 1
    st = cpu_state(a.L, a.nr, 1, a.nc)
    cpu_iterations(a.L, a.nr, a.nc, st, a.warmup, threads)
    v, dt = cpu_iterations(a.L, a.nr, a.nc, st, a.steps, threads)
    return v, dt / a.steps * 1e3, threads


def config(a):
    return {"workload": "plain micSA, L=%d periodic +-J lattice, %d samples x %d replicas, "
                        "nc=%d demons/site; step = one iteration = %d half-sweeps + demon walk"
                        % (a.L, a.nsamples, a.nr, a.nc, 2 * a.nc),
            "words": "the %d replicas of a site sit in %d uint32 words moved as one %d-byte "
                     "vector: bit-identical to the reference's uint64 multispin words, the "
                     "bitwise arithmetic done on 32-bit lanes (dtype u32)"
                     % (a.nr, a.nr // 32, a.nr // 8),
            "L": a.L, "replicas": a.nr, "samples": a.nsamples, "nc": a.nc,
            "beta": BETA, "l2": "inputs larger than L2: each step streams %.0f MB of demon planes"
                                % (a.nsamples * 2 * a.nc * 2 * a.L ** 3 / 2 * a.nr / 8 / 1e6),
            "parallelism": "replicas (an independent lattice per GPU)"}


BATCH_L = (8, 16, 24, 32, 48)          # L = 12 is not a legal size (multiple of 8)
BATCH_SWEEPS = (1 << 10, 1 << 12, 1 << 14)


def batched_jobs(a):
    """The batched configuration: a.nsamples jobs, L uniform in BATCH_L and
    sweeps uniform in BATCH_SWEEPS (or one shape with --batch-L), 64
    replicas, independent seeds from master seed 20260101."""
    rng = np.random.default_rng(20260101)
    n = a.nsamples
    Ls = rng.choice(BATCH_L, size=n) if a.batch_L is None else np.full(n, a.batch_L)
    its = rng.choice(BATCH_SWEEPS, size=n) if a.batch_L is None else np.full(n, a.iterations)
    seeds = rng.integers(1, 2 ** 63 - 1, size=(n, 2), dtype=np.int64)
    return [dict(L=int(L), nr=a.nr, nc=a.nc, iterations=int(it), seed_J=int(sj), seed_u=int(su),
                 beta=BETA) for L, it, (sj, su) in zip(Ls, its, seeds)]


def run_batched(a, dist):
    """All jobs through micsa_run_batch (host initialisation of the jobs
    outside the timed part; context creation, uploads, GPU refreshes,
    iterations and measurement readbacks inside), against the plain path of
    one micsa_run_batch call per job, timed on one job of every (L, sweeps)
    pair and weighted by the pair counts.  Both sides are timed after a call
    of every shape they use, so neither pays the launch-shape timing, which
    the library does once per shape and process."""
    import collections
    import micsa
    jobs = batched_jobs(a)
    for w in range(max(0, a.warmup)):  # the first warm-up runs every job: every group shape
        micsa.run_batch(jobs if w == 0 else jobs[:4], device=dist.local)
    dist.barrier()
    es, ed, sec = micsa.run_batch(jobs, device=dist.local)
    sec = dist.max(sec)
    attempts = sum(float(j["L"] ** 3) * j["nr"] * j["nc"] * j["iterations"] for j in jobs)
    count = collections.Counter((j["L"], j["iterations"]) for j in jobs)
    plain, per = 0.0, {}
    for L in sorted({k[0] for k in count}):  # launch shapes timed once per shape and process
        micsa.run_batch([dict(next(j for j in jobs if j["L"] == L), iterations=8)],
                        device=dist.local)
    for key in sorted(count):
        job = next(j for j in jobs if (j["L"], j["iterations"]) == key)
        _, _, t1 = micsa.run_batch([job], device=dist.local)
        per["L%d_%d" % key] = round(t1, 4)
        plain += count[key] * t1
    return {"anneals_per_s": round(len(jobs) * dist.world / sec, 2),
            "plain_anneals_per_s": round(len(jobs) / plain, 2),
            "speedup_vs_plain": round(plain / sec, 2),
            "attempts_per_ps": round(attempts * dist.world / (sec * 1e12), 4),
            "job_seconds": round(sec, 4), "plain_seconds_estimated": round(plain, 3),
            "plain_seconds_per_job": per, "jobs": len(jobs),
            "pairs": {"L%d_%d" % k: v for k, v in sorted(count.items())}}


SERVE_L = (16, 24, 32, 48, 64, 96)


def served_trace(a):
    """Poisson arrivals (mean 200 requests/s, seed 7); per request L uniform in
    SERVE_L, 32 or 64 replicas, sweeps log-uniform in [2^10, 2^16], its own
    coupling and spin seeds."""
    rng = np.random.default_rng(7)
    t, out = 0.0, []
    for _ in range(a.requests):
        t += rng.exponential(1.0 / 200.0)
        out.append(dict(arrival=t, L=int(rng.choice(SERVE_L)), nr=int(rng.choice([32, 64])),
                        nc=a.nc, iterations=int(round(2.0 ** rng.uniform(10.0, 16.0))),
                        seed_J=int(rng.integers(1, 2 ** 62)), seed_u=int(rng.integers(1, 2 ** 62)),
                        beta=BETA))
    return out


def run_served(a, dist):
    """The trace through micsa_serve (continuous batching, HBM budget), in
    real time; against the plain path: one micsa_run_batch call per request,
    first come first served, service times from a per-(L, nr) linear fit of
    single-job runs at 2^10 and 2^14 iterations."""
    import micsa
    reqs = served_trace(a)
    budget = int(a.hbm_gb * (1 << 30))
    micsa.serve([dict(r, arrival=0.0, iterations=8) for r in reqs[:6]], device=dist.local)
    es, ed, times, sec = micsa.serve(reqs, device=dist.local, hbm_budget=budget)
    lat = np.array([t[2] - r["arrival"] for t, r in zip(times, reqs)])
    wait = np.array([t[1] - r["arrival"] for t, r in zip(times, reqs)])
    attempts = sum(float(r["L"] ** 3) * r["nr"] * r["nc"] * r["iterations"] for r in reqs)
    fit = {}
    for L in SERVE_L:
        for nr in (32, 64):
            job = dict(L=L, nr=nr, nc=a.nc, seed_J=11, seed_u=13, beta=BETA)
            micsa.run_batch([dict(job, iterations=8)], device=dist.local)  # shape timing
            _, _, t1 = micsa.run_batch([dict(job, iterations=1 << 10)], device=dist.local)
            _, _, t2 = micsa.run_batch([dict(job, iterations=1 << 14)], device=dist.local)
            b = (t2 - t1) / ((1 << 14) - (1 << 10))
            fit[(L, nr)] = (t1 - b * (1 << 10), b)
    free_at, plat = 0.0, []
    for r in reqs:
        c0, c1 = fit[(r["L"], r["nr"])]
        start = max(r["arrival"], free_at)
        free_at = start + c0 + c1 * r["iterations"]
        plat.append(free_at - r["arrival"])
    plat = np.array(plat)
    return {"anneals_per_s": round(len(reqs) / sec, 3),
            "p50_latency_s": round(float(np.percentile(lat, 50)), 3),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 3),
            "p50_wait_s": round(float(np.percentile(wait, 50)), 3),
            "attempts_per_ps": round(attempts / (sec * 1e12), 4), "seconds": round(sec, 3),
            "arrival_window_s": round(reqs[-1]["arrival"], 3),
            "plain_anneals_per_s": round(len(reqs) / free_at, 3),
            "plain_p50_latency_s": round(float(np.percentile(plat, 50)), 3),
            "plain_p99_latency_s": round(float(np.percentile(plat, 99)), 3),
            "speedup_vs_plain": round(free_at / sec, 2),
            "plain_fit_s": {"L%d_nr%d" % k: [round(v[0], 4), round(v[1] * 1e6, 3)]
                            for k, v in fit.items()},
            "hbm_budget_gib": a.hbm_gb}


def main():
    a = parse()
    dist = Dist()
    if a.workload == "served":
        if a.impl == "reference" or dist.rank != 0:
            if dist.rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "served workload: timed on "
                                  "the GPU arm only"}))
            dist.close()
            return
        r = run_served(a, dist)
        print(json.dumps({
            "metric": "anneals/s, served Poisson stream", "unit": "anneals/s",
            "value": r["anneals_per_s"], "n_gpus": 1, "steps": a.requests, "warmup": 1,
            "ms_per_step": round(r["seconds"] * 1e3 / a.requests, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic: Poisson trace, 200 requests/s, seed 7, per-request seeds",
            "config": {"workload": "served: %d requests, L uniform in %s, 32/64 replicas, sweeps "
                                   "log-uniform in [2^10, 2^16], nc=%d, continuous batching "
                                   "under a %g GiB HBM budget" % (a.requests, list(SERVE_L), a.nc,
                                                                  a.hbm_gb),
                       "requests": a.requests, "nc": a.nc},
            "detail": r}))
        dist.close()
        return
    if a.workload == "batched":
        if a.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "batched workload: timed on the "
                              "GPU arm only; the CPU port's rate is the plain workload's"}))
            dist.close()
            return
        r = run_batched(a, dist)
        if dist.rank == 0:
            mixed = a.batch_L is None
            print(json.dumps({
                "metric": "anneals/s, batched %s" % ("mixed-L stream" if mixed else "L=%d" % a.batch_L),
                "unit": "anneals/s", "value": r["anneals_per_s"], "n_gpus": dist.world,
                "steps": a.nsamples, "warmup": a.warmup,
                "ms_per_step": round(r["job_seconds"] * 1e3 / a.nsamples, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic: %d jobs seeded from master seed 20260101" % a.nsamples,
                "config": {"workload": "batched: %d independent reference runs (1 sample each), L "
                                       "uniform in %s, sweeps uniform in %s, %d replicas, nc=%d, "
                                       "reference refresh/measurement schedule" % (
                                           a.nsamples, list(BATCH_L) if mixed else [a.batch_L],
                                           list(BATCH_SWEEPS) if mixed else [a.iterations],
                                           a.nr, a.nc),
                           "jobs": a.nsamples, "replicas": a.nr, "nc": a.nc},
                "detail": r}))
        dist.close()
        return
    line = {"metric": METRIC, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32",
            "data": "synthetic: seeded reference initialisation (Janus couplings, uniform spins, "
                    "heat-bath demons at beta=0.909)", "config": config(a)}
    if a.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        v, ms, threads = run_reference(a)
        line.update({"impl": "reference", "value": round(v, 6), "ms_per_step": round(ms, 3),
                     "n_gpus": dist.world, "dtype": "u64",
                     "data": "synthetic: seeded random reference-layout state",
                     "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads,
                                      "kind": "port",
                                      "sample": "each step one iteration of 1 of the %d samples "
                                                "(L=%d, %d replicas, nc=%d), CPU oracle"
                                                % (a.nsamples, a.L, a.nr, a.nc)},
                     "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0}})
        print(json.dumps(line))
        dist.close()
        return
    r = run_micsa(a, dist)
    line.update({"value": round(r["value"], 4), "ms_per_step": round(r["ms"], 4),
                 "roofline": r["roof"], "e2e": r["e2e"], "gpu_launches": r["launches"],
                 "clocks": r["clocks"]})
    if dist.rank == 0 and dist.world == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(a)
    if dist.rank == 0:
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
