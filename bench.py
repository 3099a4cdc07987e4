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
    ap.add_argument("--no-extras", action="store_true",
                    help="plain: leave out the compact batched and served results")
    ap.add_argument("--extra-requests", type=int, default=60,
                    help="plain: requests of the compact served result")
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
    fit = 1
    if "fit=" in ctx.tuning():
        fit = int(ctx.tuning().split("fit=")[1].split()[0].rstrip("|"))
    kernel = ("k_sweep_dep (dataflow sweep: the %d half-sweeps of each of %d iteration(s) in one "
              "launch; time per half-sweep)" % (2 * nc, fit) if "load=flow" in ctx.tuning()
              else "k_sweep (micSA half-sweep)")
    roof = {"bound": "hbm", "kernel": kernel,
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": kind,
            "algorithmic_bytes_per_launch": int(per_launch),
            "launch_ms": round(sweep_ms, 5), "iteration_ms_profiled": round(iter_ms, 5),
            "autotune": _tuning_summary(ctx.tuning()),
            "traffic": traffic, "traffic_source": tnote}
    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not a.no_e2e:
        e2e = e2e_job(a, dist, ctx, hm, attempts)
        e2e["upload_every_step"] = e2e_upload_every_step(a, dist, ctx, demons, attempts)
    ctx.close()
    return dict(value=value, ms=ms, roof=roof, clocks=ck, e2e=e2e, launches=launches,
                attempts=attempts)


def _tuning_summary(t):
    """The chosen launch shape, the number of candidates timed and the three
    fastest (zc/pd/split/occ/load/tile: ms per half-sweep)."""
    head, _, rest = t.partition("|")
    cands = []
    for c in rest.split():
        shape, _, ms = c.partition(":")
        try:
            cands.append((float(ms.rstrip("ms")), shape))
        except ValueError:
            pass
    cands.sort()
    best = " ".join("%s:%.5fms" % (sh, ms) for ms, sh in cands[:3])
    return "%s | %d candidates timed%s" % (head.strip(), len(cands), (", fastest " + best) if best else "")


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
            "step": "job of `steps` iterations: state upload, GPU demon refresh (asked for ahead; "
                    "drawn in place at each commit for contexts on the dataflow sweep, else on a "
                    "side stream) + energy readback at t=0,1,2,4,..., final spins+demons readback "
                    "into pinned buffers"}


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


def reference_cuda(a):
    """The reference's own CUDA build on this GPU: its kernels
    (d_oneMCstepBN_multisample, d_Walk; PROGRAM/src/main.cu compiled
    unmodified for sm_103a by oracle/ref_gpu/build_ref_gpu.sh) launched as
    Monte_Carlo launches them (main.cu:254-305: 2*nc sweeps and two walks per
    iteration, calculate_blocks' geometry), on the same workload shape with a
    seeded random reference-layout state, timed with CUDA events on the
    harness's stream.  None where the cubin of this shape was not built."""
    import oracle
    cubin = oracle.ref_gpu_cubin(a.L, a.nr, max(2, a.nsamples))
    if cubin is None:
        return {"unavailable": "reference kernels for L=%d NR=%d not built here (they are compiled "
                               "from the reference sources, absent where build() ran)" % (a.L, a.nr)}
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
    except Exception:
        return {"unavailable": "no torch"}
    st = cpu_state(a.L, a.nr, a.nsamples, a.nc, seed=11)
    ref = oracle.RefGPU(cubin, a.L, a.nr, a.nsamples, a.nc)
    try:
        for s, (J, e, o, w0, w1) in enumerate(st):
            ref.upload(s, J, e, o, w0, w1)
        n = max(5, min(a.steps, 50))
        ms = ref.time(max(3, a.warmup), n)
        tpb, nb = ref.launch_shape()
    finally:
        ref.close()
    attempts = float(a.L ** 3) * a.nr * a.nsamples * a.nc
    return {"value": round(attempts / (ms * 1e9), 4), "unit": UNIT, "ms_per_step": round(ms, 4),
            "steps": n, "kernels": "d_oneMCstepBN_multisample x %d + d_Walk x 2 per iteration"
                                   % (2 * a.nc),
            "launch": "grid (%d, %d) x %d threads" % (nb, a.nsamples, tpb),
            "source": "the reference's PROGRAM/src/main.cu compiled unmodified for sm_103a "
                      "(-DL=%d -DNBETAS=1 -DNUMBITSPREBUSQUEDAS=10 -DJANUS -DWALK, NR=%d, "
                      "MAXNSAMPLES=%d), driven by oracle/ref_gpu/ref_gpu_harness.cu"
                      % (a.L, a.nr, max(2, a.nsamples))}


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


def run_batched(a, dist, plain_sample=64):
    """All jobs through micsa_run_batch (host initialisation of the jobs
    outside the timed part; context creation, uploads, GPU refreshes,
    iterations and measurement readbacks inside), against the plain path --
    one micsa_run_batch call per job, the way one reference process runs one
    sample -- measured on a seeded sample of `plain_sample` of the jobs (all
    of them when plain_sample >= the job count), one call after another.
    Both sides are timed after a call of every shape they use, so neither
    pays the launch-shape timing, which the library does once per shape and
    process."""
    import micsa
    jobs = batched_jobs(a)
    for w in range(max(0, a.warmup)):  # the first warm-up runs every job: every group shape
        micsa.run_batch(jobs if w == 0 else jobs[:4], device=dist.local)
    dist.barrier()
    es, ed, sec = micsa.run_batch(jobs, device=dist.local)
    sec = dist.max(sec)
    attempts = sum(float(j["L"] ** 3) * j["nr"] * j["nc"] * j["iterations"] for j in jobs)
    for L in sorted({j["L"] for j in jobs}):  # launch shapes timed once per shape and process
        micsa.run_batch([dict(next(j for j in jobs if j["L"] == L), iterations=8)],
                        device=dist.local)
    rng = np.random.default_rng(4242)
    pick = (np.arange(len(jobs)) if plain_sample >= len(jobs)
            else np.sort(rng.choice(len(jobs), size=plain_sample, replace=False)))
    plain_attempts, plain_s = 0.0, 0.0
    for k in pick:
        job = jobs[int(k)]
        _, _, t1 = micsa.run_batch([job], device=dist.local)
        plain_s += t1
        plain_attempts += float(job["L"] ** 3) * job["nr"] * job["nc"] * job["iterations"]
    # the sample's measured time per attempt, applied to the whole stream
    plain_total = plain_s * attempts / plain_attempts
    return {"anneals_per_s": round(len(jobs) * dist.world / sec, 2),
            "plain_anneals_per_s": round(len(jobs) / plain_total, 2),
            "speedup_vs_plain": round(plain_total / sec, 2),
            "attempts_per_ps": round(attempts * dist.world / (sec * 1e12), 4),
            "plain_attempts_per_ps": round(plain_attempts / (plain_s * 1e12), 4),
            "job_seconds": round(sec, 4), "jobs": len(jobs),
            "plain": "%d of the %d jobs (seeded sample) run one micsa_run_batch call each, one "
                     "after another: %.3f s for %.3g attempts; the stream's plain time is that "
                     "time per attempt x the stream's attempts" % (len(pick), len(jobs), plain_s,
                                                                    plain_attempts),
            "mode": os.environ.get("MICSA_BATCH", "groups")}


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


def _replay_plain(reqs, device):
    """The per-request path of the trace: one worker takes the requests in
    arrival order, waits for each to arrive and runs it alone through
    micsa_run_batch([job]) (host initialisation, context, uploads, refreshes,
    iterations, measurements: one reference process per request).  Returns
    the finish time of each request, seconds after the start."""
    import micsa
    t0 = time.perf_counter()
    fin = []
    for r in reqs:
        wait = r["arrival"] - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        micsa.run_batch([r], device=device)
        fin.append(time.perf_counter() - t0)
    return np.array(fin)


def run_served(a, dist, requests=None):
    """The trace through micsa_serve (continuous batching, HBM budget), in
    real time, against the plain path replayed in real time on the same GPU
    after it: one request at a time, first come first served.  Both sides
    are timed after a call of every shape they use (launch shapes are timed
    once per shape and process)."""
    import micsa
    reqs = served_trace(a)
    if requests is not None:
        reqs = reqs[:requests]
    budget = int(a.hbm_gb * (1 << 30))
    micsa.serve([dict(r, arrival=0.0, iterations=8) for r in reqs[:6]], device=dist.local)
    es, ed, times, sec = micsa.serve(reqs, device=dist.local, hbm_budget=budget)
    lat = np.array([t[2] - r["arrival"] for t, r in zip(times, reqs)])
    wait = np.array([t[1] - r["arrival"] for t, r in zip(times, reqs)])
    attempts = sum(float(r["L"] ** 3) * r["nr"] * r["nc"] * r["iterations"] for r in reqs)
    for shape in sorted({(r["L"], r["nr"]) for r in reqs}):
        r0 = next(r for r in reqs if (r["L"], r["nr"]) == shape)
        micsa.run_batch([dict(r0, iterations=8)], device=dist.local)
    fin = _replay_plain(reqs, dist.local)
    plat = fin - np.array([r["arrival"] for r in reqs])
    return {"anneals_per_s": round(len(reqs) / sec, 3),
            "p50_latency_s": round(float(np.percentile(lat, 50)), 3),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 3),
            "p50_wait_s": round(float(np.percentile(wait, 50)), 3),
            "attempts_per_ps": round(attempts / (sec * 1e12), 4), "seconds": round(sec, 3),
            "arrival_window_s": round(reqs[-1]["arrival"], 3), "requests": len(reqs),
            "plain_anneals_per_s": round(len(reqs) / float(fin[-1]), 3),
            "plain_p50_latency_s": round(float(np.percentile(plat, 50)), 3),
            "plain_p99_latency_s": round(float(np.percentile(plat, 99)), 3),
            "plain_seconds": round(float(fin[-1]), 3),
            "speedup_vs_plain": round(float(fin[-1]) / sec, 2),
            "plain": "measured: the same trace replayed in real time, one request at a time in "
                     "arrival order, each through its own micsa_run_batch call",
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
        if dist.world == 1:
            try:
                line["reference_cuda"] = reference_cuda(a)
            except Exception as e:
                line["reference_cuda"] = {"unavailable": str(e)[:300]}
        print(json.dumps(line))
        dist.close()
        return
    r = run_micsa(a, dist)
    line.update({"value": round(r["value"], 4), "ms_per_step": round(r["ms"], 4),
                 "roofline": r["roof"], "e2e": r["e2e"], "gpu_launches": r["launches"],
                 "clocks": r["clocks"]})
    if dist.rank == 0 and dist.world == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(a)
    if dist.world == 1 and not a.no_extras:
        line.update(extras(a, dist))
    if dist.rank == 0:
        print(json.dumps(line))
    dist.close()


def extras(a, dist):
    """The batched and served configurations, compactly, after the headline's
    timed region: the full 512-job mixed-L batch against a measured sample of
    48 of its jobs run one call each, and the first `--extra-requests` of the
    served trace against the same requests replayed one at a time."""
    import argparse
    out = {}
    b = argparse.Namespace(**vars(a))
    b.nsamples, b.batch_L, b.nr, b.nc, b.warmup = 512, None, 64, 6, 1
    try:
        r = run_batched(b, dist, plain_sample=48)
        out["batched"] = {k: r[k] for k in ("anneals_per_s", "plain_anneals_per_s",
                                            "speedup_vs_plain", "attempts_per_ps", "job_seconds",
                                            "jobs", "plain", "mode")}
        out["batched"]["workload"] = ("512 jobs, L uniform in %s, sweeps uniform in %s, 64 "
                                      "replicas, nc=6" % (list(BATCH_L), list(BATCH_SWEEPS)))
    except Exception as e:  # the headline line is still printed
        out["batched"] = {"error": str(e)[:300]}
    c = argparse.Namespace(**vars(a))
    c.nc = 6
    try:
        r = run_served(c, dist, requests=a.extra_requests)
        out["served"] = {k: r[k] for k in (
            "anneals_per_s", "p50_latency_s", "p99_latency_s", "plain_anneals_per_s",
            "plain_p50_latency_s", "plain_p99_latency_s", "speedup_vs_plain", "attempts_per_ps",
            "requests", "plain")}
        out["served"]["workload"] = ("first %d requests of the Poisson trace (200/s, seed 7), L "
                                     "uniform in %s, 32/64 replicas, sweeps log-uniform in "
                                     "[2^10, 2^16], %g GiB HBM budget"
                                     % (a.extra_requests, list(SERVE_L), a.hbm_gb))
    except Exception as e:
        out["served"] = {"error": str(e)[:300]}
    return out


if __name__ == "__main__":
    main()
