/*
 * C ABI of libmicsa (include/micsa.h): context lifetime, reference-layout
 * uploads and downloads, the Monte_Carlo step, graph-replayed iterations
 * and measurements.  Every CUDA call is checked; failures are reported as a
 * status code plus a message, never by exiting.
 */
#include <cuda_runtime.h>

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "micsa.h"
#include "micsa_jump.h"
#include "micsa_kernels.cuh"

#define MICSA_TUNE_MAX 400

struct micsa_ctx {
  micsa_config cfg;
  micsa_geo g;
  cudaStream_t stream = nullptr;
  uint32_t *spin = nullptr, *dem0 = nullptr, *dem1 = nullptr, *rnd = nullptr;
  uint8_t *jb = nullptr, *lut = nullptr;
  uint32_t *te = nullptr, *keys = nullptr;
  int *walk = nullptr;
  uint8_t *active = nullptr; /* per-sample flags, 1 = runs */
  unsigned *flow_ctl = nullptr; /* counters of the dataflow sweep: 4 + ns*L words */
  uint64_t *stage = nullptr;
  unsigned long long *acc = nullptr;
  size_t stage_words = 0, acc_words = 0;
  int have_lut = 0;
  std::vector<int> have_j, have_spin, have_dem;
  std::vector<uint8_t> active_host; /* host copy of the run flags */
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;   /* g.fit iterations (dataflow), else one */
  std::vector<cudaGraph_t> rem_graph;     /* rem_graph[k]: one launch of k < g.fit iterations */
  std::vector<cudaGraphExec_t> rem_exec;
  std::vector<int64_t> rem_launches;
  int64_t launches = 0;
  int resident = 0;        /* small lattice: iterations run in shared memory */
  int split = 0;           /* k > 0: half-sweep launches per group of k samples, group-major
                              (a smaller L2 working set); 0: all samples per launch */
  micsa_tma tma = {};      /* tensor maps of the demon arrays (staged sweep) */
  int64_t graph_launches = 0; /* kernels per replay of the iteration graph */
  int ntune = 0;           /* launch shapes timed at creation */
  int tune_zc[MICSA_TUNE_MAX] = {0}, tune_pd[MICSA_TUNE_MAX] = {0};
  int tune_split[MICSA_TUNE_MAX] = {0}, tune_occ[MICSA_TUNE_MAX] = {0};
  int tune_load[MICSA_TUNE_MAX] = {0}, tune_tw[MICSA_TUNE_MAX] = {0}; /* load: 0 direct .. 5 quad */
  double tune_ms[MICSA_TUNE_MAX] = {0};
  int tune_cached = 0; /* the shape came from an earlier context's timing */
  /* demon refresh on the device: jump tables of one segment length */
  micsa_refresh_plan plan = {};
  uint64_t *plan_lcg = nullptr, *plan_xo = nullptr, *plan_fib = nullptr;
  uint64_t *rec = nullptr, *rec_host = nullptr; /* start records: device, pinned staging */
  size_t rec_words = 0;
  cudaEvent_t rec_copied = nullptr;  /* staging upload done */
  /* refresh drawn ahead into a back buffer on a side stream */
  cudaStream_t side = nullptr;
  uint32_t *back0 = nullptr, *back1 = nullptr;
  uint64_t *rec_b = nullptr;
  size_t rec_b_words = 0;
  cudaEvent_t ahead_done = nullptr;  /* the draw into the back buffer is done */
  cudaEvent_t commit_done = nullptr; /* the back buffer has been copied out */
  int ahead_first = 0, ahead_count = 0; /* pending drawn-ahead samples (count 0: none) */
  /* a pending refresh recorded but not drawn yet (drawn in place at the
   * commit): its records are in rec_b, its jump plan is (def_nw, def_wps) */
  int ahead_deferred = 0, def_wps = 0;
  int64_t def_nw = 0;
  uint64_t def_thr[3] = {0, 0, 0};
  std::thread advancer;              /* host advance of the last refresh's streams */
  char err[512] = {0};
};

namespace {

int fail(micsa_ctx *c, int code, const char *fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof c->err, fmt, ap);
    va_end(ap);
  }
  return code;
}

#define MICSA_CK(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(ctx, MICSA_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                              \
  } while (0)

struct sizes {
  int64_t P, H, spin_w, dem_w, rnd_w, jb_b, stage_w, acc_w;
};

sizes sizes_of(const micsa_config &c) {
  sizes s;
  const int64_t L = c.L, W = c.nr / 32;
  s.P = L * L * L / 2;
  s.H = (L / 4) * (L / 4) * (L / 4) / 2;
  s.spin_w = (int64_t)c.nsamples * 2 * s.P * W;
  s.dem_w = (int64_t)c.nsamples * 2 * c.nc * s.P * W;
  s.rnd_w = 3 * s.P * W;
  s.jb_b = (int64_t)c.nsamples * 2 * s.P;
  const int64_t st_spin = 2 * s.H * c.nr, st_dem = 2 * (int64_t)c.nc * s.H * c.nr;
  s.stage_w = st_spin > st_dem ? st_spin : st_dem;
  const int64_t nd = L / 2 + 1, npair = c.nr / 2;
  s.acc_w = (int64_t)c.nsamples * (2 * c.nr + npair + npair * 3 * nd);
  return s;
}

int check_cfg(const micsa_config *c, char *msg, size_t n) {
  if (!c) return snprintf(msg, n, "null configuration"), MICSA_ERR_ARG;
  /* int32 energies (the reference's int h_Ener): |E| <= 3 L^3 < 2^31 up to L = 888 */
  if (c->L < 8 || c->L > 888 || c->L % 8)
    return snprintf(msg, n, "L=%d must be a multiple of 8 in [8, 888] (int32 energies)", c->L),
           MICSA_ERR_ARG;
  if (c->nr < 32 || c->nr % 32)
    return snprintf(msg, n, "nr=%d must be a positive multiple of 32", c->nr),
           MICSA_ERR_UNSUPPORTED;
  if (c->nsamples < 1 || c->nsamples > MICSA_MAX_SAMPLES)
    return snprintf(msg, n, "nsamples=%d must be in [1, %d]", c->nsamples, MICSA_MAX_SAMPLES),
           MICSA_ERR_ARG;
  if (c->nc < 1 || c->nc > 6)
    return snprintf(msg, n, "nc=%d must be in [1, 6]", c->nc), MICSA_ERR_ARG;
  /* sweep kernels index one colour plane with 32-bit word offsets */
  const uint64_t words = (uint64_t)c->L * c->L * c->L / 2 * (uint64_t)(c->nr / 32);
  if (words >= (1ULL << 32))
    return snprintf(msg, n, "L=%d with nr=%d exceeds 2^32 words per colour plane", c->L, c->nr),
           MICSA_ERR_UNSUPPORTED;
  return MICSA_OK;
}

int set_device(micsa_ctx *ctx) {
  MICSA_CK(cudaSetDevice(ctx->cfg.device));
  return MICSA_OK;
}

int check_sample(micsa_ctx *ctx, int sample) {
  if (sample < 0 || sample >= ctx->cfg.nsamples)
    return fail(ctx, MICSA_ERR_ARG, "sample %d out of range [0, %d)", sample, ctx->cfg.nsamples);
  return MICSA_OK;
}

int ensure_stage(micsa_ctx *ctx) {
  if (ctx->stage) return MICSA_OK;
  MICSA_CK(cudaMalloc(&ctx->stage, ctx->stage_words * sizeof(uint64_t)));
  return MICSA_OK;
}

/* The device address of a caller's host buffer that kernels may write
 * directly (page-locked and mapped, as cudaHostAlloc and mapped registered
 * memory are), else nullptr.  A download into such a buffer converts
 * straight into it across the host link: one pass at link speed instead of a
 * conversion into the staging buffer and then a copy. */
uint64_t *device_view(uint64_t *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError(); /* not a pointer the runtime knows: the staged path */
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? (uint64_t *)a.devicePointer : nullptr;
}

int ready_for_sweeps(micsa_ctx *ctx, int need_demons) {
  for (int s = 0; s < ctx->cfg.nsamples; s++) {
    if (!ctx->active_host[s]) continue; /* frozen: never touched by the sweeps */
    if (!ctx->have_j[s] || !ctx->have_spin[s])
      return fail(ctx, MICSA_ERR_STATE, "sample %d has no couplings or spins uploaded", s);
    if (need_demons && !ctx->have_dem[s])
      return fail(ctx, MICSA_ERR_STATE, "sample %d has no demons uploaded", s);
  }
  return MICSA_OK;
}

/* f(s0, s1) over [0, n) on up to hardware_concurrency threads, at least
 * `grain` items each; the calling thread takes the first share */
template <class F>
void parallel_for(int64_t n, int64_t grain, F f) {
  const unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = n / (grain > 0 ? grain : 1);
  if (nt > (int64_t)(hw ? hw : 1)) nt = hw ? hw : 1;
  if (nt < 1) nt = 1;
  std::vector<std::thread> pool;
  for (int64_t t = 1; t < nt; t++) {
    try {
      pool.emplace_back(f, n * t / nt, n * (t + 1) / nt);
    } catch (...) {
      f(n * t / nt, n * (t + 1) / nt);
    }
  }
  f(0, n / nt);
  for (auto &th : pool) th.join();
}

/* One micSA half-sweep of samples s .. s+n-1 in one launch: of every sample
 * (s = 0, n = ns), or of a group -- the launch then sees only the group's
 * spins, couplings and demon planes through offset pointers. */
cudaError_t launch_half(micsa_ctx *ctx, const micsa_geo &g, int s, int n, int p, int ic,
                        int64_t *launches) {
  if (launches) ++*launches;
  if (s == 0 && n == g.ns)
    return micsa_launch_sweep_micsa(g, p, ic, ctx->spin, ctx->dem0, ctx->dem1, ctx->jb, ctx->walk,
                                    &ctx->tma, ctx->stream);
  const size_t PW = (size_t)g.P * g.W;
  micsa_geo g1 = g;
  g1.ns = n;
  g1.s0 = s; /* the staged sweep addresses the whole demon arrays */
  g1.active = g.active ? g.active + s : nullptr; /* a frozen sample returns at once */
  return micsa_launch_sweep_micsa(g1, p, ic, ctx->spin + s * 2 * PW,
                                  ctx->dem0 + s * 2 * (size_t)g.nc * PW,
                                  ctx->dem1 + s * 2 * (size_t)g.nc * PW,
                                  ctx->jb + (size_t)s * 2 * g.P, ctx->walk + s, &ctx->tma,
                                  ctx->stream);
}

/* The half-sweeps of one iteration (ic = ic0 .. ic1-1).  split = 0: plane by
 * plane, all samples per launch.  split = k > 0: group-major, all half-sweeps
 * of samples 0 .. k-1 (one launch each), then of the next k, ...: the spins
 * that stay hot in L2 across consecutive launches are one group's (k = 1:
 * sample-major).  g.flow (whole iterations): one dataflow launch, its tiles
 * sample-major (split > 0) or half-sweep-major. */
cudaError_t launch_halves(micsa_ctx *ctx, const micsa_geo &g, int split, int ic0, int ic1,
                          int64_t *launches) {
  cudaError_t e = cudaSuccess;
  if (g.flow && ic0 == 0 && ic1 == g.nc) { /* the whole iteration in one dataflow launch */
    if (launches) ++*launches;
    return micsa_launch_sweep_flow(g, split > 0, ctx->spin, ctx->dem0, ctx->dem1, ctx->jb,
                                   ctx->walk, ctx->flow_ctl, ctx->stream);
  }
  const int k = split > 0 && split < g.ns ? split : g.ns;
  for (int s = 0; s < g.ns; s += k)
    for (int ic = ic0; ic < ic1; ic++)
      for (int p = 0; p < 2; p++)
        if ((e = launch_half(ctx, g, s, s + k <= g.ns ? k : g.ns - s, p, ic, launches)) !=
            cudaSuccess)
          return e;
  return e;
}

/* Launch shapes chosen so far in this process, by (device, L, nr, samples,
 * nc, TMA maps usable): a context of a shape timed before takes the earlier
 * choice and table instead of timing again, so batches and servers that open
 * many contexts of a few shapes pay for each shape once. */
struct tune_entry {
  int zc, pd, split, occ, tma, async, pipe, tw, flow, quad, fit, pers, half, xs, n;
  std::vector<int> zcs, pds, splits, occs, loads, tws;
  std::vector<double> ms;
};
std::mutex tune_mu;
std::map<std::tuple<int, int, int, int, int, int>, tune_entry> tune_cache;

std::tuple<int, int, int, int, int, int> tune_key(const micsa_ctx *ctx) {
  return std::make_tuple(ctx->cfg.device, ctx->g.L, ctx->cfg.nr, ctx->g.ns, ctx->g.nc,
                         ctx->tma.ok ? 1 : 0);
}

/* Launch-shape autotuner: time whole iterations (the half-sweeps in their
 * real launch order and the walk, replayed as a graph) for every z-chunk
 * length that divides L, prefetch distance, sample order (merged or
 * sample-major), register budget, load scheme and block shape, on the
 * freshly zeroed buffers; keep the fastest, then zero the buffers and the
 * walks again.  Results do not
 * depend on the choice (each site is updated by exactly one thread either
 * way); only the speed does.  MICSA_TUNE_CACHE=0 times every context afresh
 * instead of reusing the process's earlier choice for the same shape. */
int autotune(micsa_ctx *ctx) {
  micsa_geo &g = ctx->g;
  int zcs[8];
  const int nz = micsa_sweep_zc_candidates(g.L, zcs, 8);
  const int pds[3] = {0, 2, 4};
  /* MICSA_SWEEP_ZC / MICSA_SWEEP_PD pin the shape and skip the timing
   * (reproducible launch shapes, e.g. under a profiler, whose per-launch
   * overhead would distort the choice) */
  if (const char *ez = getenv("MICSA_SWEEP_ZC")) {
    const char *ep = getenv("MICSA_SWEEP_PD");
    const int zc = atoi(ez), pd = ep ? atoi(ep) : 0;
    int ok = 0;
    for (int c = 0; c < nz; c++) ok |= zcs[c] == zc;
    if (!ok || (pd != 0 && pd != 2 && pd != 4) || (pd && pd >= zc))
      return fail(ctx, MICSA_ERR_ARG, "MICSA_SWEEP_ZC=%d / MICSA_SWEEP_PD=%d not a shape for L=%d",
                  zc, pd, g.L);
    g.zc = zc;
    g.pd = pd;
    const char *es = getenv("MICSA_SWEEP_SPLIT"), *eo = getenv("MICSA_SWEEP_OCC"),
               *et = getenv("MICSA_SWEEP_TMA"), *ea = getenv("MICSA_SWEEP_ASYNC"),
               *ep2 = getenv("MICSA_SWEEP_PIPE"), *ew = getenv("MICSA_SWEEP_TILE"),
               *ef = getenv("MICSA_SWEEP_FLOW"), *eq = getenv("MICSA_SWEEP_QUAD");
    ctx->split = es && atoi(es) > 0 && g.ns > 1 ? (atoi(es) < g.ns ? atoi(es) : g.ns) : 0;
    g.tma = et && atoi(et) && ctx->tma.ok;
    g.async = ea && atoi(ea) && g.W == 2 && !g.tma;
    g.pipe = ep2 && atoi(ep2) && !g.tma && !g.async;
    g.tw = ew && !strcmp(ew, "row") && !g.tma && micsa_sweep_wide_differs(g.L, eq && atoi(eq) ? 4 : 2);
    g.flow = ef && atoi(ef) && !g.tma && !g.async && !g.pipe;
    g.quad = eq && atoi(eq) && g.W == 1 && !g.tma && !g.async && !g.pipe && !g.flow;
    if (const char *ep = getenv("MICSA_SWEEP_PERS")) g.pers = g.flow && atoi(ep) == 1;
    if (const char *eh = getenv("MICSA_FLOW_HALF")) g.half = g.flow && !g.pers && atoi(eh) == 1;
    if (const char *ex = getenv("MICSA_FLOW_XS"))
      g.xs = g.flow && !g.pers && !g.half && atoi(ex) == 1;
    if (const char *ek = getenv("MICSA_FLOW_ITERS")) {
      const int k = atoi(ek);
      if (g.flow && k >= 1 && k <= 64) g.fit = k;
    }
    const int oc = eo ? atoi(eo) : 3;
    g.occ = g.pipe ? (oc == 2 ? 2 : 3) : (oc == 4 ? 4 : 3);
    ctx->ntune = 0;
    return MICSA_OK;
  }
  const char *ec = getenv("MICSA_TUNE_CACHE");
  const bool use_cache = !(ec && !strcmp(ec, "0"));
  if (use_cache) {
    std::lock_guard<std::mutex> lk(tune_mu);
    auto it = tune_cache.find(tune_key(ctx));
    if (it != tune_cache.end()) {
      const tune_entry &t = it->second;
      g.zc = t.zc;
      g.pd = t.pd;
      ctx->split = t.split;
      g.occ = t.occ;
      g.tma = t.tma;
      g.async = t.async;
      g.pipe = t.pipe;
      g.tw = t.tw;
      g.flow = t.flow;
      g.quad = t.quad;
      g.fit = t.fit;
      g.pers = t.pers;
      g.half = t.half;
      g.xs = t.xs;
      ctx->ntune = t.n;
      for (int c = 0; c < t.n; c++) {
        ctx->tune_zc[c] = t.zcs[c];
        ctx->tune_pd[c] = t.pds[c];
        ctx->tune_split[c] = t.splits[c];
        ctx->tune_occ[c] = t.occs[c];
        ctx->tune_load[c] = t.loads[c];
        ctx->tune_tw[c] = t.tws[c];
        ctx->tune_ms[c] = t.ms[c];
      }
      ctx->tune_cached = 1;
      return MICSA_OK;
    }
  }
  cudaEvent_t e0, e1;
  MICSA_CK(cudaEventCreate(&e0));
  MICSA_CK(cudaEventCreate(&e1));
  double best = 1e30;
  int best_zc = zcs[nz - 1], best_pd = 0, best_split = 0, best_occ = 3, best_tma = 0;
  int best_async = 0, best_pipe = 0, best_tw = 0, best_flow = 0, best_quad = 0, best_pers = 0;
  int n = 0;
  const int ntw = micsa_sweep_wide_differs(g.L) ? 2 : 1, ntw4 = micsa_sweep_wide_differs(g.L, 4) ? 2 : 1;
  /* The dataflow sweep is timed only for large lattices (many slabs per
   * half-sweep, so that its tiles rarely wait): contexts of small lattices
   * run side by side in batches and servers, where blocks that wait on
   * dependencies hold SM slots the other contexts' kernels need (the batched
   * mixed-L stream lost 30% with it).  Alone it loses as well below L=128,
   * where a half-sweep has too few slabs for tiles to find work ahead (L=64 x 8
   * samples: 1.30 against 7.02 attempts/ps; L=96 x 16: 3.85 against 6.75).
   * MICSA_SWEEP_FLOW=0 leaves it out everywhere. */
  const char *ef0 = getenv("MICSA_SWEEP_FLOW");
  const bool try_flow = !(ef0 && !strcmp(ef0, "0")) && g.L >= 128;
  const int reps = 3;
  /* sample orders: all samples per launch, or sample-major.  Launches per
   * group of 2 to 8 samples (MICSA_SWEEP_SPLIT=k) are not timed: alone they
   * beat both at L=96 x 16 samples (7.28 against 6.76 attempts/ps), but the
   * server's pools, tuned alone and run side by side, lost 9 to 12% of their
   * throughput with them */
  const int sps[2] = {0, 1}, nsp = g.ns > 1 ? 2 : 1;
  const int nocc = g.W % 4 ? 2 : 1; /* the 4-blocks variant exists for VW <= 2 */
  /* tm: 0 direct loads, 1 TMA-staged demon tiles, 2 cp.async double buffer (W = 2),
   * 3 loads pipelined one step ahead in registers (register budget for 3 or 2
   * blocks per SM instead of 3 or 4), 4 direct loads in one dataflow launch
   * per iteration (split: its tiles sample-major or half-sweep-major), 5
   * direct loads with four one-word sites per thread (W = 1) */
  /* mean ms per half-sweep of the shape in g (sample order sp): reps replays
   * of a graph of one iteration (16 for the dataflow sweep) in their launch
   * order, as micsa_iterate runs them -- timed launch by launch, small
   * lattices would measure the host's launch rate -- with the walk
   * advancing, as in a run: the x translation of the demon planes misaligns
   * their rows at most shifts, never at shift 0 */
  auto time_shape = [&](int sp, int nrep, double *per) -> int {
    cudaGraph_t gr = nullptr;
    cudaGraphExec_t ge = nullptr;
    MICSA_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = launch_halves(ctx, g, sp, 0, g.nc, nullptr);
    if (le == cudaSuccess)
      le = g.fit > 1 ? micsa_launch_walk_add(g, ctx->walk, g.fit, ctx->stream)
                     : micsa_launch_walk_advance(g, ctx->walk, ctx->stream);
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &gr);
    MICSA_CK(le);
    MICSA_CK(ce);
    const cudaError_t ie = cudaGraphInstantiate(&ge, gr, 0);
    cudaGraphDestroy(gr);
    MICSA_CK(ie);
    float ms = 0;
    cudaError_t te = cudaGraphLaunch(ge, ctx->stream); /* warm-up */
    if (te == cudaSuccess) te = cudaEventRecord(e0, ctx->stream);
    for (int rep = 0; rep < nrep && te == cudaSuccess; rep++) te = cudaGraphLaunch(ge, ctx->stream);
    if (te == cudaSuccess) te = cudaEventRecord(e1, ctx->stream);
    if (te == cudaSuccess) te = cudaEventSynchronize(e1);
    if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
    cudaGraphExecDestroy(ge);
    MICSA_CK(te);
    *per = ms / (2.0 * g.nc * nrep * g.fit);
    return MICSA_OK;
  };
  int rc = MICSA_OK;
  for (int tm = 0; tm < 7; tm++)
  for (int tw = 0; tw < (tm == 5 ? ntw4 : ntw); tw++)
  for (int oc = 0; oc < nocc; oc++)
  for (int si = 0; si < nsp; si++)
  for (int c = 0; c < nz; c++)
    for (int d = 0; d < 3; d++) {
      if (pds[d] && pds[d] >= zcs[c]) continue; /* prefetch only within a slab */
      if (tm == 1 && (!ctx->tma.ok || zcs[c] > 4)) continue; /* staged tiles: <= 4 planes */
      if (tm == 2 && (g.W != 2 || pds[d])) continue;          /* no L2 prefetch there */
      if (tw && (tm == 1 || tm == 2)) continue; /* whole-row blocks: direct and pipelined loads */
      if (((tm == 4 || tm == 6) && !try_flow) || (tm == 5 && g.W != 1)) continue;
      const int sp = sps[si];
      g.zc = zcs[c];
      g.pd = pds[d];
      g.occ = tm == 3 ? (oc ? 2 : 3) : (oc ? 4 : 3);
      g.tma = tm == 1;
      g.async = tm == 2;
      g.pipe = tm == 3;
      g.tw = tw;
      g.flow = tm == 4 || tm == 6;
      g.pers = tm == 6;
      g.quad = tm == 5;
      /* the dataflow sweep is timed carrying 16 iterations per launch, its
       * best form (the launch boundary drains the GPU); the count is
       * settled below for the chosen shape */
      g.fit = g.flow ? 16 : 1;
      /* one iteration's half-sweeps (16 for the dataflow sweep) in their
       * launch order, captured and replayed as a graph the way micsa_iterate
       * runs them: timed launch by launch, small lattices would measure the
       * host's launch rate */
      double per = 0;
      if ((rc = time_shape(sp, reps, &per))) return rc;
      if (n < MICSA_TUNE_MAX) {
        ctx->tune_zc[n] = g.zc;
        ctx->tune_pd[n] = g.pd;
        ctx->tune_split[n] = sp;
        ctx->tune_occ[n] = g.occ;
        ctx->tune_load[n] = tm;
        ctx->tune_tw[n] = tw;
        ctx->tune_ms[n] = per;
        n++;
      }
      if (per < best) {
        best = per;
        best_zc = g.zc;
        best_pd = g.pd;
        best_split = sp;
        best_occ = g.occ;
        best_tma = g.tma;
        best_async = g.async;
        best_pipe = g.pipe;
        best_tw = g.tw;
        best_flow = g.flow;
        best_pers = g.pers;
        best_quad = g.quad;
      }
    }
  /* the closest candidates differ by a few percent, about the spread of a
   * short timing: re-time the best four with three times the replays and
   * keep the fastest of those */
  {
    int top[4], nt = 0;
    for (int c = 0; c < n && c < MICSA_TUNE_MAX; c++) {
      const bool full = nt == 4;
      int k = full ? 3 : nt++;
      if (full && ctx->tune_ms[c] >= ctx->tune_ms[top[3]]) continue;
      top[k] = c;
      for (; k > 0 && ctx->tune_ms[top[k]] < ctx->tune_ms[top[k - 1]]; k--) {
        const int t = top[k];
        top[k] = top[k - 1];
        top[k - 1] = t;
      }
    }
    if (nt > 1) {
      best = 1e30;
      for (int k = 0; k < nt; k++) {
        const int c = top[k], tm = ctx->tune_load[c];
        g.zc = ctx->tune_zc[c];
        g.pd = ctx->tune_pd[c];
        g.occ = ctx->tune_occ[c];
        g.tma = tm == 1;
        g.async = tm == 2;
        g.pipe = tm == 3;
        g.tw = ctx->tune_tw[c];
        g.flow = tm == 4 || tm == 6;
        g.pers = tm == 6;
        g.quad = tm == 5;
        g.fit = g.flow ? 16 : 1;
        double per = 0;
        if ((rc = time_shape(ctx->tune_split[c], 3 * reps, &per))) return rc;
        if (per < best) {
          best = per;
          best_zc = g.zc;
          best_pd = g.pd;
          best_split = ctx->tune_split[c];
          best_occ = g.occ;
          best_tma = g.tma;
          best_async = g.async;
          best_pipe = g.pipe;
          best_tw = g.tw;
          best_flow = g.flow;
          best_pers = g.pers;
          best_quad = g.quad;
        }
      }
    }
  }
  ctx->ntune = n;
  g.zc = best_zc;
  g.pd = best_pd;
  ctx->split = best_split;
  g.occ = best_occ;
  g.tma = best_tma;
  g.async = best_async;
  g.pipe = best_pipe;
  g.tw = best_tw;
  g.flow = best_flow;
  g.pers = best_pers;
  g.quad = best_quad;
  g.fit = 1;
  if (g.flow) {
    /* iterations per dataflow launch: the wavefront runs on from one
     * iteration into the next instead of draining the GPU at every launch
     * boundary; timed per iteration on graphs of k iterations */
    double best_it = 1e30;
    int best_fit = 1;
    for (int k : {1, 4, 16}) {
      g.fit = k;
      cudaGraph_t gr = nullptr;
      cudaGraphExec_t ge = nullptr;
      MICSA_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t le = launch_halves(ctx, g, ctx->split, 0, g.nc, nullptr);
      if (le == cudaSuccess) le = micsa_launch_walk_add(g, ctx->walk, k, ctx->stream);
      const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &gr);
      MICSA_CK(le);
      MICSA_CK(ce);
      const cudaError_t ie = cudaGraphInstantiate(&ge, gr, 0);
      cudaGraphDestroy(gr);
      MICSA_CK(ie);
      const int r = k >= 16 ? 1 : (k >= 4 ? 2 : 6);
      float ms = 0;
      cudaError_t te = cudaGraphLaunch(ge, ctx->stream);
      if (te == cudaSuccess) te = cudaEventRecord(e0, ctx->stream);
      for (int rep = 0; rep < r && te == cudaSuccess; rep++) te = cudaGraphLaunch(ge, ctx->stream);
      if (te == cudaSuccess) te = cudaEventRecord(e1, ctx->stream);
      if (te == cudaSuccess) te = cudaEventSynchronize(e1);
      if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
      cudaGraphExecDestroy(ge);
      MICSA_CK(te);
      const double per = ms / ((double)r * k);
      if (per < best_it) best_it = per, best_fit = k;
    }
    g.fit = best_fit;
    if (!g.pers) {
      /* half-height tiles: twice the tiles per slab, each half as long, for a
       * sweep whose wavefront of dependencies bounds it */
      g.half = 1;
      cudaGraph_t gr = nullptr;
      cudaGraphExec_t ge = nullptr;
      MICSA_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t le = launch_halves(ctx, g, ctx->split, 0, g.nc, nullptr);
      if (le == cudaSuccess)
        le = g.fit > 1 ? micsa_launch_walk_add(g, ctx->walk, g.fit, ctx->stream)
                       : micsa_launch_walk_advance(g, ctx->walk, ctx->stream);
      const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &gr);
      MICSA_CK(le);
      MICSA_CK(ce);
      const cudaError_t ie = cudaGraphInstantiate(&ge, gr, 0);
      cudaGraphDestroy(gr);
      MICSA_CK(ie);
      const int rr = g.fit >= 16 ? 1 : (g.fit >= 4 ? 2 : 6);
      float ms = 0;
      cudaError_t te = cudaGraphLaunch(ge, ctx->stream);
      if (te == cudaSuccess) te = cudaEventRecord(e0, ctx->stream);
      for (int rep = 0; rep < rr && te == cudaSuccess; rep++) te = cudaGraphLaunch(ge, ctx->stream);
      if (te == cudaSuccess) te = cudaEventRecord(e1, ctx->stream);
      if (te == cudaSuccess) te = cudaEventSynchronize(e1);
      if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
      cudaGraphExecDestroy(ge);
      MICSA_CK(te);
      if (ms / ((double)rr * g.fit) >= best_it) g.half = 0;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (use_cache) {
    tune_entry t;
    t.zc = g.zc;
    t.pd = g.pd;
    t.split = ctx->split;
    t.occ = g.occ;
    t.tma = g.tma;
    t.async = g.async;
    t.pipe = g.pipe;
    t.tw = g.tw;
    t.flow = g.flow;
    t.quad = g.quad;
    t.fit = g.fit;
    t.pers = g.pers;
    t.half = g.half;
    t.xs = g.xs;
    t.n = n;
    t.zcs.assign(ctx->tune_zc, ctx->tune_zc + n);
    t.pds.assign(ctx->tune_pd, ctx->tune_pd + n);
    t.splits.assign(ctx->tune_split, ctx->tune_split + n);
    t.occs.assign(ctx->tune_occ, ctx->tune_occ + n);
    t.loads.assign(ctx->tune_load, ctx->tune_load + n);
    t.tws.assign(ctx->tune_tw, ctx->tune_tw + n);
    t.ms.assign(ctx->tune_ms, ctx->tune_ms + n);
    std::lock_guard<std::mutex> lk(tune_mu);
    tune_cache.emplace(tune_key(ctx), std::move(t)); /* the first timing of a shape stays */
  }
  return MICSA_OK;
}

/* the launches of k iterations (k > 1 only with the dataflow sweep, which
 * carries them in one launch); *launches counts them */
int enqueue_micsa_iterations(micsa_ctx *ctx, int k, int64_t *launches) {
  micsa_geo g = ctx->g;
  g.fit = g.flow ? k : 1;
  if (!g.flow && k != 1) return fail(ctx, MICSA_ERR_STATE, "several iterations per launch");
  MICSA_CK(launch_halves(ctx, g, ctx->split, 0, g.nc, launches));
  if (k == 1)
    MICSA_CK(micsa_launch_walk_advance(g, ctx->walk, ctx->stream));
  else
    MICSA_CK(micsa_launch_walk_add(g, ctx->walk, k, ctx->stream));
  if (launches) ++*launches;
  return MICSA_OK;
}

int enqueue_micsa_iteration(micsa_ctx *ctx, int64_t *launches) {
  return enqueue_micsa_iterations(ctx, 1, launches);
}

/* the iteration graph of k iterations */
int capture_iterations(micsa_ctx *ctx, int k, cudaGraph_t *graph, cudaGraphExec_t *exec,
                       int64_t *launches) {
  MICSA_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  *launches = 0;
  int rc = enqueue_micsa_iterations(ctx, k, launches);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  MICSA_CK(e);
  *graph = g;
  MICSA_CK(cudaGraphInstantiate(exec, g, 0));
  return MICSA_OK;
}

}  // namespace

extern "C" {

int64_t micsa_footprint_bytes(const micsa_config *cfg) {
  char msg[128];
  if (check_cfg(cfg, msg, sizeof msg) != MICSA_OK) return -1;
  sizes s = sizes_of(*cfg);
  return 4 * (s.spin_w + 2 * s.dem_w + s.rnd_w) + s.jb_b + 8 * (s.stage_w + s.acc_w) + 4096 +
         4 * (9 * (int64_t)cfg->nr) + 4 * MICSA_MAX_SAMPLES;
}

int micsa_create(const micsa_config *cfg, micsa_ctx **out) {
  if (!out) return MICSA_ERR_ARG;
  *out = nullptr;
  char msg[256];
  int rc = check_cfg(cfg, msg, sizeof msg);
  if (rc != MICSA_OK) {
    fprintf(stderr, "micsa_create: %s\n", msg);
    return rc;
  }
  micsa_ctx *ctx = new (std::nothrow) micsa_ctx();
  if (!ctx) return MICSA_ERR_NOMEM;
  ctx->cfg = *cfg;
  sizes s = sizes_of(*cfg);
  micsa_geo &g = ctx->g;
  g.L = cfg->L;
  g.Lh = cfg->L / 2;
  g.W = cfg->nr / 32;
  g.nc = cfg->nc;
  g.ns = cfg->nsamples;
  g.nr = cfg->nr;
  g.P = s.P;
  g.zc = 0;
  g.pd = 0;
  g.occ = 3;
  g.tma = 0;
  g.async = 0;
  g.pipe = 0;
  g.tw = 0;
  g.flow = 0;
  g.quad = 0;
  g.fit = 1;
  g.pers = 0;
  g.half = 0;
  g.xs = 0;
  {
    /* MICSA_SWEEP_PF=n: the dataflow sweep requests n demon planes of each
     * tile into L2 before its dependency wait (0: none) */
    const char *e = getenv("MICSA_SWEEP_PF");
    g.pf = e ? atoi(e) : 0;
    if (g.pf < 0) g.pf = 0;
  }
  {
    /* MICSA_PDL=0: plain launches of the sweeps */
    const char *e = getenv("MICSA_PDL");
    g.pdl = !(e && !strcmp(e, "0"));
  }
  g.s0 = 0;
  g.H = s.H;
  g.active = nullptr;
  ctx->stage_words = (size_t)s.stage_w;
  ctx->acc_words = (size_t)s.acc_w;
  ctx->have_j.assign(cfg->nsamples, 0);
  ctx->have_spin.assign(cfg->nsamples, 0);
  ctx->have_dem.assign(cfg->nsamples, 0);
  ctx->active_host.assign(cfg->nsamples, 1);
  *out = ctx;
#define MICSA_CK_CREATE(call)                                                  \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      fprintf(stderr, "micsa_create: %s: %s\n", #call, cudaGetErrorString(e_)); \
      micsa_destroy(ctx);                                                      \
      *out = nullptr;                                                          \
      return e_ == cudaErrorMemoryAllocation ? MICSA_ERR_NOMEM : MICSA_ERR_CUDA; \
    }                                                                          \
  } while (0)
  MICSA_CK_CREATE(cudaSetDevice(cfg->device));
  {
    /* highest priority: work drawn ahead on the side stream yields to it */
    int least = 0, greatest = 0;
    MICSA_CK_CREATE(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    MICSA_CK_CREATE(cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, greatest));
  }
  MICSA_CK_CREATE(cudaMalloc(&ctx->spin, 4 * s.spin_w));
  MICSA_CK_CREATE(cudaMalloc(&ctx->dem0, 4 * s.dem_w));
  MICSA_CK_CREATE(cudaMalloc(&ctx->dem1, 4 * s.dem_w));
  MICSA_CK_CREATE(cudaMalloc(&ctx->rnd, 4 * s.rnd_w));
  MICSA_CK_CREATE(cudaMalloc(&ctx->jb, s.jb_b));
  MICSA_CK_CREATE(cudaMalloc(&ctx->lut, 4096));
  MICSA_CK_CREATE(cudaMalloc(&ctx->te, 4 * 8 * (size_t)cfg->nr));
  MICSA_CK_CREATE(cudaMalloc(&ctx->keys, 4 * (size_t)cfg->nr));
  MICSA_CK_CREATE(cudaMalloc(&ctx->walk, sizeof(int) * MICSA_MAX_SAMPLES));
  MICSA_CK_CREATE(cudaMalloc(&ctx->acc, 8 * ctx->acc_words));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->walk, 0, sizeof(int) * MICSA_MAX_SAMPLES, ctx->stream));
  MICSA_CK_CREATE(cudaMalloc(&ctx->active, (size_t)cfg->nsamples));
  MICSA_CK_CREATE(cudaMalloc(&ctx->flow_ctl, sizeof(unsigned) * (4 + (size_t)cfg->nsamples * cfg->L)));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->flow_ctl, 0,
                                  sizeof(unsigned) * (4 + (size_t)cfg->nsamples * cfg->L), ctx->stream));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->active, 1, (size_t)cfg->nsamples, ctx->stream));
  g.active = ctx->active;
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->spin, 0, 4 * s.spin_w, ctx->stream));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->dem0, 0, 4 * s.dem_w, ctx->stream));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->dem1, 0, 4 * s.dem_w, ctx->stream));
  MICSA_CK_CREATE(cudaStreamSynchronize(ctx->stream));
  {
    /* MICSA_RESIDENT=0 keeps small lattices on the per-half-sweep kernels */
    const char *er = getenv("MICSA_RESIDENT");
    const size_t need = micsa_resident_smem(cfg->L, cfg->nc);
    int optin = 0;
    MICSA_CK_CREATE(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                           cfg->device));
    ctx->resident = need > 0 && need <= (size_t)optin && !(er && !strcmp(er, "0"));
  }
  MICSA_CK_CREATE(micsa_make_tma(ctx->g, ctx->dem0, ctx->dem1, &ctx->tma));
  if ((rc = autotune(ctx)) != MICSA_OK) {
    fprintf(stderr, "micsa_create: autotune: %s\n", ctx->err);
    micsa_destroy(ctx);
    *out = nullptr;
    return rc;
  }
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->spin, 0, 4 * s.spin_w, ctx->stream));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->dem0, 0, 4 * s.dem_w, ctx->stream));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->dem1, 0, 4 * s.dem_w, ctx->stream));
  MICSA_CK_CREATE(cudaMemsetAsync(ctx->walk, 0, sizeof(int) * MICSA_MAX_SAMPLES, ctx->stream));
  MICSA_CK_CREATE(cudaStreamSynchronize(ctx->stream));
#undef MICSA_CK_CREATE
  return MICSA_OK;
}

int micsa_tuning_report(const micsa_ctx *ctx, char *buf, size_t n) {
  if (!ctx || !buf || n == 0) return MICSA_ERR_ARG;
  int k = snprintf(buf, n, "zc=%d pd=%d split=%d occ=%d load=%s tile=%s%s%s fit=%d%s |", ctx->g.zc,
                   ctx->g.pd, ctx->split, ctx->g.occ,
                   ctx->g.tma ? "tma" : (ctx->g.async ? "async" : (ctx->g.pipe ? "pipe" : (ctx->g.flow ? (ctx->g.pers ? "pflow" : "flow") : (ctx->g.quad ? "quad" : "direct")))),
                   ctx->g.tw ? "row" : "default", ctx->g.flow && ctx->g.half ? "/2" : "",
                   ctx->g.flow && ctx->g.xs ? "+xs" : "",
                   ctx->g.flow ? ctx->g.fit : 1,
                   ctx->tune_cached ? " cached" : "");
  for (int c = 0; c < ctx->ntune && k > 0 && (size_t)k < n; c++)
    k += snprintf(buf + k, n - (size_t)k, " %d/%d/%d/%d/%d/%d:%.5fms", ctx->tune_zc[c],
                  ctx->tune_pd[c], ctx->tune_split[c], ctx->tune_occ[c], ctx->tune_load[c],
                  ctx->tune_tw[c], ctx->tune_ms[c]);
  return MICSA_OK;
}

int micsa_destroy(micsa_ctx *ctx) {
  if (!ctx) return MICSA_OK;
  if (ctx->advancer.joinable()) ctx->advancer.join();
  if (ctx->side) {
    cudaSetDevice(ctx->cfg.device);
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->back0) cudaFree(ctx->back0);
  if (ctx->back1) cudaFree(ctx->back1);
  if (ctx->rec_b) cudaFree(ctx->rec_b);
  if (ctx->ahead_done) cudaEventDestroy(ctx->ahead_done);
  if (ctx->commit_done) cudaEventDestroy(ctx->commit_done);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  for (cudaGraphExec_t e : ctx->rem_exec)
    if (e) cudaGraphExecDestroy(e);
  for (cudaGraph_t gr : ctx->rem_graph)
    if (gr) cudaGraphDestroy(gr);
  void *bufs[] = {ctx->spin, ctx->dem0,     ctx->dem1,    ctx->rnd,      ctx->jb,
                  ctx->lut,  ctx->te,       ctx->keys,    ctx->walk,     ctx->stage,
                  ctx->acc,  ctx->plan_lcg, ctx->plan_xo, ctx->plan_fib, ctx->rec,
                  ctx->active, ctx->flow_ctl};
  for (void *b : bufs)
    if (b) cudaFree(b);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  micsa_refresh_plan_free(&ctx->plan);
  if (ctx->rec_host) cudaFreeHost(ctx->rec_host);
  if (ctx->rec_copied) cudaEventDestroy(ctx->rec_copied);
  delete ctx;
  return MICSA_OK;
}

const char *micsa_last_error(const micsa_ctx *ctx) { return ctx ? ctx->err : "null context"; }

int64_t micsa_kernel_launches(const micsa_ctx *ctx) { return ctx ? ctx->launches : 0; }

void *micsa_stream(micsa_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int micsa_set_lut(micsa_ctx *ctx, const void *lut, size_t bytes) {
  if (!ctx || !lut) return fail(ctx, MICSA_ERR_ARG, "null argument");
  if (bytes != 4096) return fail(ctx, MICSA_ERR_ARG, "LUT must be 4096 bytes, got %zu", bytes);
  /* thresholds non-decreasing, prebisection ranges ordered */
  const uint32_t *w = (const uint32_t *)lut;
  for (int i = 1; i < 256; i++) {
    const uint64_t a = ((uint64_t)w[2 * i - 2] << 32) | w[2 * i - 1];
    const uint64_t b = ((uint64_t)w[2 * i] << 32) | w[2 * i + 1];
    if (b < a) return fail(ctx, MICSA_ERR_ARG, "LUT thresholds decrease at %d", i);
  }
  const uint16_t *pre = (const uint16_t *)((const uint8_t *)lut + 2048);
  for (int i = 0; i < 1024; i++)
    if ((pre[i] & 255) > (pre[i] >> 8))
      return fail(ctx, MICSA_ERR_ARG, "LUT prebisection entry %d has min > max", i);
  int rc = set_device(ctx);
  if (rc) return rc;
  MICSA_CK(cudaMemcpyAsync(ctx->lut, lut, 4096, cudaMemcpyHostToDevice, ctx->stream));
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_lut = 1;
  return MICSA_OK;
}

int micsa_upload_couplings(micsa_ctx *ctx, int sample, const uint64_t *J) {
  if (!ctx || !J) return fail(ctx, MICSA_ERR_ARG, "null argument");
  int rc = check_sample(ctx, sample);
  if (rc || (rc = set_device(ctx)) || (rc = ensure_stage(ctx))) return rc;
  const micsa_geo &g = ctx->g;
  /* the 12*H reference words go up as they are; one bond byte per site is
   * built on the device (bit d = bond in direction d, taken from the words
   * the way d_oneMCstepBN consumes them, main.cu:910-927) */
  MICSA_CK(cudaMemcpyAsync(ctx->stage, J, 12 * 8 * (size_t)g.H, cudaMemcpyHostToDevice,
                           ctx->stream));
  MICSA_CK(micsa_launch_couplings_from_ref(g, ctx->stage, ctx->jb + (int64_t)sample * 2 * g.P,
                                           ctx->stream));
  ctx->launches++;
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_j[sample] = 1;
  return MICSA_OK;
}

int micsa_upload_spins(micsa_ctx *ctx, int sample, const uint64_t *even, const uint64_t *odd) {
  if (!ctx || !even || !odd) return fail(ctx, MICSA_ERR_ARG, "null argument");
  int rc = check_sample(ctx, sample);
  if (rc || (rc = set_device(ctx)) || (rc = ensure_stage(ctx))) return rc;
  const micsa_geo &g = ctx->g;
  const int64_t n = g.H * g.nr;
  MICSA_CK(cudaMemcpyAsync(ctx->stage, even, 8 * n, cudaMemcpyHostToDevice, ctx->stream));
  MICSA_CK(cudaMemcpyAsync(ctx->stage + n, odd, 8 * n, cudaMemcpyHostToDevice, ctx->stream));
  for (int p = 0; p < 2; p++) {
    MICSA_CK(micsa_launch_from_ref(g, p, 0, 0, ctx->stage + p * n,
                                   ctx->spin + ((int64_t)sample * 2 + p) * g.P * g.W, ctx->stream));
    ctx->launches++;
  }
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_spin[sample] = 1;
  return MICSA_OK;
}

int micsa_upload_demons(micsa_ctx *ctx, int sample, const uint64_t *w0, const uint64_t *w1) {
  if (!ctx || !w0 || !w1) return fail(ctx, MICSA_ERR_ARG, "null argument");
  int rc = check_sample(ctx, sample);
  if (rc || (rc = set_device(ctx)) || (rc = ensure_stage(ctx))) return rc;
  const micsa_geo &g = ctx->g;
  const int64_t plane = g.H * g.nr, n = 2 * g.nc * plane;
  const uint64_t *src[2] = {w0, w1};
  uint32_t *dst[2] = {ctx->dem0, ctx->dem1};
  for (int k = 0; k < 2; k++) {
    MICSA_CK(cudaMemcpyAsync(ctx->stage, src[k], 8 * n, cudaMemcpyHostToDevice, ctx->stream));
    for (int p = 0; p < 2; p++)
      for (int ic = 0; ic < g.nc; ic++) {
        const int64_t pi = (int64_t)p * g.nc + ic;
        MICSA_CK(micsa_launch_from_ref(g, p, ic, 0, ctx->stage + pi * plane,
                                       dst[k] + ((int64_t)sample * 2 * g.nc + pi) * g.P * g.W,
                                       ctx->stream));
        ctx->launches++;
      }
  }
  MICSA_CK(cudaMemsetAsync(ctx->walk + sample, 0, sizeof(int), ctx->stream));
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_dem[sample] = 1;
  return MICSA_OK;
}

namespace {

/* jump tables for segments of wps words, on the host and the device */
int ensure_refresh_plan(micsa_ctx *ctx, int64_t nw, int wps) {
  if (ctx->plan.lcg && ctx->plan.nwords == nw && ctx->plan.words_per_seg == wps) return MICSA_OK;
  MICSA_CK(cudaStreamSynchronize(ctx->stream)); /* the old tables may still be read */
  if (ctx->side) MICSA_CK(cudaStreamSynchronize(ctx->side));
  micsa_refresh_plan_free(&ctx->plan);
  for (uint64_t **b : {&ctx->plan_lcg, &ctx->plan_xo, &ctx->plan_fib}) {
    if (*b) cudaFree(*b);
    *b = nullptr;
  }
  if (micsa_refresh_plan_make(nw, wps, &ctx->plan))
    return fail(ctx, MICSA_ERR_NOMEM, "refresh jump tables (%lld words, %d per segment)",
                (long long)nw, wps);
  const int64_t ns = ctx->plan.nseg;
  MICSA_CK(cudaMalloc(&ctx->plan_lcg, 2 * ns * sizeof(uint64_t)));
  MICSA_CK(cudaMalloc(&ctx->plan_xo, 4 * ns * sizeof(uint64_t)));
  MICSA_CK(cudaMalloc(&ctx->plan_fib, MICSA_FIB_R * ns * sizeof(uint64_t)));
  MICSA_CK(cudaMemcpy(ctx->plan_lcg, ctx->plan.lcg, 2 * ns * 8, cudaMemcpyHostToDevice));
  MICSA_CK(cudaMemcpy(ctx->plan_xo, ctx->plan.xo, 4 * ns * 8, cudaMemcpyHostToDevice));
  MICSA_CK(cudaMemcpy(ctx->plan_fib, ctx->plan.fib, MICSA_FIB_R * ns * 8, cudaMemcpyHostToDevice));
  return MICSA_OK;
}

}  // namespace

int micsa_refresh_wait(micsa_ctx *ctx) {
  if (!ctx) return MICSA_ERR_ARG;
  if (ctx->advancer.joinable()) ctx->advancer.join();
  return MICSA_OK;
}

namespace {

/* Whether a refresh asked for ahead is drawn at once on the side stream or
 * recorded and drawn in place on the context's stream at the commit.  A
 * context whose sweep is the dataflow kernel fills the GPU, and a draw
 * beside it slows both: L=160 x 2 samples, a 20-iteration job with 6
 * refreshes took 59.4 ms drawn ahead (whose commit also copies the demon
 * planes) against 56.6 ms drawn in place.  MICSA_REFRESH_AHEAD=1 keeps the
 * side stream for every context, =0 defers for every context. */
bool refresh_deferred(const micsa_ctx *ctx) {
  if (const char *e = getenv("MICSA_REFRESH_AHEAD")) return atoi(e) == 0;
  return ctx->g.flow != 0;
}

int refresh_occ() {
  const char *e = getenv("MICSA_REFRESH_OCC"); /* 1: the unconstrained-register variant */
  return e && atoi(e) == 1 ? 1 : 6;
}

/* One refresh of samples first .. first+count-1: drawn on the context's
 * stream into the current demons (ahead = 0), or on the side stream into
 * the back buffer (ahead = 1, made current by micsa_refresh_commit), or
 * (ahead = 1 and refresh_deferred) recorded, to be drawn in place by
 * micsa_refresh_commit. */
int refresh_into(micsa_ctx *ctx, int first, int count, void *prc, void *xo, const uint64_t *thr,
                 int ahead) {
  if (!ctx || !prc || !xo || !thr) return fail(ctx, MICSA_ERR_ARG, "null argument");
  if (first < 0 || count < 1 || first + count > ctx->cfg.nsamples)
    return fail(ctx, MICSA_ERR_ARG, "samples [%d, %d) out of range [0, %d)", first, first + count,
                ctx->cfg.nsamples);
  micsa_refresh_wait(ctx); /* the previous refresh's structs may be these */
  int rc = set_device(ctx);
  if (rc) return rc;
  if (ahead && ctx->ahead_count)
    return fail(ctx, MICSA_ERR_STATE, "a refresh drawn ahead is not committed yet");
  const micsa_geo &g = ctx->g;
  micsa_prc_t *P = (micsa_prc_t *)prc;
  micsa_xoshiro_t *X = (micsa_xoshiro_t *)xo;
  const int64_t nw = 2 * g.H * g.nc, nstreams = (int64_t)count * g.nr;
  const size_t words = (size_t)nstreams * MICSA_STREAM_REC;
  /* Segment length in words (64 draws per lane each): each segment's start
   * costs a fixed jump (about 17k instructions per lane), so long segments
   * while enough warps remain -- the longest of 192 ... 64 words that still
   * gives about four waves of the kernel's 12 resident warps per SM (7000
   * warps); below that 48 words while that gives 1024 warps, else 32, else
   * 16, since small calls are latency-bound.  Measured on GB300 over
   * 8 ... 256 words for L = 16 ... 160 (L=160, 2 samples: 7.0 ms at 192
   * words against 7.8 ms at 48).  MICSA_REFRESH_WPS pins the length. */
  auto warps_at = [&](int w) { return (int64_t)count * g.W * ((nw + w - 1) / w); };
  int wps = 0;
  for (int w : {192, 128, 96, 64})
    if (!wps && warps_at(w) >= 7000) wps = w;
  if (!wps) {
    wps = 48;
    while (wps > 16 && warps_at(wps) < 1024) wps -= 16;
  }
  if (const char *e = getenv("MICSA_REFRESH_WPS")) {
    const int v = atoi(e);
    if (v < 1 || v > 4096) return fail(ctx, MICSA_ERR_ARG, "MICSA_REFRESH_WPS=%s", e);
    wps = v;
  }

  /* pinned staging for the start records; the previous upload from it must
   * have completed before it is rewritten */
  if (ctx->rec_copied) MICSA_CK(cudaEventSynchronize(ctx->rec_copied));
  if (ctx->rec_words < words) {
    MICSA_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->side) MICSA_CK(cudaStreamSynchronize(ctx->side));
    if (ctx->rec) cudaFree(ctx->rec);
    if (ctx->rec_host) cudaFreeHost(ctx->rec_host);
    ctx->rec = ctx->rec_host = nullptr;
    ctx->rec_words = 0;
    MICSA_CK(cudaMalloc(&ctx->rec, words * sizeof(uint64_t)));
    MICSA_CK(cudaHostAlloc(&ctx->rec_host, words * sizeof(uint64_t), cudaHostAllocDefault));
    ctx->rec_words = words;
  }
  const bool defer = ahead && refresh_deferred(ctx);
  if (ahead && !defer) {
    const size_t dw = (size_t)ctx->cfg.nsamples * 2 * g.nc * g.P * g.W;
    if (!ctx->side) {
      /* the draw ahead fills what the sweeps leave idle: lowest priority */
      int least = 0, greatest = 0;
      MICSA_CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      MICSA_CK(cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, least));
    }
    if (!ctx->ahead_done)
      MICSA_CK(cudaEventCreateWithFlags(&ctx->ahead_done, cudaEventDisableTiming));
    if (!ctx->commit_done)
      MICSA_CK(cudaEventCreateWithFlags(&ctx->commit_done, cudaEventDisableTiming));
    /* the last commit's copy out of the back buffer must have run */
    MICSA_CK(cudaStreamWaitEvent(ctx->side, ctx->commit_done, 0));
    if (!ctx->back0) MICSA_CK(cudaMalloc(&ctx->back0, 4 * dw));
    if (!ctx->back1) MICSA_CK(cudaMalloc(&ctx->back1, 4 * dw));
  }
  if (ahead) {
    if (ctx->rec_b_words < words) {
      /* a committed draw may still read the old records */
      MICSA_CK(cudaStreamSynchronize(ctx->stream));
      if (ctx->side) MICSA_CK(cudaStreamSynchronize(ctx->side));
      if (ctx->rec_b) cudaFree(ctx->rec_b);
      ctx->rec_b = nullptr;
      ctx->rec_b_words = 0;
      MICSA_CK(cudaMalloc(&ctx->rec_b, words * sizeof(uint64_t)));
      ctx->rec_b_words = words;
    }
  }
  cudaStream_t st = ahead && !defer ? ctx->side : ctx->stream;
  uint64_t *drec = ahead ? ctx->rec_b : ctx->rec;
  if (!ctx->rec_copied) MICSA_CK(cudaEventCreateWithFlags(&ctx->rec_copied, cudaEventDisableTiming));

  /* start records, grouped by warp, built in parallel; checked before
   * anything on the device changes */
  uint64_t *rec = ctx->rec_host;
  std::atomic<int64_t> bad(-1);
  parallel_for(nstreams, 256, [&](int64_t s0, int64_t s1) {
    uint64_t one[MICSA_STREAM_REC];
    for (int64_t s = s0; s < s1; s++) {
      if (micsa_stream_record(&P[s], &X[s], one)) {
        bad.store(s);
        continue;
      }
      const int64_t grp = s / 32, lane = s % 32;
      for (int k = 0; k < MICSA_STREAM_REC; k++) rec[(grp * MICSA_STREAM_REC + k) * 32 + lane] = one[k];
    }
  });
  if (bad.load() >= 0)
    return fail(ctx, MICSA_ERR_ARG, "stream %lld: PR ring pointers are not 24, 55, 61 apart",
                (long long)bad.load());
  if ((rc = ensure_refresh_plan(ctx, nw, wps))) return rc;
  MICSA_CK(cudaMemcpyAsync(drec, rec, words * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
  MICSA_CK(cudaEventRecord(ctx->rec_copied, st));
  if (!defer) {
    micsa_geo gr = g;
    gr.occ = refresh_occ();
    MICSA_CK(micsa_launch_refresh(gr, first, count, nw, wps, ctx->plan.nseg, drec, ctx->plan_lcg,
                                  ctx->plan_xo, ctx->plan_fib, thr, ahead ? ctx->back0 : ctx->dem0,
                                  ahead ? ctx->back1 : ctx->dem1, st));
    ctx->launches++;
  }
  if (defer) { /* drawn in place by micsa_refresh_commit */
    ctx->ahead_deferred = 1;
    ctx->def_nw = nw;
    ctx->def_wps = wps;
    for (int k = 0; k < 3; k++) ctx->def_thr[k] = thr[k];
    ctx->ahead_first = first;
    ctx->ahead_count = count;
  } else if (ahead) {
    MICSA_CK(cudaEventRecord(ctx->ahead_done, ctx->side));
    ctx->ahead_first = first;
    ctx->ahead_count = count;
  } else {
    MICSA_CK(cudaMemsetAsync(ctx->walk + first, 0, count * sizeof(int), ctx->stream));
    for (int s = first; s < first + count; s++) ctx->have_dem[s] = 1;
  }

  /* the caller's streams move past the draws on host threads while the
   * device draws (and runs whatever is queued next) */
  const micsa_refresh_plan *plan = &ctx->plan;
  auto advance = [plan, P, X, nstreams]() {
    parallel_for(nstreams, 64, [&](int64_t s0, int64_t s1) {
      for (int64_t s = s0; s < s1; s++) micsa_streams_advance_plan(plan, &P[s], &X[s]);
    });
  };
  try {
    ctx->advancer = std::thread(advance);
  } catch (...) {
    advance();
  }
  return MICSA_OK;
}

}  // namespace

int micsa_refresh_demons_async(micsa_ctx *ctx, int first, int count, void *prc, void *xo,
                               const uint64_t *thr) {
  return refresh_into(ctx, first, count, prc, xo, thr, 0);
}

int micsa_refresh_demons_ahead(micsa_ctx *ctx, int first, int count, void *prc, void *xo,
                               const uint64_t *thr) {
  return refresh_into(ctx, first, count, prc, xo, thr, 1);
}

int micsa_refresh_commit(micsa_ctx *ctx) {
  if (!ctx) return MICSA_ERR_ARG;
  if (!ctx->ahead_count) return fail(ctx, MICSA_ERR_STATE, "no refresh drawn ahead");
  int rc = set_device(ctx);
  if (rc) return rc;
  const micsa_geo &g = ctx->g;
  if (ctx->ahead_deferred) {
    /* the recorded draw, in place, after the work already queued (the plan
     * is rebuilt only if a refresh of another size came in between) */
    if ((rc = ensure_refresh_plan(ctx, ctx->def_nw, ctx->def_wps))) return rc;
    micsa_geo gr = g;
    gr.occ = refresh_occ();
    MICSA_CK(micsa_launch_refresh(gr, ctx->ahead_first, ctx->ahead_count, ctx->def_nw,
                                  ctx->def_wps, ctx->plan.nseg, ctx->rec_b, ctx->plan_lcg,
                                  ctx->plan_xo, ctx->plan_fib, ctx->def_thr, ctx->dem0, ctx->dem1,
                                  ctx->stream));
    ctx->launches++;
    ctx->ahead_deferred = 0;
    /* a later draw on the side stream rewrites rec_b only after this one */
    if (!ctx->commit_done)
      MICSA_CK(cudaEventCreateWithFlags(&ctx->commit_done, cudaEventDisableTiming));
    MICSA_CK(cudaEventRecord(ctx->commit_done, ctx->stream));
  } else {
    const size_t per = 2 * (size_t)g.nc * g.P * g.W; /* words per sample and plane type */
    const size_t off = (size_t)ctx->ahead_first * per, n = (size_t)ctx->ahead_count * per;
    MICSA_CK(cudaStreamWaitEvent(ctx->stream, ctx->ahead_done, 0));
    MICSA_CK(cudaMemcpyAsync(ctx->dem0 + off, ctx->back0 + off, 4 * n,
                             cudaMemcpyDeviceToDevice, ctx->stream));
    MICSA_CK(cudaMemcpyAsync(ctx->dem1 + off, ctx->back1 + off, 4 * n,
                             cudaMemcpyDeviceToDevice, ctx->stream));
    MICSA_CK(cudaEventRecord(ctx->commit_done, ctx->stream));
  }
  MICSA_CK(cudaMemsetAsync(ctx->walk + ctx->ahead_first, 0, ctx->ahead_count * sizeof(int),
                           ctx->stream));
  for (int s = ctx->ahead_first; s < ctx->ahead_first + ctx->ahead_count; s++) ctx->have_dem[s] = 1;
  ctx->ahead_count = 0;
  return MICSA_OK;
}

int micsa_refresh_demons(micsa_ctx *ctx, int first, int count, void *prc, void *xo,
                         const uint64_t *thr) {
  const int rc = micsa_refresh_demons_async(ctx, first, count, prc, xo, thr);
  micsa_refresh_wait(ctx);
  return rc;
}

int micsa_monte_carlo(micsa_ctx *ctx, int flag, const uint32_t *te, const uint32_t *keys) {
  if (!ctx) return MICSA_ERR_ARG;
  int rc = set_device(ctx);
  if (rc) return rc;
  const micsa_geo &g = ctx->g;
  if (flag == 1) {
    if ((rc = ready_for_sweeps(ctx, 1))) return rc;
    int64_t nl = 0;
    if ((rc = enqueue_micsa_iteration(ctx, &nl))) return rc;
    ctx->launches += nl;
    return MICSA_OK;
  }
  if (flag != 0) return fail(ctx, MICSA_ERR_ARG, "flag must be 0 or 1, got %d", flag);
  if (!te || !keys) return fail(ctx, MICSA_ERR_ARG, "flag 0 needs counters and keys");
  if (!ctx->have_lut) return fail(ctx, MICSA_ERR_STATE, "no LUT uploaded");
  if ((rc = ready_for_sweeps(ctx, 0))) return rc;
  MICSA_CK(cudaMemcpyAsync(ctx->te, te, 4 * 8 * (size_t)g.nr, cudaMemcpyHostToDevice, ctx->stream));
  MICSA_CK(cudaMemcpyAsync(ctx->keys, keys, 4 * (size_t)g.nr, cudaMemcpyHostToDevice, ctx->stream));
  for (int p = 0; p < 2; p++) {
    MICSA_CK(micsa_launch_gen_rnd(g, p, ctx->te + 4 * g.nr * p, ctx->keys, ctx->lut, ctx->rnd,
                                  ctx->stream));
    MICSA_CK(micsa_launch_sweep_metropolis(g, p, ctx->spin, ctx->jb, ctx->rnd, ctx->stream));
  }
  ctx->launches += 4;
  return MICSA_OK;
}

int micsa_iterate(micsa_ctx *ctx, int64_t n) {
  if (!ctx || n < 0) return fail(ctx, MICSA_ERR_ARG, "bad argument");
  int rc = set_device(ctx);
  if (rc || (rc = ready_for_sweeps(ctx, 1))) return rc;
  /* the graph replays ctx->g.fit iterations at a time (the dataflow sweep may
   * carry several per launch); the remainder k < fit runs as one launch of k
   * iterations, from a graph made on first use */
  const int unit = ctx->g.flow && ctx->g.fit > 1 ? ctx->g.fit : 1;
  if (!ctx->graph_exec && !ctx->resident &&
      (rc = capture_iterations(ctx, unit, &ctx->graph, &ctx->graph_exec, &ctx->graph_launches)))
    return rc;
  const int left = unit > 1 ? (int)(n % unit) : 0;
  if (left) {
    if (ctx->rem_exec.size() < (size_t)unit) {
      ctx->rem_graph.resize((size_t)unit, nullptr);
      ctx->rem_exec.resize((size_t)unit, nullptr);
      ctx->rem_launches.resize((size_t)unit, 0);
    }
    if (!ctx->rem_exec[left] &&
        (rc = capture_iterations(ctx, left, &ctx->rem_graph[left], &ctx->rem_exec[left],
                                 &ctx->rem_launches[left])))
      return rc;
  }
  if (ctx->resident) {
    /* small lattices: whole iterations in shared memory, up to 1024 per launch */
    for (int64_t done = 0; done < n;) {
      const int m = (int)(n - done < 1024 ? n - done : 1024);
      MICSA_CK(micsa_launch_resident(ctx->g, m, ctx->spin, ctx->dem0, ctx->dem1, ctx->jb,
                                     ctx->walk, ctx->stream));
      ctx->launches += 2;
      done += m;
    }
    return MICSA_OK;
  }
  for (int64_t i = 0; i < n / unit; i++) MICSA_CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
  ctx->launches += n / unit * ctx->graph_launches;
  if (left) {
    MICSA_CK(cudaGraphLaunch(ctx->rem_exec[left], ctx->stream));
    ctx->launches += ctx->rem_launches[left];
  }
  return MICSA_OK;
}

int micsa_measure(micsa_ctx *ctx, int32_t *e_spin, uint64_t *e_demon, int64_t *q, int64_t *c4) {
  if (!ctx) return MICSA_ERR_ARG;
  int rc = set_device(ctx);
  if (rc) return rc;
  const micsa_geo &g = ctx->g;
  const int ns = g.ns, nr = g.nr, np = nr / 2, nd = g.L / 2 + 1;
  unsigned long long *unsat = ctx->acc, *dem = unsat + ns * nr, *qd = dem + ns * nr,
                     *c4d = qd + ns * np;
  if (e_spin || e_demon) {
    if ((rc = ready_for_sweeps(ctx, e_demon != nullptr))) return rc;
  } else if (q || c4) {
    if ((rc = ready_for_sweeps(ctx, 0))) return rc;
  }
  MICSA_CK(cudaMemsetAsync(ctx->acc, 0, 8 * ctx->acc_words, ctx->stream));
  if (e_spin) { MICSA_CK(micsa_launch_energy(g, ctx->spin, ctx->jb, unsat, ctx->stream)); ctx->launches++; }
  if (e_demon) { MICSA_CK(micsa_launch_demon_energy(g, ctx->dem0, ctx->dem1, dem, ctx->stream)); ctx->launches++; }
  if (q || c4) { MICSA_CK(micsa_launch_overlap(g, ctx->spin, qd, c4d, ctx->stream)); ctx->launches++; }
  std::vector<unsigned long long> h(ctx->acc_words);
  MICSA_CK(cudaMemcpyAsync(h.data(), ctx->acc, 8 * ctx->acc_words, cudaMemcpyDeviceToHost, ctx->stream));
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  const int64_t V = 2 * g.P;
  const unsigned long long *hu = h.data(), *hd = hu + ns * nr, *hq = hd + ns * nr,
                           *hc = hq + ns * np;
  const std::vector<uint8_t> &on = ctx->active_host; /* frozen samples read 0 */
  for (int i = 0; i < ns * nr; i++) {
    if (e_spin) e_spin[i] = on[i / nr] ? (int32_t)(3 * V - 2 * (int64_t)hu[i]) : 0;
    if (e_demon) e_demon[i] = on[i / nr] ? hd[i] : 0;
  }
  for (int i = 0; i < ns * np; i++)
    if (q) q[i] = on[i / np] ? V - 2 * (int64_t)hq[i] : 0;
  if (c4)
    for (int64_t i = 0; i < (int64_t)ns * np * 3 * nd; i++)
      c4[i] = on[i / (np * 3 * nd)] ? V - 2 * (int64_t)hc[i] : 0;
  return MICSA_OK;
}

int micsa_download_spins(micsa_ctx *ctx, int sample, uint64_t *even, uint64_t *odd) {
  if (!ctx || !even || !odd) return fail(ctx, MICSA_ERR_ARG, "null argument");
  int rc = check_sample(ctx, sample);
  if (rc || (rc = set_device(ctx)) || (rc = ensure_stage(ctx))) return rc;
  const micsa_geo &g = ctx->g;
  const int64_t n = g.H * g.nr;
  uint64_t *dv[2] = {device_view(even), device_view(odd)};
  const bool direct = dv[0] && dv[1];
  for (int p = 0; p < 2; p++) {
    MICSA_CK(micsa_launch_to_ref(g, p, 0, nullptr, sample,
                                 ctx->spin + ((int64_t)sample * 2 + p) * g.P * g.W,
                                 direct ? dv[p] : ctx->stage + p * n, ctx->stream));
    ctx->launches++;
  }
  if (!direct) {
    MICSA_CK(cudaMemcpyAsync(even, ctx->stage, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    MICSA_CK(cudaMemcpyAsync(odd, ctx->stage + n, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  return MICSA_OK;
}

int micsa_download_demons(micsa_ctx *ctx, int sample, uint64_t *w0, uint64_t *w1) {
  if (!ctx || !w0 || !w1) return fail(ctx, MICSA_ERR_ARG, "null argument");
  int rc = check_sample(ctx, sample);
  if (rc || (rc = set_device(ctx)) || (rc = ensure_stage(ctx))) return rc;
  const micsa_geo &g = ctx->g;
  const int64_t plane = g.H * g.nr, n = 2 * g.nc * plane;
  const uint32_t *src[2] = {ctx->dem0, ctx->dem1};
  uint64_t *dst[2] = {w0, w1};
  uint64_t *dv[2] = {device_view(w0), device_view(w1)};
  const bool direct = dv[0] && dv[1];
  for (int k = 0; k < 2; k++) {
    for (int p = 0; p < 2; p++)
      for (int ic = 0; ic < g.nc; ic++) {
        const int64_t pi = (int64_t)p * g.nc + ic;
        MICSA_CK(micsa_launch_to_ref(g, p, ic, ctx->walk, sample,
                                     src[k] + ((int64_t)sample * 2 * g.nc + pi) * g.P * g.W,
                                     (direct ? dv[k] : ctx->stage) + pi * plane, ctx->stream));
        ctx->launches++;
      }
    if (!direct)
      MICSA_CK(cudaMemcpyAsync(dst[k], ctx->stage, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  return MICSA_OK;
}

int micsa_profile(micsa_ctx *ctx, int64_t n, double *sweep_ms, double *iteration_ms) {
  if (!ctx || n < 1) return fail(ctx, MICSA_ERR_ARG, "bad argument");
  int rc = set_device(ctx);
  if (rc || (rc = ready_for_sweeps(ctx, 1))) return rc;
  const micsa_geo &g = ctx->g;
  const int unit = g.flow && g.fit > 1 ? g.fit : 1;
  const int per = 2 * g.nc * unit;
  /* one launch unit (g.fit iterations of the dataflow sweep, else one) as a
   * CUDA graph, as micsa_iterate runs it, with event nodes before the
   * half-sweeps, between them and the walk, and after it; each replay is
   * read back before the next */
  cudaEvent_t ev[3];
  for (auto &e : ev) MICSA_CK(cudaEventCreate(&e));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t nl = 0;
  double sweep = 0, total = 0;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    e = cudaEventRecordWithFlags(ev[0], ctx->stream, cudaEventRecordExternal);
    if (e == cudaSuccess) e = launch_halves(ctx, g, ctx->split, 0, g.nc, &nl);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[1], ctx->stream, cudaEventRecordExternal);
    if (e == cudaSuccess)
      e = unit > 1 ? micsa_launch_walk_add(g, ctx->walk, unit, ctx->stream)
                   : micsa_launch_walk_advance(g, ctx->walk, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[2], ctx->stream, cudaEventRecordExternal);
    const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  for (int64_t it = 0; it < n && e == cudaSuccess; it++) {
    e = cudaGraphLaunch(exec, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float a = 0, b = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&a, ev[0], ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&b, ev[1], ev[2]);
    sweep += a;
    total += a + b;
  }
  ctx->launches += n * (nl + 1);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (auto &x : ev) cudaEventDestroy(x);
  MICSA_CK(e);
  if (sweep_ms) *sweep_ms = sweep / (double)(n * per);
  if (iteration_ms) *iteration_ms = total / (double)(n * unit);
  return MICSA_OK;
}

int micsa_set_active(micsa_ctx *ctx, const uint8_t *active) {
  if (!ctx) return MICSA_ERR_ARG;
  int rc = set_device(ctx);
  if (rc) return rc;
  const int ns = ctx->cfg.nsamples;
  if (!active) {
    MICSA_CK(cudaMemsetAsync(ctx->active, 1, (size_t)ns, ctx->stream));
    ctx->active_host.assign(ns, 1);
    return MICSA_OK;
  }
  std::vector<uint8_t> a(active, active + ns);
  for (auto &v : a) v = v ? 1 : 0;
  ctx->active_host = a;
  /* pageable source: returns once staged; ordered with the queued work */
  MICSA_CK(cudaMemcpyAsync(ctx->active, a.data(), (size_t)ns, cudaMemcpyHostToDevice, ctx->stream));
  return MICSA_OK;
}

int micsa_synchronize(micsa_ctx *ctx) {
  if (!ctx) return MICSA_ERR_ARG;
  int rc = set_device(ctx);
  if (rc) return rc;
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  MICSA_CK(cudaGetLastError());
  unsigned to = 0;
  MICSA_CK(micsa_tma_timeout_count(&to));
  if (to) return fail(ctx, MICSA_ERR_CUDA, "%u staged demon loads timed out (read directly)", to);
  MICSA_CK(micsa_flow_timeout_count(&to));
  if (to) {
    /* reported once: cleared so that later launches wait again */
    MICSA_CK(micsa_flow_timeout_clear());
    return fail(ctx, MICSA_ERR_CUDA,
                "%u waits of the dataflow sweep timed out: the results of that iteration are "
                "not valid", to);
  }
  return MICSA_OK;
}

int micsa_debug_flow_waits(micsa_ctx *ctx, uint64_t limit_ns, int unreachable) {
  if (!ctx) return MICSA_ERR_ARG;
  int rc = set_device(ctx);
  if (rc) return rc;
  MICSA_CK(cudaStreamSynchronize(ctx->stream));
  MICSA_CK(micsa_flow_set_waits(limit_ns ? (unsigned long long)limit_ns : 2000000000ull,
                                unreachable ? 0x40000000u : 0u, ctx->stream));
  return MICSA_OK;
}


/* ------------------------------------------------ mixed-lattice launches */
struct micsa_multi {
  std::vector<micsa_ctx *> ctx;
  int device = 0;
  cudaStream_t stream = nullptr;
  unsigned *ctl = nullptr;
  size_t ctl_words = 0;
  std::vector<int> zc, pd; /* per group */
  int occ = 6, smaj = 1;
  int spt = 1; /* 1: several samples per tile where a plane is smaller than a block */
  std::vector<int> own; /* 1: the group runs its own resident kernel beside the launch */
  int iters = 1; /* iterations per launch */
  std::vector<unsigned> graph_ns; /* ns_run of each group in the captured graphs */
  cudaGraphExec_t exec = nullptr;     /* one launch of `iters` iterations */
  std::vector<cudaGraphExec_t> rem;   /* rem[k]: one launch of k < iters iterations */
  int64_t graph_kernels = 0, launches = 0;
  cudaEvent_t done = nullptr;
  std::vector<cudaEvent_t> ev;
  int cached = 0, tuned = 0;
  std::string table; /* candidates timed */
  char err[512] = {0};
};

namespace {

int mfail(micsa_multi *m, int code, const char *fmt, ...) {
  if (m) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(m->err, sizeof m->err, fmt, ap);
    va_end(ap);
  }
  return code;
}
#define MULTI_CK(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return mfail(m, MICSA_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                   __FILE__, __LINE__);                                                \
  } while (0)

/* the slab depth a group starts from: deep slabs at large L, more tiles at
 * small L (every candidate divides L) */
int multi_default_zc(int L) { return L % 8 == 0 && L >= 32 ? 8 : (L % 4 == 0 ? 4 : 2); }

/* launch arguments for the groups' running prefixes ns[g] (0: the group
 * takes no tickets) */
int multi_args(micsa_multi *m, const std::vector<unsigned> &ns, unsigned iters,
               micsa_multi_args *a) {
  memset(a, 0, sizeof *a);
  a->smaj = m->smaj;
  a->iters = iters;
  unsigned first = 0, cnt = 0;
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    if (!ns[gi]) continue;
    const micsa_ctx *c = m->ctx[gi];
    micsa_mgroup &x = a->gr[a->n++];
    x.g = c->g;
    x.spin = c->spin;
    x.d0 = c->dem0;
    x.d1 = c->dem1;
    x.jb = c->jb;
    x.walk = c->walk;
    x.zc = m->zc[gi];
    x.pd = m->pd[gi] < m->zc[gi] ? m->pd[gi] : 0;
    x.nslab = (unsigned)(c->g.L / x.zc);
    const int VW = c->g.W % 4 == 0 ? 4 : (c->g.W % 2 == 0 ? 2 : 1);
    x.G = (unsigned)(c->g.W / VW);
    const uint64_t units = (uint64_t)c->g.L * (c->g.Lh / 2) * x.G; /* per sample and plane */
    x.spt = units < (uint64_t)MTPB && m->spt ? (unsigned)(MTPB / units) : 1u;
    x.ns_run = ns[gi];
    x.nsg = (ns[gi] + x.spt - 1) / x.spt;
    x.T = (unsigned)((units * x.spt + MTPB - 1) / MTPB);
    x.first = first;
    x.cnt_off = cnt;
    const uint64_t t = (uint64_t)x.nsg * iters * 2 * c->g.nc * x.nslab * x.T;
    if (first + t >= (1ull << 31)) return mfail(m, MICSA_ERR_UNSUPPORTED, "more than 2^31 tiles");
    first += (unsigned)t;
    cnt += x.nsg * x.nslab;
  }
  a->total = first;
  a->ncnt = cnt;
  if (4 + (size_t)cnt > m->ctl_words) return mfail(m, MICSA_ERR_STATE, "counter space");
  return MICSA_OK;
}

/* one launch of k iterations of the groups' running prefixes, as a graph */
int multi_graph(micsa_multi *m, const std::vector<unsigned> &ns, unsigned k,
                cudaGraphExec_t *exec) {
  micsa_multi_args a;
  int rc = multi_args(m, ns, k, &a);
  if (rc) return rc;
  *exec = nullptr;
  if (!a.n) return MICSA_OK;
  MULTI_CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  const cudaError_t le = micsa_launch_sweep_multi(a, m->occ, m->ctl, m->stream);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
  if (le != cudaSuccess || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return mfail(m, MICSA_ERR_CUDA, "capture of the mixed launch: %s",
                 cudaGetErrorString(le != cudaSuccess ? le : ce));
  }
  const cudaError_t ie = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  MULTI_CK(ie);
  return MICSA_OK;
}

void multi_drop_graphs(micsa_multi *m) {
  if (m->exec) cudaGraphExecDestroy(m->exec);
  for (cudaGraphExec_t &e : m->rem)
    if (e) cudaGraphExecDestroy(e);
  m->exec = nullptr;
  m->rem.clear();
  m->graph_ns.clear();
}

/* the graph of m->iters iterations for the running prefixes ns (the
 * remainders' graphs are made when first needed) */
int multi_capture(micsa_multi *m, const std::vector<unsigned> &ns) {
  multi_drop_graphs(m);
  int rc = multi_graph(m, ns, (unsigned)m->iters, &m->exec);
  if (rc) return rc;
  m->rem.assign((size_t)m->iters, nullptr);
  m->graph_ns = ns;
  bool any = false;
  for (unsigned v : ns) any |= v > 0;
  m->graph_kernels = any ? 2 : 0;
  return MICSA_OK;
}

std::vector<unsigned> multi_running(const micsa_multi *m) {
  std::vector<unsigned> ns(m->ctx.size(), 0);
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    if (m->own[gi]) continue; /* not in the launch */
    const std::vector<uint8_t> &on = m->ctx[gi]->active_host;
    for (int s = (int)on.size() - 1; s >= 0; s--)
      if (on[s]) {
        ns[gi] = (unsigned)s + 1;
        break;
      }
  }
  return ns;
}

/* mean ms of one iteration of all groups, the current shape */
int multi_time(micsa_multi *m, double *ms) {
  std::vector<unsigned> all(m->ctx.size());
  bool any = false;
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    all[gi] = m->own[gi] ? 0u : (unsigned)m->ctx[gi]->cfg.nsamples;
    any |= all[gi] > 0;
  }
  if (!any) return *ms = 0, MICSA_OK;
  int rc = multi_capture(m, all);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  MULTI_CK(cudaEventCreate(&e0));
  MULTI_CK(cudaEventCreate(&e1));
  const int reps = m->iters >= 8 ? 2 : (m->iters >= 4 ? 3 : 6);
  for (int i = 0; i < 2; i++) MULTI_CK(cudaGraphLaunch(m->exec, m->stream));
  MULTI_CK(cudaEventRecord(e0, m->stream));
  for (int i = 0; i < reps; i++) MULTI_CK(cudaGraphLaunch(m->exec, m->stream));
  MULTI_CK(cudaEventRecord(e1, m->stream));
  MULTI_CK(cudaEventSynchronize(e1));
  float t = 0;
  MULTI_CK(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t / (reps * m->iters); /* per iteration */
  return MICSA_OK;
}

struct multi_tune_entry {
  std::vector<int> zc, pd;
  int occ, smaj, spt, iters;
  std::string table;
};
std::mutex multi_mu;
std::map<std::vector<int>, multi_tune_entry> multi_cache;

/* Shape of the mixed launch, by coordinate descent on whole-iteration
 * timings (graph replays on the contexts' zeroed buffers): the register
 * budget and ticket order first, then each group's slab depth and L2
 * prefetch distance with the others held.  Kept per process by the list of
 * (device, L, nr, samples, nc) of the groups. */
int multi_tune(micsa_multi *m) {
  std::vector<int> key = {m->device};
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    const micsa_ctx *c = m->ctx[gi];
    key.push_back(c->g.L);
    key.push_back(c->cfg.nr);
    key.push_back(c->cfg.nsamples);
    key.push_back(c->g.nc);
    key.push_back(m->own[gi]);
  }
  const char *ec = getenv("MICSA_TUNE_CACHE");
  const bool use_cache = !(ec && atoi(ec) == 0);
  if (use_cache) {
    std::lock_guard<std::mutex> lk(multi_mu);
    auto it = multi_cache.find(key);
    if (it != multi_cache.end()) {
      m->zc = it->second.zc;
      m->pd = it->second.pd;
      m->occ = it->second.occ;
      m->smaj = it->second.smaj;
      m->spt = it->second.spt;
      m->iters = it->second.iters;
      m->table = it->second.table;
      m->cached = 1;
      return MICSA_OK;
    }
  }
  char buf[96];
  double best = 1e30, ms = 0;
  int rc;
  auto trial = [&](const char *what) -> int {
    if ((rc = multi_time(m, &ms))) return rc;
    snprintf(buf, sizeof buf, "%s:%.4fms ", what, ms);
    m->table += buf;
    return MICSA_OK;
  };
  if ((rc = trial("start"))) return rc;
  best = ms;
  const int occs[3] = {6, 5, 8};
  int bo = m->occ;
  const int W = m->ctx[0]->g.W;
  for (int o : occs) {
    if (o == m->occ || (o == 5 && W != 2)) continue;
    m->occ = o;
    snprintf(buf, sizeof buf, "occ=%d", o);
    if ((rc = trial(buf))) return rc;
    if (ms < best) best = ms, bo = o;
  }
  m->occ = bo;
  m->smaj ^= 1;
  if ((rc = trial(m->smaj ? "smaj=1" : "smaj=0"))) return rc;
  if (ms < best) best = ms;
  else m->smaj ^= 1;
  m->spt ^= 1;
  if ((rc = trial(m->spt ? "spt=1" : "spt=0"))) return rc;
  if (ms < best) best = ms;
  else m->spt ^= 1;
  {
    int bi = m->iters;
    for (int k : {4, 16}) {
      m->iters = k;
      snprintf(buf, sizeof buf, "iters=%d", k);
      if ((rc = trial(buf))) return rc;
      if (ms < best) best = ms, bi = k;
    }
    m->iters = bi;
  }
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    if (m->own[gi]) continue;
    const int L = m->ctx[gi]->g.L;
    int zs[8];
    const int nz = micsa_sweep_zc_candidates(L, zs, 8);
    int bz = m->zc[gi], bp = m->pd[gi];
    for (int k = 0; k < nz; k++) {
      if (zs[k] > 16 || L / zs[k] < 1) continue;
      for (int pdv : {0, 2}) {
        if ((zs[k] == bz && pdv == bp) || (pdv && zs[k] <= pdv)) continue;
        m->zc[gi] = zs[k];
        m->pd[gi] = pdv;
        snprintf(buf, sizeof buf, "L%d/zc=%d/pd=%d", L, zs[k], pdv);
        if ((rc = trial(buf))) return rc;
        if (ms < best) best = ms, bz = zs[k], bp = pdv;
      }
    }
    m->zc[gi] = bz;
    m->pd[gi] = bp;
  }
  m->tuned = 1;
  /* the timing ran iterations on the zeroed buffers: zero them again */
  for (micsa_ctx *c : m->ctx) {
    const micsa_geo &g = c->g;
    const size_t sw = (size_t)c->cfg.nsamples * 2 * g.P * g.W;
    const size_t dw = (size_t)c->cfg.nsamples * 2 * g.nc * g.P * g.W;
    MULTI_CK(cudaMemsetAsync(c->spin, 0, 4 * sw, m->stream));
    MULTI_CK(cudaMemsetAsync(c->dem0, 0, 4 * dw, m->stream));
    MULTI_CK(cudaMemsetAsync(c->dem1, 0, 4 * dw, m->stream));
    MULTI_CK(cudaMemsetAsync(c->walk, 0, sizeof(int) * c->cfg.nsamples, m->stream));
  }
  MULTI_CK(cudaStreamSynchronize(m->stream));
  if (use_cache) {
    multi_tune_entry t{m->zc, m->pd, m->occ, m->smaj, m->spt, m->iters, m->table};
    std::lock_guard<std::mutex> lk(multi_mu);
    multi_cache.emplace(key, std::move(t));
  }
  return MICSA_OK;
}

}  // namespace

namespace {
int multi_setup(micsa_multi *m, micsa_ctx *const *ctxs, int n);
}

int micsa_multi_create(micsa_ctx *const *ctxs, int n, micsa_multi **out, char *err,
                       size_t errlen) {
  if (err && errlen) err[0] = 0;
  if (!out) return MICSA_ERR_ARG;
  *out = nullptr;
  if (!ctxs || n < 1 || n > MICSA_MULTI_MAX) {
    if (err) snprintf(err, errlen, "need 1 to %d contexts, got %d", MICSA_MULTI_MAX, n);
    return MICSA_ERR_ARG;
  }
  micsa_multi *m = new (std::nothrow) micsa_multi;
  if (!m) return MICSA_ERR_NOMEM;
  const int rc = multi_setup(m, ctxs, n);
  if (rc) {
    if (err) snprintf(err, errlen, "%s", m->err);
    micsa_multi_destroy(m);
    return rc;
  }
  *out = m;
  return MICSA_OK;
}

namespace {
int multi_setup(micsa_multi *m, micsa_ctx *const *ctxs, int n) {
  bool fresh = true;
  size_t words = 4;
  for (int i = 0; i < n; i++) {
    micsa_ctx *c = ctxs[i];
    if (!c) return mfail(m, MICSA_ERR_ARG, "context %d is NULL", i);
    for (int k = 0; k < i; k++)
      if (ctxs[k] == c) return mfail(m, MICSA_ERR_ARG, "context %d given twice", i);
    if (c->cfg.device != ctxs[0]->cfg.device)
      return mfail(m, MICSA_ERR_ARG, "contexts on different devices");
    if (c->g.W != ctxs[0]->g.W)
      return mfail(m, MICSA_ERR_UNSUPPORTED, "contexts with different replica words (nr %d, %d)",
                   ctxs[0]->cfg.nr, c->cfg.nr);
    m->ctx.push_back(c);
    m->zc.push_back(multi_default_zc(c->g.L));
    m->pd.push_back(0);
    /* a context whose samples fit one block's shared memory keeps its
     * resident kernel (whole iterations per launch, HBM touched only at the
     * ends) and runs it beside the mixed launch; MICSA_MULTI_RESIDENT=0 puts
     * it in the launch as well */
    const char *er = getenv("MICSA_MULTI_RESIDENT");
    m->own.push_back(c->resident && !(er && atoi(er) == 0) ? 1 : 0);
    words += (size_t)c->cfg.nsamples * c->g.L; /* slabs of depth >= 1 */
    for (int s = 0; s < c->cfg.nsamples; s++)
      if (c->have_spin[s] || c->have_dem[s]) fresh = false;
  }
  m->device = ctxs[0]->cfg.device;
  MULTI_CK(cudaSetDevice(m->device));
  int least = 0, greatest = 0;
  MULTI_CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  MULTI_CK(cudaStreamCreateWithPriority(&m->stream, cudaStreamNonBlocking, greatest));
  MULTI_CK(cudaMalloc(&m->ctl, 4 * words));
  m->ctl_words = words;
  MULTI_CK(cudaMemsetAsync(m->ctl, 0, 4 * words, m->stream));
  MULTI_CK(cudaEventCreateWithFlags(&m->done, cudaEventDisableTiming));
  m->ev.resize(n);
  for (int i = 0; i < n; i++) MULTI_CK(cudaEventCreateWithFlags(&m->ev[i], cudaEventDisableTiming));
  for (micsa_ctx *c : m->ctx) MULTI_CK(cudaStreamSynchronize(c->stream));
  /* the shape is timed on buffers that hold no state yet; with state
   * uploaded already, the defaults stand (the timing would advance it) */
  if (const char *e = getenv("MICSA_MULTI_ITERS")) {
    const int k = atoi(e);
    if (k >= 1 && k <= 64) m->iters = k;
  }
  if (const char *e = getenv("MICSA_MULTI_ZC")) {
    const int z = atoi(e);
    for (size_t gi = 0; gi < m->ctx.size(); gi++)
      if (z > 0 && m->ctx[gi]->g.L % z == 0) m->zc[gi] = z;
  } else if (fresh) {
    int rc = multi_tune(m);
    if (rc) return rc;
  }
  m->graph_ns.clear();
  return MICSA_OK;
}
}  // namespace

int micsa_multi_destroy(micsa_multi *m) {
  if (!m) return MICSA_OK;
  if (m->stream) {
    cudaSetDevice(m->device);
    cudaStreamSynchronize(m->stream);
  }
  multi_drop_graphs(m);
  if (m->ctl) cudaFree(m->ctl);
  if (m->done) cudaEventDestroy(m->done);
  for (cudaEvent_t e : m->ev)
    if (e) cudaEventDestroy(e);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return MICSA_OK;
}

const char *micsa_multi_last_error(const micsa_multi *m) { return m ? m->err : "null handle"; }

int micsa_multi_iterate(micsa_multi *m, int64_t n) {
  if (!m || n < 0) return mfail(m, MICSA_ERR_ARG, "bad argument");
  MULTI_CK(cudaSetDevice(m->device));
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    micsa_ctx *c = m->ctx[gi];
    if (ready_for_sweeps(c, 1)) return mfail(m, MICSA_ERR_STATE, "group %zu: %s", gi, c->err);
  }
  if (n == 0) return MICSA_OK;
  for (size_t gi = 0; gi < m->ctx.size(); gi++)
    if (m->own[gi]) {
      micsa_ctx *c = m->ctx[gi];
      bool on = false;
      for (uint8_t v : c->active_host) on |= v != 0;
      if (on && micsa_iterate(c, n))
        return mfail(m, MICSA_ERR_CUDA, "group %zu: %s", gi, c->err);
    }
  const std::vector<unsigned> ns = multi_running(m);
  bool any = false;
  for (unsigned v : ns) any |= v > 0;
  if (!any) return MICSA_OK;
  if (!m->exec || ns != m->graph_ns) {
    const int rc = multi_capture(m, ns);
    if (rc) return rc;
  }
  /* ordered after the work queued on every group's stream, and before what
   * is queued there next */
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    if (m->own[gi]) continue;
    MULTI_CK(cudaEventRecord(m->ev[gi], m->ctx[gi]->stream));
    MULTI_CK(cudaStreamWaitEvent(m->stream, m->ev[gi], 0));
  }
  const int64_t whole = n / m->iters, left = n % m->iters;
  for (int64_t i = 0; i < whole; i++) MULTI_CK(cudaGraphLaunch(m->exec, m->stream));
  if (left) {
    if (!m->rem[(size_t)left]) {
      const int rc = multi_graph(m, ns, (unsigned)left, &m->rem[(size_t)left]);
      if (rc) return rc;
    }
    MULTI_CK(cudaGraphLaunch(m->rem[(size_t)left], m->stream));
  }
  m->launches += (whole + (left ? 1 : 0)) * m->graph_kernels;
  MULTI_CK(cudaEventRecord(m->done, m->stream));
  for (size_t gi = 0; gi < m->ctx.size(); gi++)
    if (!m->own[gi]) MULTI_CK(cudaStreamWaitEvent(m->ctx[gi]->stream, m->done, 0));
  return MICSA_OK;
}

int micsa_multi_synchronize(micsa_multi *m) {
  if (!m) return MICSA_ERR_ARG;
  MULTI_CK(cudaSetDevice(m->device));
  MULTI_CK(cudaStreamSynchronize(m->stream));
  for (size_t gi = 0; gi < m->ctx.size(); gi++)
    if (m->own[gi]) MULTI_CK(cudaStreamSynchronize(m->ctx[gi]->stream));
  MULTI_CK(cudaGetLastError());
  unsigned to = 0;
  MULTI_CK(micsa_flow_timeout_count(&to));
  if (to) {
    MULTI_CK(micsa_flow_timeout_clear());
    return mfail(m, MICSA_ERR_CUDA, "%u waits of the mixed dataflow sweep timed out", to);
  }
  return MICSA_OK;
}

int64_t micsa_multi_kernel_launches(const micsa_multi *m) { return m ? m->launches : 0; }

int micsa_multi_report(const micsa_multi *m, char *buf, size_t n) {
  if (!m || !buf || !n) return MICSA_ERR_ARG;
  std::string s;
  char t[96];
  snprintf(t, sizeof t, "occ=%d smaj=%d spt=%d iters=%d%s |", m->occ, m->smaj, m->spt,
           m->iters, m->cached ? " cached" : "");
  s += t;
  for (size_t gi = 0; gi < m->ctx.size(); gi++) {
    if (m->own[gi])
      snprintf(t, sizeof t, " L%d:resident", m->ctx[gi]->g.L);
    else
      snprintf(t, sizeof t, " L%d:zc=%d,pd=%d", m->ctx[gi]->g.L, m->zc[gi], m->pd[gi]);
    s += t;
  }
  s += " | ";
  s += m->table;
  snprintf(buf, n, "%s", s.c_str());
  return MICSA_OK;
}

}  // extern "C"
