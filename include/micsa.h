/*
 * micsa.h -- C ABI of libmicsa, the GB300 (sm_103a) drop-in for the
 * microcanonical simulated-annealing sweep of IsidoroGlez/micSA-EA-MC.
 *
 * The reference drives its GPU through a handful of host functions that
 * communicate via globals (PROGRAM/src/main.cu:197-543).  Each entry point
 * below replaces one of them with explicit state (a micsa_ctx), plain
 * pointers and sizes, and an int status (MICSA_OK == 0) instead of exit().
 * Buffers passed in or out use the reference's host layouts, so a caller
 * that already builds those arrays can switch without re-packing:
 *
 *   H            = (L/4)^3 / 2, words per colour of the reference MSC layout
 *   spins        even[h*nr + r], odd[h*nr + r]            (h_MSC_u_even/odd)
 *   couplings    J[(p*6 + d)*H + h], d = E,N,U,O,S,D      (viciniB/N[h].J[d])
 *   demons       w[((p*nc + ic)*H + h)*nr + r]            (CPUwalker0/1)
 *   LUT          4096-byte s_lut_heat_bath (header.h:113-116)
 *
 * On the device the library keeps its own layout (replicas bit-packed in
 * 32-bit words, colour-split lattice); conversion happens on the GPU.
 * Calls on one context must come from one thread at a time.  All device work
 * is issued on the context's own stream; calls that return data to the host
 * synchronise that stream.
 *
 * Environment variables the library reads (all optional):
 *   MICSA_SWEEP_ZC, MICSA_SWEEP_PD, MICSA_SWEEP_SPLIT, MICSA_SWEEP_OCC,
 *   MICSA_SWEEP_TILE, MICSA_SWEEP_TMA, MICSA_SWEEP_ASYNC, MICSA_SWEEP_PIPE,
 *   MICSA_SWEEP_FLOW, MICSA_SWEEP_QUAD   pin the sweep's launch shape at
 *                        micsa_create (meanings at micsa_tuning_report)
 *   MICSA_TUNE_CACHE=0   time every context instead of reusing the process's
 *                        choice for its shape
 *   MICSA_RESIDENT=0     keep L <= 16 on the per-half-sweep kernels
 *   MICSA_PDL=0          plain launches instead of programmatic dependent launch
 *   MICSA_REFRESH_WPS=n  segment length of the GPU demon refresh, in words
 *   MICSA_REFRESH_OCC=1  the refresh kernel without its register budget
 *   MICSA_REFRESH_AHEAD=0|1  refreshes asked for ahead: drawn in place at the
 *                        commit (0) or at once on the side stream (1); default:
 *                        in place for contexts on the dataflow sweep
 *   MICSA_FLOW_ITERS=k   iterations per dataflow launch, with a pinned shape
 *   MICSA_SWEEP_PERS=1   the dataflow sweep's persistent form, with a pinned shape
 *   MICSA_FLOW_HALF=1    half-height dataflow tiles, with a pinned shape
 *   MICSA_FLOW_XS=1      the dataflow sweep takes the remaining x-neighbour word
 *                        from the adjacent lane (warp shuffle), with a pinned shape
 *   MICSA_SWEEP_PF=n     the dataflow sweep requests n demon planes of each tile
 *                        into L2 before its dependency wait
 *   MICSA_MULTI_ZC=z     slab depth of the mixed-lattice launch (no timing)
 *   MICSA_MULTI_ITERS=k  iterations per mixed-lattice launch
 *   MICSA_MULTI_RESIDENT=0  small lattices inside the mixed launch too
 *   MICSA_BATCH=groups|multi  how micsa_run_batch runs its shape groups
 * The command-line driver micsa_run adds MICSA_REFRESH=host,
 * MICSA_HOST_THREADS=n and MICSA_OBSERVABLES=1 (see its usage comment).
 */
#ifndef MICSA_H
#define MICSA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MICSA_OK 0
#define MICSA_ERR_ARG 1         /* invalid argument or configuration */
#define MICSA_ERR_CUDA 2        /* CUDA runtime error (message via micsa_last_error) */
#define MICSA_ERR_NOMEM 3       /* host or device allocation failed */
#define MICSA_ERR_STATE 4       /* call not valid in the context's current state */
#define MICSA_ERR_UNSUPPORTED 5 /* configuration outside what this build supports */

#define MICSA_MAX_SAMPLES 4096  /* samples per context (reference: MAXNSAMPLES = 2) */

typedef struct micsa_ctx micsa_ctx;

typedef struct {
  int device;   /* CUDA device ordinal (argv[7], main.cu:39,52-59) */
  int L;        /* lattice side: multiple of 8, 8..888 (header.h:38-40; int32 energies) */
  int nr;       /* replicas per sample, multiple of 32 (header.h:17 NR) */
  int nsamples; /* samples simulated together, 1..4096 (nbits, main.cu:64) */
  int nc;       /* demons per site, 1..6 (input.in line 6; d_Walk limit main.cu:1082) */
} micsa_config;

/* Create a context and allocate its device state.
 * Replaces CopyDataOnDevice's allocations (main.cu:404-471) and mmcuda
 * (main.cu:1219-1289). */
int micsa_create(const micsa_config *cfg, micsa_ctx **out);
/* Free everything (FreeDevice, main.cu:508-528). NULL is accepted. */
int micsa_destroy(micsa_ctx *ctx);
/* Message describing the last failure on this context (never NULL). */
const char *micsa_last_error(const micsa_ctx *ctx);
/* Device bytes held by a context of this configuration (for admission). */
int64_t micsa_footprint_bytes(const micsa_config *cfg);

/* Heat-bath LUT for the Metropolis branch (CopyConstOnDevice,
 * main.cu:395-397).  bytes must be 4096. */
int micsa_set_lut(micsa_ctx *ctx, const void *lut, size_t bytes);

/* Couplings of one sample, reference layout (CopyDataOnDevice,
 * main.cu:436-455). */
int micsa_upload_couplings(micsa_ctx *ctx, int sample, const uint64_t *J);
/* Spins of one sample, reference layout (CopyDataOnDevice, main.cu:429-434). */
int micsa_upload_spins(micsa_ctx *ctx, int sample, const uint64_t *even,
                       const uint64_t *odd);
/* Demons of one sample, CPUwalker layout; resets that sample's demon walk
 * (refresh_walkers, main.cu:340-366). */
int micsa_upload_demons(micsa_ctx *ctx, int sample, const uint64_t *w0,
                        const uint64_t *w1);

/* One demon refresh drawn on the GPU: InitWalkers (ini.c:712-781) for the nr
 * replica streams of samples first .. first+count-1, written straight into
 * the device demons (the upload of refresh_walkers, main.cu:340-366), each
 * sample's demon walk reset.  prc and xo are those samples' streams,
 * [count][nr] of the reference's s_aleatorio_HQ_64bits (2080 bytes) and
 * s_xoshiro256pp (48 bytes, random_generator.h:28-44), in the state
 * InitWalkers would start from; on return they hold, byte for byte, the
 * state it leaves.  thr are get_thresholds' three thresholds
 * (ini.c:680-710).  Every demon equals the reference's draw: each stream is
 * cut into segments whose start states are reached by jump-ahead.  The
 * device work is queued on the context's stream; the call returns once the
 * caller's structs are advanced.  No counterpart in the reference, which
 * draws on host threads. */
int micsa_refresh_demons(micsa_ctx *ctx, int first, int count, void *prc, void *xo,
                         const uint64_t *thr);
/* The same refresh, returning as soon as the device work is queued: the
 * advance of the caller's structs runs on host threads meanwhile, while the
 * GPU draws and runs whatever is queued after it.  Until micsa_refresh_wait
 * returns (or the next refresh call on this context, or micsa_destroy) the
 * caller must neither read, write nor free prc and xo.  No counterpart in
 * the reference. */
int micsa_refresh_demons_async(micsa_ctx *ctx, int first, int count, void *prc, void *xo,
                               const uint64_t *thr);
int micsa_refresh_wait(micsa_ctx *ctx);
/* The next refresh drawn ahead: as micsa_refresh_demons_async, but the
 * demons go into a back buffer (allocated on first use, the size of the
 * demon planes) on a side stream, so the draw overlaps the iterations queued
 * on the context's stream -- the GPU form of the reference's background
 * InitWalkers thread (main.cu:340-377).  micsa_refresh_commit makes them
 * current (ordered after the draw and after the work already queued: a
 * device copy, and the walks of those samples reset).  One refresh may be
 * pending at a time.  A context on the dataflow sweep (large lattices, which
 * fill the GPU) instead records the draw -- its start states are taken and
 * the caller's structs advanced now, as above -- and micsa_refresh_commit
 * draws it in place on the context's stream: the two kernels side by side
 * are slower than one after the other there, and no copy is needed
 * (MICSA_REFRESH_AHEAD overrides the choice).  The demons, spins and
 * structs are the same either way.  No counterpart in the reference. */
int micsa_refresh_demons_ahead(micsa_ctx *ctx, int first, int count, void *prc, void *xo,
                               const uint64_t *thr);
int micsa_refresh_commit(micsa_ctx *ctx);

/* One iteration of Monte_Carlo (main.cu:197-313) on all samples.
 *   flag = 1: nc x (even, odd) microcanonical half-sweeps, then the demon
 *             walk.  te and keys are ignored (may be NULL).
 *   flag = 0: Metropolis even then odd half-sweep with Philox4x32-10 heat-bath
 *             bits; te holds the two counters produced by _fill_bits
 *             (fill_bits.h:47-68) for parity 0 then 1: te[(par*nr + r)*4 + k],
 *             keys[r] the per-replica Philox keys (seed_keys). */
int micsa_monte_carlo(micsa_ctx *ctx, int flag, const uint32_t *te,
                      const uint32_t *keys);
/* n microcanonical iterations back to back (flag = 1 each), replayed from a
 * CUDA graph of one iteration; at L = 8 and 16 (where a sample's state fits
 * in one block's shared memory) up to 1024 whole iterations per launch of a
 * shared-memory-resident kernel instead (MICSA_RESIDENT=0 in the environment
 * at micsa_create turns that off).  Results are identical either way.
 * Asynchronous. */
int micsa_iterate(micsa_ctx *ctx, int64_t n);

/* Measurements of every sample at the current state (Measure_Energy_Spins
 * main.cu:315-336, Measure_Energy_Clerics med.c:55-83).  Any output may be
 * NULL.  Layouts:
 *   e_spin [s*nr + r]  = sum over bonds of J s s  (h_Ener; -e_spin/V is E_s)
 *   e_demon[s*nr + r]  = sum over sites and demons of D (ener_C)
 *   q      [s*(nr/2) + k]  overlap of replicas 2k, 2k+1: sum_x s^a_x s^b_x
 *   c4     [((s*(nr/2) + k)*3 + axis)*(L/2+1) + d] = sum_x q_x q_{x + d e_axis}
 * q and c4 have no counterpart in the reference. */
int micsa_measure(micsa_ctx *ctx, int32_t *e_spin, uint64_t *e_demon,
                  int64_t *q, int64_t *c4);

/* State of one sample back in the reference layouts (copy_from_GPU_for_write,
 * main.cu:473-490).  Demons are returned in the frame of the current walk.
 * When both host buffers are page-locked and mapped (cudaHostAlloc,
 * cudaHostRegister with mapping), the conversion kernels write them directly
 * across the host link; other buffers are filled from a device staging
 * buffer.  The results are the same either way. */
int micsa_download_spins(micsa_ctx *ctx, int sample, uint64_t *even,
                         uint64_t *odd);
int micsa_download_demons(micsa_ctx *ctx, int sample, uint64_t *w0,
                          uint64_t *w1);

/* Run n microcanonical iterations, each a replay of the iteration's CUDA
 * graph (as micsa_iterate runs it) with event nodes around its half-sweeps
 * and around its walk, and report the mean device time of one half-sweep
 * (of all samples) and of one whole iteration, in milliseconds (the
 * per-kernel view of measure_time, timing.c:3-33).  Advances the state like
 * micsa_iterate. */
int micsa_profile(micsa_ctx *ctx, int64_t n, double *sweep_ms, double *iteration_ms);

/* Text line describing the launch shape the context's autotuner chose at
 * creation: "zc=<z planes per thread> pd=<L2 prefetch distance> split=<0: one
 * launch for all samples, k > 0: group-major, one launch per group of k
 * samples (1: sample-major; the tuner times 0 and 1, MICSA_SWEEP_SPLIT=k
 * pins larger groups)>
 * occ=<blocks per SM the registers are allocated for> load=<direct | tma:
 * demon tiles staged by TMA | async: operands double-buffered by cp.async |
 * pipe: each z step's loads issued one step ahead into registers |
 * flow: the iteration's half-sweeps in one dataflow launch, one block per
 * tile, ordered by per-slab dependency counters; split then orders its
 * tiles sample-major (1) or half-sweep-major (0) | pflow: the same in its
 * persistent form, as many blocks as fit the GPU, each looping over tickets
 * and taking the next during its tile | quad: direct loads with
 * four one-word sites per thread (32 replicas)>
 * tile=<default | row: blocks span whole rows along x>[/2: half-height
 * dataflow tiles]
 * fit=<iterations per launch of the dataflow sweep: its wavefront runs on
 * from one iteration into the next; 1 for the other loads> |
 * <zc>/<pd>/<split>/<occ>/<load 0|1|2|3|4|5|6 (6: pflow)>/<tile 0|1>:<ms per half-sweep> ...",
 * with " cached" before the "|" when the choice and its table were taken
 * over from an earlier context of the same device, L, nr, samples and nc in
 * this process (MICSA_TUNE_CACHE=0 times every context instead).  The
 * environment variables MICSA_SWEEP_ZC, MICSA_SWEEP_PD, MICSA_SWEEP_SPLIT,
 * MICSA_SWEEP_OCC, MICSA_SWEEP_TMA, MICSA_SWEEP_ASYNC, MICSA_SWEEP_PIPE,
 * MICSA_SWEEP_FLOW, MICSA_SWEEP_QUAD and MICSA_SWEEP_TILE (=row), read by
 * micsa_create, pin the shape and skip the timing (no candidates listed
 * then).  The dataflow sweep is timed for L >= 128 only; MICSA_SWEEP_FLOW=0
 * alone leaves it out everywhere.  The reference has fixed launch geometry
 * (calculate_blocks, ini.c:580-602). */
int micsa_tuning_report(const micsa_ctx *ctx, char *buf, size_t n);

/* Spin energies computed without allocating any device memory; this entry
 * point has no counterpart in the reference.  It is for callers that cannot
 * call cudaMalloc when they measure: processes that size their device memory
 * once at start-up (services, real-time loops), whose device memory belongs
 * to another allocator, or that must not let an allocation synchronise their
 * streams.  The caller passes the reference's own device rows through the
 * host-side pointer tables the reference keeps for them (mmcuda,
 * main.cu:1219-1289, filled by CopyDataOnDevice, main.cu:404-471), one
 * table entry per row, samples one after another:
 *   spin_rows[2*s + p]   = h_spin[s][p], p = 0 even, 1 odd: [H][nr] uint64
 *   J_rows[12*s + k]     = h_J[s][k], k = colour*6 + direction: [H] uint64
 * (host arrays of device pointers, read during the call only) and a device
 * int32 output e_spin[s*nr + r] (h_Ener of Measure_Energy_Spins,
 * main.cu:315-336).  Work is queued on `stream` (a cudaStream_t; NULL = the
 * legacy default stream).  L must be a multiple of 8 in [8, 888]: the
 * energies are int32, as the reference's h_Ener, and |E| <= 3 L^3.
 * The per-replica counters live in one fixed device array of
 * MICSA_NOALLOC_MAX_REPLICAS entries per GPU, kept until the process exits:
 * nr * nsamples above that limit is rejected with MICSA_ERR_ARG.  Every call
 * shares the array (each call zeroes the part it uses), so calls that overlap
 * on the GPU race: keep them in one stream or otherwise ordered.  Each call
 * looks up the array's address in the current device's context; the first
 * call on a device also loads the library's device code there, so make that
 * first call before any stream capture.  err (optional) receives a message
 * on failure. */
#define MICSA_NOALLOC_MAX_REPLICAS 8192
#define MICSA_NOALLOC_MAX_L 888
int micsa_energy_noalloc(int L, int nr, int nsamples, const uint64_t *const *spin_rows,
                         const uint64_t *const *J_rows, int32_t *e_spin, void *stream, char *err,
                         size_t errlen);

/* ---- Batched runs: no counterpart in the reference ----
 * A job is one reference run of one sample (nbits = 1, nterm = 0, flag 1):
 * Init (ini.c:8-32) from the job's own seeds -- spins and demon-stream seeds
 * from seed_u (Init_Random ini.c:34-60, Init_u ini.c:275-299), couplings from
 * the Janus generator seeded with seed_J (Init_J ini.c:457-471; the
 * reference's -DJANUS build fixes that seed, a batch gives each job its
 * own) -- then the main loop (main.cu:130-180): demon refresh at t = 0 and at
 * every power of two, energies measured at every power of two and at the
 * end. */
typedef struct {
  int L, nr, nc;       /* as in micsa_config */
  int64_t iterations;  /* maxtime */
  uint64_t seed_J;     /* coupling seed */
  uint64_t seed_u;     /* spin / demon-stream seed (0: drawn from /dev/urandom) */
  double beta;         /* demon temperature (beta.in) */
  double beta_end;     /* 0 or beta: constant; else the refresh at iteration t draws
                          at beta + (beta_end - beta) * t / iterations (a linear
                          schedule; the reference has one beta, NBETAS = 1) */
} micsa_job;
/* The inverse temperature a job's refresh at iteration t uses. */
double micsa_job_beta(const micsa_job *job, int64_t t);
/* Measurement points of a job: t = 1, 2, 4, ... <= iterations, plus
 * iterations itself when it is not a power of two. */
int64_t micsa_job_measurements(int64_t iterations);
/* Run njobs jobs together.  Jobs of one shape (L, nr, nc, beta) share a
 * context, one job per sample slot, longest first; each shape group runs in
 * its own context and stream on `device`, concurrently with the others.  In
 * a group one launch per half-sweep (or per 1024 iterations at L <= 16),
 * refresh and measurement serves every running job; a job whose iterations
 * are done is frozen (micsa_set_active) after its last measurement.
 * Outputs (either may be NULL), m = measurement point, nm_j =
 * micsa_job_measurements(jobs[j].iterations), off_j = sum over i < j of
 * nm_i * nr_i:
 *   e_spin [off_j + m*nr_j + r]   as micsa_measure's e_spin
 *   e_demon[off_j + m*nr_j + r]   as micsa_measure's e_demon
 * seconds (optional) receives the wall time from the first context's
 * creation to the end of the last group; host initialisation of the jobs
 * (on threads) precedes it.  Each job's numbers equal those of the same job
 * run alone.  err (optional) receives a message on failure. */
int micsa_run_batch(int device, const micsa_job *jobs, int njobs, int32_t *e_spin,
                    uint64_t *e_demon, double *seconds, char *err, size_t errlen);

/* ---- Serving: no counterpart in the reference ----
 * Anneal requests (jobs) arrive over time and are continuously batched: per
 * shape (L, nr, nc) one context of S sample slots on its own stream
 * and host thread, S chosen so that all shapes' contexts fit hbm_budget; a
 * request is initialised on host threads once it has arrived, admitted into
 * the next free slot, runs its own reference schedule (refresh at its own
 * t = 0 and powers of two, measurements at powers of two and at the end)
 * in rounds shared with the other slots, and leaves its slot to the next
 * request when done.  Results equal the job run alone (micsa_run_batch). */
typedef struct {
  double arrival;  /* seconds after the start of the run */
  micsa_job job;
} micsa_request;
typedef struct {
  double prepared, admitted, finished; /* seconds after the start; latency = finished - arrival */
} micsa_request_result;
typedef struct {
  int device;
  int64_t hbm_budget;  /* bytes all contexts may hold together (0: 48 GiB) */
  int slots_max;       /* slots per shape (0: 64) */
  int64_t chunk;       /* most iterations per round (0: 1024) */
  int prep_threads;    /* host threads initialising requests (0: cores - 1) */
} micsa_serve_config;
/* Replay n requests in real time (request j becomes visible at its arrival
 * time after the start; contexts are created before the start).  Outputs as
 * micsa_run_batch's (offsets over the requests in the given order); res[j]
 * receives the request's times; seconds (optional) the time of the last
 * finish.  A replay of the trace through a micsa_server (below). */
int micsa_serve(const micsa_serve_config *cfg, const micsa_request *req, int n,
                micsa_request_result *res, int32_t *e_spin, uint64_t *e_demon, double *seconds,
                char *err, size_t errlen);

/* A long-lived server for callers that produce requests as they go: the
 * same pools, slots and rounds as micsa_serve, fed by micsa_submit from any
 * thread.  The shapes it serves are fixed at creation (their contexts are
 * created and tuned then, sized so that all fit hbm_budget). */
typedef struct micsa_server micsa_server;
typedef struct {
  int L, nr, nc;
  int slots; /* sample slots of this shape's context (0: as many as the budget allows,
                at most slots_max) */
} micsa_pool_shape;
typedef struct {
  int device;
  int64_t hbm_budget;  /* bytes all contexts may hold together (0: 48 GiB) */
  int slots_max;       /* slots per shape (0: 64) */
  int64_t chunk;       /* most iterations per round (0: 1024) */
  int prep_threads;    /* host threads initialising requests (0: cores - 1) */
  const micsa_pool_shape *shapes;
  int nshapes;
} micsa_server_config;
int micsa_server_create(const micsa_server_config *cfg, micsa_server **out, char *err,
                        size_t errlen);
/* Queue one job; *id identifies it in micsa_poll.  MICSA_ERR_UNSUPPORTED if
 * the server has no pool of the job's shape; a pool that failed returns its
 * error for its shape from then on. */
int micsa_submit(micsa_server *sv, const micsa_job *job, int64_t *id);
/* Wait up to timeout_s seconds (0: just look) for request id.  *done = 1 when
 * it has finished: its measurements are copied out (e_spin
 * [micsa_job_measurements(iterations) * nr] and e_demon likewise, either may
 * be NULL), times (optional) receives the seconds from its submission to its
 * initialisation, admission and finish, and the id is released.  A request
 * whose pool failed returns that error (and is released).  Unknown or
 * released ids: MICSA_ERR_ARG. */
int micsa_poll(micsa_server *sv, int64_t id, double timeout_s, int *done, int32_t *e_spin,
               uint64_t *e_demon, micsa_request_result *times);
/* Let every submitted request finish, stop the threads and free the
 * contexts; results not yet polled are dropped.  NULL is accepted. */
int micsa_server_destroy(micsa_server *sv);

/* ---- Mixed-lattice launches: no counterpart in the reference ----
 * One launch per iteration advances every running sample of several
 * contexts -- of different L, with the same nr, on one device -- instead of
 * one launch sequence per context: a dataflow sweep over a device work
 * queue of (context, sample, half-sweep, slab, tile) tiles, each tile
 * ordered after the half-sweep before it on its own and the neighbouring
 * slabs, then the demon walks; replayed from a CUDA graph.  The reference
 * runs one lattice shape per executable (header.h:20, main.cu:197-313).
 * micsa_multi_create picks each context's slab depth and L2 prefetch
 * distance and the launch's register budget and ticket order by timing
 * whole iterations, which runs iterations on the contexts' buffers: create
 * it before any state is uploaded (with state present the defaults are
 * kept; MICSA_MULTI_ZC=z pins the slab depth where it divides L).  The
 * choice is kept per process for the same list of shapes.  At most 16
 * contexts.  A context whose samples fit one block's shared memory (L <= 16,
 * the resident kernel of micsa_iterate) keeps that kernel, issued on its own
 * stream beside the mixed launch (MICSA_MULTI_RESIDENT=0 puts it in the
 * launch too); a launch carries one or more iterations (timed: 1, 4 or 16;
 * MICSA_MULTI_ITERS=k pins it).  The contexts stay usable as before (uploads, refreshes,
 * measurements, run flags); micsa_multi_iterate is ordered after the work
 * queued on every context's stream and before what is queued there next.
 * Results equal micsa_iterate on each context alone.  The contexts must
 * outlive the mixed launch object (destroy it first); their sample counts and shapes
 * are fixed, their run flags (micsa_set_active) may change between calls.
 * err (optional) receives a message on failure. */
typedef struct micsa_multi micsa_multi;
int micsa_multi_create(micsa_ctx *const *ctxs, int n, micsa_multi **out, char *err,
                       size_t errlen);
/* n iterations of every running sample of every context (asynchronous);
 * samples beyond a context's last running one take no tiles. */
int micsa_multi_iterate(micsa_multi *m, int64_t n);
/* wait for the launches and report a device error or timed-out waits */
int micsa_multi_synchronize(micsa_multi *m);
int micsa_multi_destroy(micsa_multi *m);
const char *micsa_multi_last_error(const micsa_multi *m);
int64_t micsa_multi_kernel_launches(const micsa_multi *m);
/* "occ=<blocks per SM budget> smaj=<1: tiles sample-major> spt=<1: several small
 * samples per tile> iters=<per launch> [cached] | L<L>:zc=<slab
 * depth>,pd=<prefetch> ... | <candidate>:<ms per iteration> ..." */
int micsa_multi_report(const micsa_multi *m, char *buf, size_t n);

/* Per-sample run flags, active[s] != 0 = sample s runs (all, after
 * micsa_create; NULL restores that).  A frozen sample is skipped by the
 * sweeps, the demon walk and the measurements (its measured values read 0)
 * and keeps its state; uploads, downloads and refreshes still act on it.
 * Ordered with the context's queued work.  No counterpart in the reference;
 * the batched and served runs use it for finished and empty slots. */
int micsa_set_active(micsa_ctx *ctx, const uint8_t *active);

/* Wait for all work issued on the context (cudaDeviceSynchronize,
 * main.cu:144,149) and report any asynchronous error. */
int micsa_synchronize(micsa_ctx *ctx);
/* Test hook for the bounded device waits; no counterpart in the reference,
 * whose failed CUDA calls exit (cudamacro.h:1-16).  The dataflow sweep
 * (load=flow) orders its tiles by waiting on per-slab counters; each wait
 * gives up after limit_ns nanoseconds of the GPU's global timer (0: the
 * default, 2 s), after which every later wait of the launch gives up at
 * once and micsa_synchronize reports the count as MICSA_ERR_CUDA (and
 * clears it).  unreachable != 0 raises every wait's target beyond what the
 * counters reach, so that every wait runs out: the iteration then completes
 * without its ordering and its results are not valid.  The setting holds
 * for every context on the device until changed; micsa_debug_flow_waits(ctx,
 * 0, 0) restores operation.  Synchronises the context's stream. */
int micsa_debug_flow_waits(micsa_ctx *ctx, uint64_t limit_ns, int unreachable);

/* Number of kernels this context has launched so far (graph replays count
 * each kernel node). */
int64_t micsa_kernel_launches(const micsa_ctx *ctx);
/* The context's CUDA stream, as a void* (cudaStream_t). */
void *micsa_stream(micsa_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
