/*
 * Device layout and kernel launchers of libmicsa.
 *
 * Device layout (one sample s; all arrays 32-bit words):
 *   colour     p = (x + y + z) & 1; a colour holds P = L*L*L/2 sites
 *   site index i = (z*L + y)*Lh + (x >> 1),  Lh = L/2
 *   replica    r lives in word r/32, bit r%32; W = nr/32 words per site
 *   spin       spin[((s*2 + p)*P + i)*W + w]
 *   demons     d0/d1[(((s*2 + p)*nc + ic)*P + i)*W + w]   (D = d0 + 2*d1)
 *   couplings  jb[(s*2 + p)*P + i]: bit d = coupling of the bond from the
 *              site in direction d = +x,+y,+z,-x,-y,-z
 *   walk       walk[s] = k: demon plane (p, ic) of sample s is stored
 *              translated; the demon of site x sits at x - sgn*2k*e_axis,
 *              axis = ic%3, sgn = +1 when (p == 0) == (ic < 3), else -1.
 * The reference's demon walk (main.cu:1084-1193) moves, per iteration, the
 * colour-0 demons of plane ic by +2 e_ic and the colour-1 demons by -2 e_ic
 * (e_3..e_5 = -e_0..-e_2), so keeping k instead of moving data is exact.
 */
#ifndef MICSA_KERNELS_CUH
#define MICSA_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

struct micsa_geo {
  int L, Lh, W, nc, ns, nr;
  int64_t P;  /* sites per colour */
  int64_t H;  /* reference words per colour, (L/4)^3/2 */
  int zc;     /* z planes per thread in the sweeps (divides L; 0 = default) */
  int pd;     /* L2 prefetch distance of the demon stream, in z steps (0 = off) */
  int occ;    /* sweep register budget in blocks per SM: 4 = cap for 4 blocks, 3 = the
                 default (the pipelined variant: 3 or 2) */
  int tma;    /* 1: the sweep stages its demon tiles in shared memory by TMA */
  int async;  /* 1: the sweep double-buffers each step's operands with cp.async (W = 2) */
  int pipe;   /* 1: the sweep loads each z step's operands into registers one step ahead */
  int pdl;    /* 1: sweeps launched with programmatic dependent launch */
  int tw;     /* 1: sweep blocks span whole rows along x (when that differs) */
  int flow;   /* 1: an iteration's half-sweeps run as one dataflow launch */
  int quad;   /* 1: four one-word sites per sweep thread (W = 1, direct loads) */
  int pf;     /* dataflow sweep: demon planes of its tile requested into L2 before its
                 dependency wait (0 = none) */
  int fit;    /* dataflow sweep: iterations carried by one launch (>= 1) */
  int pers;   /* 1: the dataflow sweep in its persistent form (blocks loop over tickets) */
  int half;   /* 1: the dataflow sweep with half-height tiles (blocks of about 128
                 threads, twice as many per SM) */
  int xs;     /* 1: the dataflow sweep takes the remaining x-neighbour word from the
                 adjacent lane by warp shuffle instead of loading it */
  int s0;     /* context index of this launch's first sample (per-sample launches) */
  const uint8_t *active; /* device flags [ns]: 0 = sample frozen (skipped by the
                            sweeps, the walk and the measurements); null = all */
};

__host__ __device__ inline bool micsa_frozen(const micsa_geo &g, int s) {
  return g.active && !g.active[s];
}

/* Tensor maps of the two demon arrays for the TMA-staged sweep: each array
 * seen as [planes (s, p, ic, z)][y][x/2 * W] 32-bit words; box = the demon
 * tile of one block in one z plane (box_w words x ty rows).  Opaque storage
 * for two CUtensorMap objects. */
struct micsa_tma {
  alignas(64) unsigned char map[2][128];
  int box_w, ty;
  int ok; /* built */
};
/* Build the maps for the context's demon arrays (0 when this L, W or the
 * driver does not allow the staged sweep: then ok = 0). */
cudaError_t micsa_make_tma(const micsa_geo &g, const uint32_t *d0, const uint32_t *d1,
                           micsa_tma *out);

/* waits of the staged sweep that ran out since the process started (0 unless
 * a TMA copy never completed; the sweep then read the words directly) */
cudaError_t micsa_tma_timeout_count(unsigned *n);

/* 1 if whole-row sweep blocks (micsa_geo.tw) differ from the default shape
 * at this L, with 2 or 4 sites per thread */
int micsa_sweep_wide_differs(int L, int sites = 2);

/* slab depths the sweep can use for this L (divisors of L, ascending) */
int micsa_sweep_zc_candidates(int L, int *out, int max);

/* flag = 1 half-sweep of colour p on demon plane ic, all samples; with
 * g.tma and tm->ok the demon tiles are staged by TMA */
cudaError_t micsa_launch_sweep_micsa(const micsa_geo &g, int p, int ic,
                                     uint32_t *spin, uint32_t *d0, uint32_t *d1,
                                     const uint8_t *jb, const int *walk,
                                     const micsa_tma *tm, cudaStream_t st);
/* flag = 1: all 2*nc half-sweeps of g.fit (>= 1) iterations of every sample
 * in one launch (dataflow sweep, one block per tile), tiles taken
 * sample-major or half-sweep-major; the demon walks are not advanced (the
 * caller adds g.fit afterwards); ctl = 4 + ns*L zeroed words of the context,
 * left zeroed by the launch */
cudaError_t micsa_launch_sweep_flow(const micsa_geo &g, int sample_major, uint32_t *spin,
                                    uint32_t *d0, uint32_t *d1, const uint8_t *jb,
                                    const int *walk, unsigned *ctl, cudaStream_t st);
/* Mixed-lattice dataflow sweep: one launch advances every running sample of
 * up to MICSA_MULTI_MAX groups (contexts, possibly of different L, same W)
 * by one iteration, then their demon walks.  Block of MTPB threads over
 * consecutive (word group, row, x/2 pair) units of a slab. */
#define MICSA_MULTI_MAX 16
constexpr int MTPB = 128;
struct micsa_mgroup {
  micsa_geo g;               /* the group's geometry (active flags included) */
  uint32_t *spin, *d0, *d1;  /* the group's device state */
  const uint8_t *jb;
  int *walk;
  unsigned first;            /* first ticket of the group */
  unsigned ns_run;           /* samples [0, ns_run) take tickets */
  unsigned spt;              /* samples per tile (small lattices: several per block) */
  unsigned nsg;              /* sample groups of spt samples covering [0, ns_run) */
  unsigned cnt_off;          /* the group's [nsg][nslab] counters start at ctl[4 + cnt_off] */
  unsigned nslab, T;         /* slabs (L/zc) and tiles per slab and sample group */
  unsigned G;                /* word groups per site, W / VW */
  int zc, pd;                /* slab depth, L2 prefetch distance */
};
struct micsa_multi_args {
  int n;                     /* groups */
  int smaj;                  /* 1: tickets sample-major within a group, 0: half-sweep-major */
  unsigned iters;            /* iterations carried by one launch (then the walks advance by it) */
  unsigned total;            /* tickets = blocks */
  unsigned ncnt;             /* counter words after the 4 header words */
  micsa_mgroup gr[MICSA_MULTI_MAX];
};
/* occ: blocks per SM the registers are budgeted for: 8 (64 registers), 5
 * (96, two-word sites only) or 6 (80, the default) */
cudaError_t micsa_launch_sweep_multi(const micsa_multi_args &a, int occ, unsigned *ctl,
                                     cudaStream_t st);
/* waits of the dataflow sweep that ran out since the process started */
cudaError_t micsa_flow_timeout_count(unsigned *n);
cudaError_t micsa_flow_timeout_clear();
/* dataflow wait limit and target offset (0 in operation), see micsa_debug_flow_waits */
cudaError_t micsa_flow_set_waits(unsigned long long limit_ns, unsigned need_offset,
                                 cudaStream_t st);
/* flag = 0 half-sweep of colour p with random words rnd[(k*P + i)*W + w] */
cudaError_t micsa_launch_sweep_metropolis(const micsa_geo &g, int p,
                                          uint32_t *spin, const uint8_t *jb,
                                          const uint32_t *rnd, cudaStream_t st);
/* Philox4x32-10 heat-bath words for colour p: te[r*4+k], keys[r] on device,
 * lut = 4096-byte table on device */
cudaError_t micsa_launch_gen_rnd(const micsa_geo &g, int p, const uint32_t *te,
                                 const uint32_t *keys, const uint8_t *lut,
                                 uint32_t *rnd, cudaStream_t st);
/* walk[s] = (walk[s] + 1) mod L/2 for all samples */
cudaError_t micsa_launch_walk_advance(const micsa_geo &g, int *walk,
                                      cudaStream_t st);
/* walk[s] = (walk[s] + n) mod L/2 for the running samples */
cudaError_t micsa_launch_walk_add(const micsa_geo &g, int *walk, int n, cudaStream_t st);

/* reference-layout words ref[h*nr + r] (one colour, one sample/plane) ->
 * device words dst (colour p base of that plane), demon translation k
 * (0 for spins) applied with plane index ic (ignored when k == 0) */
cudaError_t micsa_launch_from_ref(const micsa_geo &g, int p, int ic, int k,
                                  const uint64_t *ref, uint32_t *dst,
                                  cudaStream_t st);
/* reference coupling words J[(p*6 + d)*H + h] of one sample (device) ->
 * that sample's bond bytes jb[2][P] */
cudaError_t micsa_launch_couplings_from_ref(const micsa_geo &g, const uint64_t *J, uint8_t *jb,
                                            cudaStream_t st);
cudaError_t micsa_launch_to_ref(const micsa_geo &g, int p, int ic,
                                const int *walk, int sample,
                                const uint32_t *src, uint64_t *ref,
                                cudaStream_t st);

/* measurement accumulators (unsigned long long, zeroed by the caller):
 *   unsat[s*nr + r], dem[s*nr + r], qd[s*(nr/2) + k],
 *   c4d[((s*(nr/2) + k)*3 + axis)*(L/2+1) + d] */
cudaError_t micsa_launch_energy(const micsa_geo &g, const uint32_t *spin,
                                const uint8_t *jb, unsigned long long *unsat,
                                cudaStream_t st);
cudaError_t micsa_launch_demon_energy(const micsa_geo &g, const uint32_t *d0,
                                      const uint32_t *d1,
                                      unsigned long long *dem, cudaStream_t st);
cudaError_t micsa_launch_overlap(const micsa_geo &g, const uint32_t *spin,
                                 unsigned long long *qd, unsigned long long *c4d,
                                 cudaStream_t st);

/* One demon refresh of samples first .. first+count-1 drawn from the
 * streams' start records rec (grouped by warp, 120 words per stream) and
 * the segment jump tables lcg/xoq/fib of wps words per segment; writes
 * every demon word of those samples with walk translation 0. */
cudaError_t micsa_launch_refresh(const micsa_geo &g, int first, int count, int64_t nwords,
                                 int wps, int64_t nseg, const uint64_t *rec,
                                 const uint64_t *lcg, const uint64_t *xoq,
                                 const uint64_t *fib, const uint64_t thr[3],
                                 uint32_t *dem0, uint32_t *dem1, cudaStream_t st);

/* Shared-memory bytes of the resident small-lattice kernel for this L and
 * nc (0: L not supported by it), and its launch: n whole iterations of all
 * samples, walk counters advanced by n. */
size_t micsa_resident_smem(int L, int nc);
cudaError_t micsa_launch_resident(const micsa_geo &g, int n, uint32_t *spin, uint32_t *d0,
                                  uint32_t *d1, const uint8_t *jb, int *walk, cudaStream_t st);

#endif
