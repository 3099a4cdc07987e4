/*
 * Spin energies without any device allocation.
 *
 * Some callers cannot call cudaMalloc at the point where they need a
 * measurement: code that must not allocate after start-up (a long-running
 * service that sizes its memory once, a real-time loop, a process whose
 * device memory is owned by another allocator such as a framework's caching
 * pool), or code whose stream ordering must not be broken by the implicit
 * synchronisation an allocation can cause.  The measurement kernel of a
 * micsa context accumulates into counters the context allocated; this file
 * gives such callers the same energies with the counters in a fixed,
 * file-scope device array instead.  The caller owns and passes every input
 * and output buffer; nothing here allocates or frees device memory.
 *
 * The inputs are the reference's own device rows, passed as the host-side
 * tables of device pointers the reference keeps: h_spin[s][p] (two rows per
 * sample, [H][nr] words each) and h_J[s][k] (twelve rows per sample, [H]
 * words each), both filled by mmcuda and CopyDataOnDevice
 * (PROGRAM/src/main.cu:404-471,1219-1289).  The row pointers travel to the
 * kernel by value, a chunk of samples per launch, so no table is copied to
 * the device.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "micsa.h"

/* Per-replica counters of unsatisfied bonds, shared by every call on a
 * device; each call clears the part it uses before counting. */
static __device__ __align__(256) unsigned long long micsa_noalloc_counters[MICSA_NOALLOC_MAX_REPLICAS];

namespace {

constexpr int ROWS_PER_LAUNCH = 16; /* samples whose row pointers one launch carries */

struct sample_rows {
  const uint64_t *spin[ROWS_PER_LAUNCH][2];
  const uint64_t *J[ROWS_PER_LAUNCH][12];
};

/* block-edge rotations of the reference words (main.cu:706-742) */
__device__ __forceinline__ uint64_t rot_dir(int d, uint64_t v) {
  switch (d) {
    case 0: { const uint64_t m = 0x1111111111111111ULL; return ((v & m) << 3) | ((v & ~m) >> 1); }
    case 1: { const uint64_t m = 0x000F000F000F000FULL; return ((v & m) << 12) | ((v & ~m) >> 4); }
    case 2: { const uint64_t m = 0x000000000000FFFFULL; return ((v & m) << 48) | ((v & ~m) >> 16); }
    case 3: { const uint64_t m = 0x8888888888888888ULL; return ((v & m) >> 3) | ((v & ~m) << 1); }
    case 4: { const uint64_t m = 0xF000F000F000F000ULL; return ((v & m) >> 12) | ((v & ~m) << 4); }
    default: { const uint64_t m = 0xFFFF000000000000ULL; return ((v & m) >> 48) | ((v & ~m) << 16); }
  }
}

/* Unsatisfied bonds of the colour-0 words, per replica (the counting of
 * d_computeEne, main.cu:745-815, on the reference layout).  Thread = replica
 * r and a stride of words h; blockIdx.y = sample within this launch's chunk.
 * Each word holds 64 sites of one replica, so a popcount is already a
 * per-replica count. */
__global__ void k_energy_ref(int L, int nr, const sample_rows rows,
                             unsigned long long *__restrict__ counters) {
  const int s = blockIdx.y;
  const int m = L / 4, mh = m / 2;
  const int64_t H = (int64_t)m * m * m / 2;
  const uint64_t *__restrict__ ev = rows.spin[s][0];
  const uint64_t *__restrict__ od = rows.spin[s][1];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = (int)(t % nr);
  const int64_t chunks = ((int64_t)gridDim.x * blockDim.x) / nr;
  if (t >= chunks * nr) return;
  unsigned long long un = 0;
  for (int64_t h = t / nr; h < H; h += chunks) {
    const int a2 = (int)(h % mh), b = (int)((h / mh) % m), c = (int)(h / ((int64_t)mh * m));
    const int a = 2 * a2 + ((b + c) & 1);
    const int na[6] = {a == m - 1 ? 0 : a + 1, a, a, a == 0 ? m - 1 : a - 1, a, a};
    const int nb[6] = {b, b == m - 1 ? 0 : b + 1, b, b, b == 0 ? m - 1 : b - 1, b};
    const int nc[6] = {c, c, c == m - 1 ? 0 : c + 1, c, c, c == 0 ? m - 1 : c - 1};
    const bool wrap[6] = {a == m - 1, b == m - 1, c == m - 1, a == 0, b == 0, c == 0};
    const uint64_t sw = ev[h * nr + r];
#pragma unroll
    for (int d = 0; d < 6; d++) {
      const int64_t nh = (na[d] + (int64_t)m * nb[d] + (int64_t)m * m * nc[d]) / 2;
      uint64_t n = od[nh * nr + r];
      const uint64_t jw = rows.J[s][d][h]; /* colour-0 rows are k = d */
      uint64_t f;
      if (d < 3) {
        if (wrap[d]) n = rot_dir(d, n);
        f = sw ^ jw ^ n;
      } else {
        n ^= jw; /* backward couplings sit at the owner's bit */
        if (wrap[d]) n = rot_dir(d, n);
        f = sw ^ n;
      }
      un += (unsigned long long)__popcll(f);
    }
  }
  atomicAdd(counters + (int64_t)s * nr + r, un);
}

__global__ void k_energy_ref_finish(int n, long long threeV,
                                    const unsigned long long *__restrict__ counters,
                                    int32_t *__restrict__ e_spin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) e_spin[i] = (int32_t)(threeV - 2LL * (long long)counters[i]);
}

}  // namespace

extern "C" int micsa_energy_noalloc(int L, int nr, int nsamples,
                                    const uint64_t *const *spin_rows,
                                    const uint64_t *const *J_rows, int32_t *e_spin,
                                    void *stream, char *err, size_t errlen) {
  if (err && errlen) err[0] = 0;
  /* 3*L^3 must fit the int32 energies (the reference's int h_Ener has the
   * same bound): L <= 888 */
  if (L < 8 || L > MICSA_NOALLOC_MAX_L || L % 8 || nr < 1 || nsamples < 1 || !spin_rows ||
      !J_rows || !e_spin) {
    if (err)
      snprintf(err, errlen,
               "invalid arguments (L=%d must be a multiple of 8 in [8, %d]; nr=%d, nsamples=%d "
               "must be positive; row tables and output must be given)",
               L, MICSA_NOALLOC_MAX_L, nr, nsamples);
    return MICSA_ERR_ARG;
  }
  if ((long long)nr * nsamples > MICSA_NOALLOC_MAX_REPLICAS) {
    if (err)
      snprintf(err, errlen, "nr*nsamples = %lld exceeds the %d counters of the no-allocation path",
               (long long)nr * nsamples, MICSA_NOALLOC_MAX_REPLICAS);
    return MICSA_ERR_ARG;
  }
  for (int i = 0; i < 2 * nsamples; i++)
    if (!spin_rows[i]) {
      if (err) snprintf(err, errlen, "spin row %d (sample %d) is NULL", i, i / 2);
      return MICSA_ERR_ARG;
    }
  for (int i = 0; i < 12 * nsamples; i++)
    if (!J_rows[i]) {
      if (err) snprintf(err, errlen, "coupling row %d (sample %d) is NULL", i, i / 12);
      return MICSA_ERR_ARG;
    }
  /* The array's device address in the current device's context, looked up
   * on every call: a lookup allocates nothing, and a cached address would
   * go stale if the caller reset the device and a new context reloaded this
   * module.  The first call on a device also loads the module there. */
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, micsa_noalloc_counters);
  if (e != cudaSuccess) {
    if (err) snprintf(err, errlen, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    return MICSA_ERR_CUDA;
  }
  unsigned long long *counters = (unsigned long long *)p;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = nr * nsamples;
  e = cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * (size_t)n, st);
  const int64_t m = L / 4, H = m * m * m / 2;
  const int64_t chunks = H < 256 ? H : 256; /* words per replica handled in parallel */
  const int tpb = 256;
  const int blocks = (int)((chunks * nr + tpb - 1) / tpb);
  for (int s0 = 0; e == cudaSuccess && s0 < nsamples; s0 += ROWS_PER_LAUNCH) {
    const int cnt = nsamples - s0 < ROWS_PER_LAUNCH ? nsamples - s0 : ROWS_PER_LAUNCH;
    sample_rows rows = {};
    for (int s = 0; s < cnt; s++) {
      rows.spin[s][0] = spin_rows[2 * (s0 + s)];
      rows.spin[s][1] = spin_rows[2 * (s0 + s) + 1];
      for (int k = 0; k < 12; k++) rows.J[s][k] = J_rows[12 * (s0 + s) + k];
    }
    k_energy_ref<<<dim3(blocks, cnt), tpb, 0, st>>>(L, nr, rows, counters + (int64_t)s0 * nr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_energy_ref_finish<<<(n + 255) / 256, 256, 0, st>>>(n, 3LL * L * L * L, counters, e_spin);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    if (err) snprintf(err, errlen, "launch: %s", cudaGetErrorString(e));
    return MICSA_ERR_CUDA;
  }
  return MICSA_OK;
}
