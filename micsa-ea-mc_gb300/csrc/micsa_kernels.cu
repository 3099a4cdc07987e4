/*
 * sm_103a kernels of libmicsa: the microcanonical (ISI) and Metropolis
 * checkerboard half-sweeps, the Philox4x32-10 heat-bath bit generator,
 * reference-layout conversion and the popcount measurements.
 * Layout and walk convention: see micsa_kernels.cuh.
 *
 * All of this is integer/bitwise work bounded by memory bandwidth: every
 * half-sweep streams one demon plane (read + write) and the spins of both
 * colours; there is no contraction for tensor cores.
 */
#include <string.h>

#include <cuda.h> /* CUtensorMap and the encode function's types (resolved at run time) */

#include "micsa_kernels.cuh"

namespace {

constexpr int TPB = 256;
constexpr unsigned FULL = 0xffffffffu;

/* ------------------------------------------------------- memory access */
/* L2 residency policies for the sweeps: the spin lattice and the coupling
 * bytes (re-read by every half-sweep) are kept with evict_last; the demon
 * planes (touched once per iteration) are streamed with evict_first. */
__device__ __forceinline__ uint64_t l2_keep() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_stream() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

/* loads/stores with an L2 cache policy: nc = read-only (non-coherent) path,
 * na = no L1 allocation (data used once), co = coherent load the compiler
 * may schedule freely (for words other blocks of the same launch write,
 * ordered by an acquire before the address is known) */
template <int VW> struct hint;
template <> struct hint<1> {
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t (&o)[1], uint64_t pol) {
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(o[0]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t (&o)[1], uint64_t pol) {
    asm("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(o[0]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t (&o)[1], uint64_t pol) {
    asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(o[0]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t (&o)[1], uint64_t pol) {
    asm volatile("ld.global.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
                 : "=r"(o[0]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void st(uint32_t *a, const uint32_t (&o)[1], uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" :: "l"(a), "r"(o[0]), "l"(pol) : "memory");
  }
};
template <> struct hint<2> {
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t (&o)[2], uint64_t pol) {
    asm("ld.global.nc.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
        : "=r"(o[0]), "=r"(o[1]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t (&o)[2], uint64_t pol) {
    asm("ld.global.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
        : "=r"(o[0]), "=r"(o[1]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t (&o)[2], uint64_t pol) {
    asm volatile("ld.global.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
                 : "=r"(o[0]), "=r"(o[1]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t (&o)[2], uint64_t pol) {
    asm volatile("ld.global.L1::no_allocate.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
                 : "=r"(o[0]), "=r"(o[1]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void st(uint32_t *a, const uint32_t (&o)[2], uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1,%2}, %3;"
                 :: "l"(a), "r"(o[0]), "r"(o[1]), "l"(pol) : "memory");
  }
};
template <> struct hint<4> {
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t (&o)[4], uint64_t pol) {
    asm("ld.global.nc.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
        : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t (&o)[4], uint64_t pol) {
    asm("ld.global.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
        : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t (&o)[4], uint64_t pol) {
    asm volatile("ld.global.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t (&o)[4], uint64_t pol) {
    asm volatile("ld.global.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]) : "l"(a), "l"(pol));
  }
  static __device__ __forceinline__ void st(uint32_t *a, const uint32_t (&o)[4], uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1,%2,%3,%4}, %5;"
                 :: "l"(a), "r"(o[0]), "r"(o[1]), "r"(o[2]), "r"(o[3]), "l"(pol) : "memory");
  }
};
__device__ __forceinline__ void prefetch_l2(const uint32_t *a) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

/* ------------------------------------------------------------ geometry */
struct site_xyz { int x, y, z; };

/* real site of the reference word (colour p, h, bit b) (ini.c:317-337) */
__device__ __forceinline__ site_xyz ref_site(const micsa_geo &g, int p, int64_t h, int b) {
  const int m = g.L >> 2, mh = m >> 1;
  const int a2 = (int)(h % mh);
  const int64_t q = h / mh;
  const int bb = (int)(q % m);
  const int c = (int)(q / m);
  const int a = 2 * a2 + ((bb + c + p) & 1);
  site_xyz s;
  s.x = (b & 3) * m + a;
  s.y = ((b >> 2) & 3) * m + bb;
  s.z = (b >> 4) * m + c;
  return s;
}

/* where the demon of site (x,y,z) is stored after k walks (header note) */
__device__ __forceinline__ int64_t demon_slot(const micsa_geo &g, int p, int ic, int k,
                                              int x, int y, int z) {
  const int L = g.L;
  const int sh = ((p == 0) == (ic < 3)) ? 2 * k : -2 * k; /* lattice units */
  const int axis = ic < 3 ? ic : ic - 3;
  if (axis == 0) { x -= sh; if (x < 0) x += L; else if (x >= L) x -= L; }
  else if (axis == 1) { y -= sh; if (y < 0) y += L; else if (y >= L) y -= L; }
  else { z -= sh; if (z < 0) z += L; else if (z >= L) z -= L; }
  return ((int64_t)z * L + y) * g.Lh + (x >> 1);
}

/* all-ones if bond bit d of the site's coupling byte is set (one signed
 * bit-field extract) */
__device__ __forceinline__ uint32_t jmask(uint32_t jb, int d) {
  uint32_t r;
  asm("bfe.s32 %0, %1, %2, 1;" : "=r"(r) : "r"(jb), "r"(d));
  return r;
}

/* three-input bitwise function by truth table (a = 0xF0, b = 0xCC, c = 0xAA) */
template <int LUT>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(d) : "r"(a), "r"(b), "r"(c), "n"(LUT));
  return d;
}
__device__ __forceinline__ uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) { return lop3<0x96>(a, b, c); }
__device__ __forceinline__ uint32_t maj3(uint32_t a, uint32_t b, uint32_t c) { return lop3<0xe8>(a, b, c); }

/* 32x32 bit transpose across a warp: lane c returns the word whose bit i is
 * bit c of lane i's input. */
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane) {
  uint32_t m = 0x0000FFFFu;
#pragma unroll
  for (int j = 16; j != 0; j >>= 1, m ^= m << j) {
    const uint32_t p = __shfl_xor_sync(FULL, x, j);
    if (lane & j)
      x ^= ((p >> j) ^ x) & m;
    else
      x ^= (((x >> j) ^ p) & m) << j;
  }
  return x;
}

/* --------------------------------------------------------------- sweeps */

/* Programmatic dependent launch: let the next grid in the stream be
 * scheduled now, then wait until the previous grid has completed and its
 * memory operations are visible (a no-op for a plain launch). */
__device__ __forceinline__ void grid_dependency_sync() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

/* Microcanonical update with demon D = D0 + 2*D1 and unsatisfied-bond
 * counts (j1 + 2*j2) + (j3 + 2*j4): accept iff 0 <= D + u - 3 <= 3, then
 * D <- D + u - 3 -- the function the reference's ISI boolean algebra
 * computes (main.cu:1037-1074), equal to it on all 64 inputs, in a
 * shorter circuit: T = D + u summed carry-save into bits s0 + 2 s1 + 4 s2
 * + 8 c3; accepted iff 3 <= T <= 6, i.e. !c3 and s2 ^ (s1 & s0); then
 * D0 = !s0 and D1 = s2 & (s0 | s1). */
__device__ __forceinline__ uint32_t isi_update(uint32_t j1, uint32_t j2, uint32_t j3,
                                               uint32_t j4, uint32_t &D0, uint32_t &D1) {
  const uint32_t s0 = xor3(D0, j1, j3), c0 = maj3(D0, j1, j3);
  const uint32_t t = xor3(D1, j2, j4), cc = maj3(D1, j2, j4);
  const uint32_t s1 = t ^ c0, s2 = lop3<0x78>(cc, t, c0), c3 = lop3<0x80>(cc, t, c0);
  const uint32_t flip = lop3<0x78>(s2, s1, s0) & ~c3;
  const uint32_t d1 = lop3<0xe0>(s2, s0, s1);
  D0 = lop3<0x3a>(flip, s0, D0); /* flip ? !s0 : D0 */
  D1 = lop3<0xca>(flip, d1, D1); /* flip ? d1 : D1 */
  return flip;
}

/* Metropolis acceptance with Bernoulli words (main.cu:945-957). */
__device__ __forceinline__ uint32_t metropolis_flip(uint32_t j1, uint32_t j2, uint32_t j3,
                                                    uint32_t j4, uint32_t b0, uint32_t b1,
                                                    uint32_t b2) {
  b1 &= b0;
  b2 &= b1;
  const uint32_t id2 = b1, id1 = (b0 ^ b1) | b2, j24 = j2 | j4;
  return (j1 & j3 & id1) | ((j24 | id2) & (j1 | j3 | id1)) | ((j2 & j4) | (j24 & id2));
}

/* Loads of 2*VW consecutive words (the same VW words of two adjacent sites). */
/* ----------------------------------------------- TMA and mbarriers */
/* transaction barriers in shared memory, bulk tensor loads (sm_90+ PTX) */
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
/* bounded wait on phase `phase`; false if the limit ran out */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase) {
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < (1 << 20); i++) {
    uint32_t done;
    asm volatile("{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2; selp.u32 %0, 1, 0, q; }"
                 : "=r"(done) : "r"(a), "r"(phase) : "memory");
    if (done) return true;
  }
  return false;
}
/* box of the 3-d tensor `map` at (x, y, z) into shared memory; completes on bar */
__device__ __forceinline__ void tma_load_3d(void *dst, const void *map, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4}], [%5];"
               ::"r"(smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
               : "memory");
}
/* waits that ran out (a TMA copy that never completed): counted, and the
 * sweep falls back to global loads for that step */
__device__ unsigned int micsa_tma_timeouts;

template <int VW> struct pair_io;
template <> struct pair_io<1> {
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t (&o)[2], uint64_t p) { hint<2>::ld_nc(a, o, p); }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t (&o)[2], uint64_t p) { hint<2>::ld_co(a, o, p); }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t (&o)[2], uint64_t p) { hint<2>::ld(a, o, p); }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t (&o)[2], uint64_t p) { hint<2>::ld_na(a, o, p); }
  static __device__ __forceinline__ void st(uint32_t *a, const uint32_t (&o)[2], uint64_t p) { hint<2>::st(a, o, p); }
};
template <> struct pair_io<2> {
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t (&o)[4], uint64_t p) { hint<4>::ld_nc(a, o, p); }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t (&o)[4], uint64_t p) { hint<4>::ld_co(a, o, p); }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t (&o)[4], uint64_t p) { hint<4>::ld(a, o, p); }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t (&o)[4], uint64_t p) { hint<4>::ld_na(a, o, p); }
  static __device__ __forceinline__ void st(uint32_t *a, const uint32_t (&o)[4], uint64_t p) { hint<4>::st(a, o, p); }
};
template <> struct pair_io<4> {
  static __device__ __forceinline__ void split(const uint32_t (&o)[8], uint32_t (&a)[4], uint32_t (&b)[4]) {
#pragma unroll
    for (int k = 0; k < 4; k++) { a[k] = o[k]; b[k] = o[4 + k]; }
  }
  static __device__ __forceinline__ void join(uint32_t (&o)[8], const uint32_t (&a)[4], const uint32_t (&b)[4]) {
#pragma unroll
    for (int k = 0; k < 4; k++) { o[k] = a[k]; o[4 + k] = b[k]; }
  }
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t (&o)[8], uint64_t p) {
    uint32_t x[4], y[4]; hint<4>::ld_nc(a, x, p); hint<4>::ld_nc(a + 4, y, p); join(o, x, y);
  }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t (&o)[8], uint64_t p) {
    uint32_t x[4], y[4]; hint<4>::ld_co(a, x, p); hint<4>::ld_co(a + 4, y, p); join(o, x, y);
  }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t (&o)[8], uint64_t p) {
    uint32_t x[4], y[4]; hint<4>::ld(a, x, p); hint<4>::ld(a + 4, y, p); join(o, x, y);
  }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t (&o)[8], uint64_t p) {
    uint32_t x[4], y[4]; hint<4>::ld_na(a, x, p); hint<4>::ld_na(a + 4, y, p); join(o, x, y);
  }
  static __device__ __forceinline__ void st(uint32_t *a, const uint32_t (&o)[8], uint64_t p) {
    uint32_t x[4], y[4]; split(o, x, y); hint<4>::st(a, x, p); hint<4>::st(a + 4, y, p);
  }
};
__device__ __forceinline__ uint32_t ld_u16_keep(const uint8_t *a, uint64_t pol) {
  uint32_t v;
  asm("ld.global.nc.L2::cache_hint.u16 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}

/* The two sites of a pair: with one word group per site (WIDE, G = 1) their
 * words are adjacent and move as one vector; otherwise they are W words
 * apart and move as two vectors. */
template <int VW, bool WIDE> struct pairs {
  static constexpr int N = 2 * VW;
  static __device__ __forceinline__ void cat(uint32_t (&o)[N], const uint32_t (&a)[VW],
                                             const uint32_t (&b)[VW]) {
#pragma unroll
    for (int k = 0; k < VW; k++) { o[k] = a[k]; o[VW + k] = b[k]; }
  }
  static __device__ __forceinline__ void cut(const uint32_t (&o)[N], uint32_t (&a)[VW],
                                             uint32_t (&b)[VW]) {
#pragma unroll
    for (int k = 0; k < VW; k++) { a[k] = o[k]; b[k] = o[VW + k]; }
  }
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t W, uint32_t (&o)[N], uint64_t p) {
    if (WIDE) { pair_io<VW>::ld_nc(a, o, p); return; }
    uint32_t x[VW], y[VW];
    hint<VW>::ld_nc(a, x, p); hint<VW>::ld_nc(a + W, y, p); cat(o, x, y);
  }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t W, uint32_t (&o)[N], uint64_t p) {
    if (WIDE) { pair_io<VW>::ld_co(a, o, p); return; }
    uint32_t x[VW], y[VW];
    hint<VW>::ld_co(a, x, p); hint<VW>::ld_co(a + W, y, p); cat(o, x, y);
  }
  /* the other colour's words: read-only in a plain half-sweep launch, written
   * by other tiles of the same launch in the dataflow sweep */
  template <bool FLOW>
  static __device__ __forceinline__ void ld_oth(const uint32_t *a, uint32_t W, uint32_t (&o)[N], uint64_t p) {
    if (FLOW) ld_co(a, W, o, p); else ld_nc(a, W, o, p);
  }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t W, uint32_t (&o)[N], uint64_t p) {
    if (WIDE) { pair_io<VW>::ld(a, o, p); return; }
    uint32_t x[VW], y[VW];
    hint<VW>::ld(a, x, p); hint<VW>::ld(a + W, y, p); cat(o, x, y);
  }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t W, uint32_t (&o)[N], uint64_t p) {
    if (WIDE) { pair_io<VW>::ld_na(a, o, p); return; }
    uint32_t x[VW], y[VW];
    hint<VW>::ld_na(a, x, p); hint<VW>::ld_na(a + W, y, p); cat(o, x, y);
  }
  static __device__ __forceinline__ void st(uint32_t *a, uint32_t W, const uint32_t (&o)[N], uint64_t p) {
    if (WIDE) { pair_io<VW>::st(a, o, p); return; }
    uint32_t x[VW], y[VW];
    cut(o, x, y); hint<VW>::st(a, x, p); hint<VW>::st(a + W, y, p);
  }
};

/* Four sites of one word each (one word group, W = 1): their words are
 * adjacent and move as one 16-byte vector. */
struct quads {
  static __device__ __forceinline__ void ld_nc(const uint32_t *a, uint32_t, uint32_t (&o)[4], uint64_t p) { hint<4>::ld_nc(a, o, p); }
  static __device__ __forceinline__ void ld_co(const uint32_t *a, uint32_t, uint32_t (&o)[4], uint64_t p) { hint<4>::ld_co(a, o, p); }
  static __device__ __forceinline__ void ld(const uint32_t *a, uint32_t, uint32_t (&o)[4], uint64_t p) { hint<4>::ld(a, o, p); }
  static __device__ __forceinline__ void ld_na(const uint32_t *a, uint32_t, uint32_t (&o)[4], uint64_t p) { hint<4>::ld_na(a, o, p); }
  static __device__ __forceinline__ void st(uint32_t *a, uint32_t, const uint32_t (&o)[4], uint64_t p) { hint<4>::st(a, o, p); }
  template <bool FLOW>
  static __device__ __forceinline__ void ld_oth(const uint32_t *a, uint32_t W, uint32_t (&o)[4], uint64_t p) {
    if (FLOW) ld_co(a, W, o, p); else ld_nc(a, W, o, p);
  }
};
/* the loader of S sites x VW words: pairs (S = 2) or quads (S = 4, VW = 1) */
template <int VW, bool WIDE, int S> struct sites_io { using type = pairs<VW, WIDE>; };
template <> struct sites_io<1, true, 4> { using type = quads; };

__device__ __forceinline__ uint32_t ld_u32_keep(const uint8_t *a, uint64_t pol) {
  uint32_t v;
  asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ uint32_t ld_na_u32(const uint32_t *a, uint64_t pol) {
  uint32_t o[1];
  hint<1>::ld_na(a, o, pol);
  return o[0];
}
__device__ __forceinline__ void st_u32(uint32_t *a, uint32_t v, uint64_t pol) {
  const uint32_t o[1] = {v};
  hint<1>::st(a, o, pol);
}

/* Half-sweep of colour p.  One thread owns two adjacent columns (x/2 = 2j,
 * 2j+1; y) of one sample, VW replica words each (group grp of G = W/VW), and
 * marches over the z chunk [z0, z0 + zc).  The two sites share their row
 * offset, so each load brings the pair: own spins, the other-colour words at
 * (2j, 2j+1) of planes z-1, z, z+1 (z-neighbours of the pair and two of its
 * four x-neighbours; kept in registers along z), the pairs at y+-1, one
 * extra other-colour word for the remaining x-neighbour, the two coupling
 * bytes and the two demon words per plane.  Block = (TX pairs along x/2) x
 * (TY rows); TX divides L/4; grid = (L/4/TX, ytiles*ns*G, L/zc).
 * With S = 4 (one word per site, W = 1) a thread owns four adjacent columns
 * (x/2 = 4j .. 4j+3) instead of two, and every load moves 16 bytes, as a
 * pair of 64-replica sites does: TX divides L/8.
 * In-plane offsets are 32-bit (P*W < 2^32 is checked at creation). */
/* One block's tile of a half-sweep: sample s, word group grp, row tile
 * `tile`, x block bx, z planes [z0, z0 + zc), demon walk kwalk.  FLOW: the
 * other colour is read through the coherent path (other tiles of the same
 * dataflow launch write it). */
/* LIN: the thread's row and x/2 pair come from the caller (tile = y,
 * bx = pair index), not from the block shape -- the mixed-lattice launch
 * maps a fixed block onto consecutive (row, pair) units of any L. */
/* UNR: the z loop unrolled UNR times (2 lets the loads of one step overlap
 * the arithmetic of the other; at 64 registers or fewer per thread the
 * second step's registers spill, and 1 is faster) */
template <int VW, bool MICSA, bool WIDE, bool TMA, bool FLOW, int S = 2, bool LIN = false,
          bool XS = false, int UNR = 2>
__device__ __forceinline__ void sweep_block(
    const micsa_geo &g, const int p, const int ic, const uint32_t s, const uint32_t grp,
    const uint32_t tile, const uint32_t bx, const uint32_t z0, const int zc, const int pd,
    const int kwalk, uint32_t *__restrict__ spin, uint32_t *__restrict__ d0,
    uint32_t *__restrict__ d1, const uint8_t *__restrict__ jb, const uint32_t *__restrict__ rnd,
    const micsa_tma &tm) {
  static_assert(S == 2 || (S == 4 && VW == 1 && WIDE && !TMA), "four sites: one word each");
  static_assert(!(LIN && TMA), "TMA staging needs the block-shaped tile");
  static_assert(!XS || (S == 2 && !LIN && !TMA), "x halo by shuffle: pairs, block-shaped tiles");
  constexpr int N = S * VW; /* words per thread and plane */
  using PR = typename sites_io<VW, WIDE, S>::type;
  const uint32_t L = g.L, Lh = g.Lh, W = g.W;
  const uint32_t y = LIN ? tile : tile * blockDim.y + threadIdx.y;
  /* XS: the lanes of this warp that stay (rows inside the lattice) */
  unsigned xs_mask = 0;
  if (XS) {
    const unsigned lin = threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned in_warp = blockDim.x * blockDim.y - (lin & ~31u);
    xs_mask = __ballot_sync(in_warp >= 32 ? 0xffffffffu : (1u << in_warp) - 1u, y < L);
  }
  if (y >= L) return;
  const uint32_t xa = S * (LIN ? bx : bx * blockDim.x + threadIdx.x); /* x/2 of the first site */
  const uint32_t plane = L * Lh;
  const uint32_t row = y * Lh + xa;
  const uint32_t rowN = (y + 1 == L) ? xa : row + Lh;
  const uint32_t rowS = (y == 0) ? row + (L - 1) * Lh : row - Lh;
  const uint32_t rowXp = (xa + S == Lh) ? row + S - Lh : row + S; /* x/2 = xa+S */
  const uint32_t rowXm = (xa == 0) ? row + Lh - 1 : row - 1;      /* x/2 = xa-1 */
  const size_t P = (size_t)g.P;
  uint32_t *mine = spin + (size_t)(s * 2 + p) * P * W + grp * VW;
  const uint32_t *oth = spin + (size_t)(s * 2 + (p ^ 1)) * P * W + grp * VW;
  const uint8_t *jbp = jb + (size_t)(s * 2 + p) * P;
  const uint64_t keep = l2_keep(), strm = l2_stream();

  /* demon plane (p, ic): the demon of site x sits at x - sgn*2k*e_axis after
   * k walks (see micsa_kernels.cuh).  An x shift by an odd number of x/2
   * steps separates the pair's two demon words (and may wrap between them);
   * with four sites, any shift that is not a multiple of 4 x/2 steps makes
   * the four words separate loads. */
  uint32_t *q0b = nullptr, *q1b = nullptr;
  uint32_t drowA = row, drowB = row + 1, zd = z0;
  bool dpair = true;
  if (MICSA) {
    const int k = kwalk;
    const int sh = ((p == 0) == (ic < 3)) ? k : -k; /* in units of 2 sites */
    const int axis = ic < 3 ? ic : ic - 3;
    if (axis == 0) {
      int xd = (int)xa - sh;
      xd += xd < 0 ? (int)Lh : (xd >= (int)Lh ? -(int)Lh : 0);
      const int xe = (xd + 1 == (int)Lh) ? 0 : xd + 1;
      drowA = y * Lh + (uint32_t)xd;
      drowB = y * Lh + (uint32_t)xe;
      dpair = !(sh & (S - 1));
    } else if (axis == 1) {
      int yd = (int)y - 2 * sh;
      yd += yd < 0 ? (int)L : (yd >= (int)L ? -(int)L : 0);
      drowA = (uint32_t)yd * Lh + xa;
      drowB = drowA + 1;
    } else {
      int t = (int)z0 - 2 * sh;
      t += t < 0 ? (int)L : (t >= (int)L ? -(int)L : 0);
      zd = (uint32_t)t;
    }
    const size_t base = ((size_t)(s * 2 + p) * g.nc + ic) * P * W + grp * VW;
    q0b = d0 + base;
    q1b = d1 + base;
  }

  /* TMA variant (W == VW, whole row tiles): the block's demon tile in each
   * of its zc planes -- blockDim.y rows of the block's 2*blockDim.x pairs,
   * shifted by the walk -- is loaded by one thread into shared memory at the
   * start, completing on one mbarrier per plane.  The box is 4 words wider
   * than the tile so that its start can be rounded down to 16 bytes; tiles
   * that would wrap around the lattice keep the global loads. */
  extern __shared__ __align__(128) uint32_t smem_dyn[];
  uint64_t *bars = nullptr;
  int off = 0;
  bool staged = false;
  if (TMA && MICSA) {
    const int k = kwalk;
    const int sh = ((p == 0) == (ic < 3)) ? k : -k;
    const int axis = ic < 3 ? ic : ic - 3;
    const int xb = 2 * bx * blockDim.x, yb = tile * blockDim.y;
    int cx = xb, ry = yb;
    if (axis == 0) { cx = xb - sh; cx += cx < 0 ? (int)Lh : (cx >= (int)Lh ? -(int)Lh : 0); }
    if (axis == 1) { ry = yb - 2 * sh; ry += ry < 0 ? (int)L : (ry >= (int)L ? -(int)L : 0); }
    const int c0 = cx * VW, cal = c0 & ~3;
    off = c0 - cal;
    staged = cx + 2 * (int)blockDim.x <= (int)Lh && ry + (int)blockDim.y <= (int)L &&
             off + 2 * (int)blockDim.x * VW <= tm.box_w;
    const int tile_words = (int)blockDim.y * tm.box_w;
    bars = (uint64_t *)(smem_dyn + 2 * zc * tile_words);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (staged) {
      if (tid == 0) {
        for (int t = 0; t < zc; t++) mbar_init(bars + t, 1);
        mbar_fence_init();
      }
      __syncthreads();
      if (tid == 0) {
        const int zplane = (((g.s0 + (int)s) * 2 + p) * g.nc + ic) * (int)L;
        for (int t = 0; t < zc; t++) {
          int zt = (int)zd + t;
          zt -= zt >= (int)L ? (int)L : 0;
          mbar_expect_tx(bars + t, 2u * (uint32_t)tile_words * 4u);
          tma_load_3d(smem_dyn + (2 * t) * tile_words, &tm.map[0], cal, ry, zplane + zt, bars + t);
          tma_load_3d(smem_dyn + (2 * t + 1) * tile_words, &tm.map[1], cal, ry, zplane + zt,
                      bars + t);
        }
      }
    }
  }

  /* other colour at (2j, 2j+1; y) for planes z0-1 and z0 */
  uint32_t vm[N], v0[N];
  PR::template ld_oth<FLOW>(oth + ((z0 == 0 ? L - 1 : z0 - 1) * plane + row) * W, W, vm, keep);
  PR::template ld_oth<FLOW>(oth + (z0 * plane + row) * W, W, v0, keep);

  /* XS: the remaining x neighbour is a word the adjacent thread of the row
   * holds in v0 -- its first site's words when the row looks at +x, its
   * second site's at -x (rowoff is the same along a row) -- taken by shuffle
   * when that thread is in the same warp, loaded otherwise (row ends, the
   * periodic wrap, warp boundaries).  Source lane (bits 0-4) and "taken"
   * (bit 5) per direction, -x in bits 0-7 and +x in bits 8-15: */
  uint32_t xs_code = 0;
  if (XS) {
    const unsigned lin = threadIdx.y * blockDim.x + threadIdx.x;
    const bool okp = threadIdx.x + 1 < blockDim.x && xa + S < Lh && ((lin + 1) & 31u) != 0;
    const bool okm = threadIdx.x > 0 && xa > 0 && (lin & 31u) != 0;
    xs_code = (((okm ? lin - 1 : lin) & 31u) | (okm ? 32u : 0u)) |
              ((((okp ? lin + 1 : lin) & 31u) | (okp ? 32u : 0u)) << 8);
  }

  uint32_t zdd = zd;
#pragma unroll(UNR)
  for (uint32_t t = 0; t < (uint32_t)zc; t++) {
    const uint32_t z = z0 + t;
    const uint32_t zo = z * plane;
    const uint32_t rowoff = (y + z + p) & 1; /* x = 2*(x/2) + rowoff for both */
    uint32_t own[N], up[N], vn[N], vs[N], ext[VW], a0[N], a1[N], a2[N];
    PR::ld(mine + (zo + row) * W, W, own, keep);
    PR::template ld_oth<FLOW>(oth + ((z + 1 == L ? 0 : zo + plane) + row) * W, W, up, keep);
    PR::template ld_oth<FLOW>(oth + (zo + rowN) * W, W, vn, keep);
    PR::template ld_oth<FLOW>(oth + (zo + rowS) * W, W, vs, keep);
    bool ext_done = false;
    if (XS) {
      const uint32_t c = xs_code >> (8 * rowoff);
      ext_done = (c & 32u) != 0;
#pragma unroll
      for (int w = 0; w < VW; w++)
        ext[w] = __shfl_sync(xs_mask, rowoff ? v0[w] : v0[VW + w], (int)(c & 31u));
    }
    if (!ext_done) {
      if (FLOW)
        hint<VW>::ld_co(oth + (zo + (rowoff ? rowXp : rowXm)) * W, ext, keep);
      else
        hint<VW>::ld_nc(oth + (zo + (rowoff ? rowXp : rowXm)) * W, ext, keep);
    }
    const uint32_t jbs = S == 4 ? ld_u32_keep(jbp + zo + row, keep) : ld_u16_keep(jbp + zo + row, keep);
    bool from_smem = false;
    if (TMA && staged) {
      if (mbar_wait(bars + t, 0)) {
        const int tile_words = (int)blockDim.y * tm.box_w;
        const uint32_t *r0 = smem_dyn + (2 * t) * tile_words + threadIdx.y * tm.box_w + off +
                             2 * threadIdx.x * VW;
        const uint32_t *r1 = r0 + tile_words;
#pragma unroll
        for (int w = 0; w < N; w++) {
          a0[w] = r0[w];
          a1[w] = r1[w];
        }
        from_smem = true;
      } else {
        atomicAdd(&micsa_tma_timeouts, 1u);
      }
    }
    if (MICSA) {
      if (!from_smem) {
        const uint32_t sa = (zdd * plane + drowA) * W;
        if (dpair) {
          PR::ld_na(q0b + sa, W, a0, strm);
          PR::ld_na(q1b + sa, W, a1, strm);
        } else if (S == 4) { /* four single words, each wrapped along the row */
          const uint32_t xd = drowA % Lh, rbase = zdd * plane + (drowA - xd);
#pragma unroll
          for (int k = 0; k < N; k++) {
            uint32_t xk = xd + k;
            xk -= xk >= Lh ? Lh : 0;
            a0[k] = ld_na_u32(q0b + rbase + xk, strm);
            a1[k] = ld_na_u32(q1b + rbase + xk, strm);
          }
        } else {
          const uint32_t sb = (zdd * plane + drowB) * W;
          uint32_t x0[VW], x1[VW], y0[VW], y1[VW];
          hint<VW>::ld_na(q0b + sa, x0, strm);
          hint<VW>::ld_na(q0b + sb, x1, strm);
          hint<VW>::ld_na(q1b + sa, y0, strm);
          hint<VW>::ld_na(q1b + sb, y1, strm);
#pragma unroll
          for (int w = 0; w < VW; w++) {
            a0[w] = x0[w]; a0[VW + w] = x1[w];
            a1[w] = y0[w]; a1[VW + w] = y1[w];
          }
        }
      }
      if (!staged && pd > 0 && t + (uint32_t)pd < (uint32_t)zc) {
        uint32_t zf = zdd + (uint32_t)pd;
        if (zf >= L) zf -= L;
        prefetch_l2(q0b + (zf * plane + drowA) * W);
        prefetch_l2(q1b + (zf * plane + drowA) * W);
      }
    } else {
      const uint32_t *rb = rnd + (size_t)(zo + row) * W + grp * VW;
      PR::ld_na(rb, W, a0, strm);
      PR::ld_na(rb + P * W, W, a1, strm);
      PR::ld_na(rb + 2 * P * W, W, a2, strm);
    }
    /* x-neighbours: the thread's site k (x/2 = xa + k) of colour p sees, in
     * the other colour, +x at x/2 + rowoff and -x at x/2 + rowoff - 1: words
     * of v0, or ext past either end */
#pragma unroll
    for (int site = 0; site < S; site++) {
      const uint32_t jb6 = (jbs >> (8 * site)) & 0xffu;
      const uint32_t mE = jmask(jb6, 0), mN = jmask(jb6, 1), mU = jmask(jb6, 2);
      const uint32_t mO = jmask(jb6, 3), mS = jmask(jb6, 4), mD = jmask(jb6, 5);
#pragma unroll
      for (int w = 0; w < VW; w++) {
        const int o = site * VW + w;
        /* site k: +x = rowoff ? (k+1 < S ? v0[k+1] : ext) : v0[k],
         *         -x = rowoff ? v0[k] : (k > 0 ? v0[k-1] : ext) */
        uint32_t nE, nO;
        if constexpr (S == 2) { /* A = site 0, B = site 1 */
          const uint32_t cA = v0[w], cB = v0[VW + w], ex = ext[w];
          nE = site == 0 ? (rowoff ? cB : cA) : (rowoff ? ex : cB);
          nO = site == 0 ? (rowoff ? cA : ex) : (rowoff ? cB : cA);
        } else {
          const uint32_t ck = v0[o], ex = ext[w];
          const uint32_t cn = site + 1 < S ? v0[(site + 1 < S ? site + 1 : 0) * VW + w] : ex;
          const uint32_t cp = site > 0 ? v0[(site > 0 ? site - 1 : 0) * VW + w] : ex;
          nE = rowoff ? cn : ck;
          nO = rowoff ? ck : cp;
        }
        const uint32_t sw = own[o];
        const uint32_t f0 = xor3(sw, nE, mE), f1 = xor3(sw, vn[o], mN), f2 = xor3(sw, up[o], mU);
        const uint32_t f3 = xor3(sw, nO, mO), f4 = xor3(sw, vs[o], mS), f5 = xor3(sw, vm[o], mD);
        const uint32_t j1 = xor3(f0, f1, f2), j2 = maj3(f0, f1, f2);
        const uint32_t j3 = xor3(f3, f4, f5), j4 = maj3(f3, f4, f5);
        uint32_t flip;
        if (MICSA)
          flip = isi_update(j1, j2, j3, j4, a0[o], a1[o]);
        else
          flip = metropolis_flip(j1, j2, j3, j4, a0[o], a1[o], a2[o]);
        own[o] = sw ^ flip;
      }
    }
    PR::st(mine + (zo + row) * W, W, own, keep);
    if (MICSA) {
      const uint32_t sa = (zdd * plane + drowA) * W;
      if (dpair) {
        PR::st(q0b + sa, W, a0, strm);
        PR::st(q1b + sa, W, a1, strm);
      } else if (S == 4) {
        const uint32_t xd = drowA % Lh, rbase = zdd * plane + (drowA - xd);
#pragma unroll
        for (int k = 0; k < N; k++) {
          uint32_t xk = xd + k;
          xk -= xk >= Lh ? Lh : 0;
          st_u32(q0b + rbase + xk, a0[k], strm);
          st_u32(q1b + rbase + xk, a1[k], strm);
        }
      } else {
        const uint32_t sb = (zdd * plane + drowB) * W;
        uint32_t x0[VW], x1[VW], y0[VW], y1[VW];
#pragma unroll
        for (int w = 0; w < VW; w++) {
          x0[w] = a0[w]; x1[w] = a0[VW + w];
          y0[w] = a1[w]; y1[w] = a1[VW + w];
        }
        hint<VW>::st(q0b + sa, x0, strm);
        hint<VW>::st(q0b + sb, x1, strm);
        hint<VW>::st(q1b + sa, y0, strm);
        hint<VW>::st(q1b + sb, y1, strm);
      }
    }
#pragma unroll
    for (int w = 0; w < N; w++) {
      vm[w] = v0[w];
      v0[w] = up[w];
    }
    zdd = (zdd + 1 == L) ? 0 : zdd + 1;
  }
}

template <int VW, bool MICSA, bool WIDE, int MINB, bool TMA, int S = 2>
__global__ void __launch_bounds__(TPB, MINB)
k_sweep(const micsa_geo g, const int p, const int ic, const int ytiles, const int G,
        const int zc, const int pd, uint32_t *__restrict__ spin, uint32_t *__restrict__ d0,
        uint32_t *__restrict__ d1, const uint8_t *__restrict__ jb,
        const int *__restrict__ walk, const uint32_t *__restrict__ rnd,
        const __grid_constant__ micsa_tma tm) {
  grid_dependency_sync();
  const uint32_t by = blockIdx.y;
  const uint32_t tile = by % ytiles, sg = by / ytiles; /* block-uniform */
  const uint32_t s = sg / G, grp = sg % G;
  /* the walk and the run flag are loaded together: one round trip */
  const int kwalk = MICSA ? __ldg(walk + s) : 0;
  if (micsa_frozen(g, (int)s)) return;
  sweep_block<VW, MICSA, WIDE, TMA, false, S>(g, p, ic, s, grp, tile, blockIdx.x, blockIdx.z * zc,
                                              zc, pd, kwalk, spin, d0, d1, jb, rnd, tm);
}

/* ---------------------------------------------------- dataflow sweep */
/* All 2*nc half-sweeps of one iteration, of every sample, in one launch:
 * the launch boundaries between half-sweeps (each a drain of the whole GPU)
 * become per-slab dependencies.  The grid has one block per tile -- one
 * k_sweep block over one slab of zc z planes -- and a block takes its tile
 * from a ticket counter when it starts (not from blockIdx, whose dispatch
 * order is not guaranteed), in this order: sample then half-sweep j
 * (sample-major, the L2 then holds one sample's spins) or half-sweep then
 * sample (many small samples side by side), then slab (the half-sweep's
 * slabs start at slab j mod L/zc), then tile.  Half-sweep j has ic = j/2
 * and colour p = j%2, the order of the reference's Monte_Carlo loop
 * (main.cu:254-284).
 *
 * A tile of half-sweep j on slab b reads the other colour on planes
 * z0-1 .. z0+zc and its demon slots, and writes its own colour on slab b.
 * It starts once half-sweep j-1 has finished slabs b-1, b and b+1, so it
 * reads exactly what the j-th half-sweep of the reference reads; and no tile
 * still running reads what it writes (a tile of j+k runs beside one of j
 * only more than k slabs away, and reads one plane beyond its slab).  The
 * demon walk moves by whole iterations, between launches.
 *
 * Counters: ctl[0] tickets, ctl[1] blocks done, ctl[4 + s*nslab + b] tiles
 * of slab b of sample s finished in this launch.  No tile of j starts on
 * slab b before all of slab b's tiles of j-1 are done, so slab b has
 * finished half-sweeps 0 .. j-1 exactly when its counter reaches (tiles per
 * slab) * j.  Tiles wait only on earlier tickets, and a ticket is only held
 * by a running block, so the earliest unfinished tile can always run: the
 * launch needs no co-residency.  The lead thread polls the three counters
 * with relaxed loads issued together, then an acquire fence and a block
 * barrier order the tile's loads after the producers' stores; a producer
 * releases with a block barrier, a fence and an atomic add.  Waits are
 * bounded (2 s by the global timer; after one runs out every later wait
 * gives up at once, and micsa_flow_timeouts counts them); the last block to
 * finish resets the counters for the next launch. */
__device__ unsigned int micsa_flow_timeouts;
/* The wait limit, and an offset added to every wait's target count: 0 in
 * operation; set through micsa_debug_flow_waits so that a test can make the
 * waits run out (counters never reach a target raised by the offset). */
__device__ unsigned long long micsa_flow_limit_ns = 2000000000ull;
__device__ unsigned int micsa_flow_need_offset = 0u;

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *a) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
/* wait until *a, *b and *c are all >= need, then acquire; false when the
 * limit ran out (or an earlier wait's did) */
__device__ __forceinline__ bool flow_wait3(const unsigned *a, const unsigned *b,
                                           const unsigned *c, unsigned need) {
  uint64_t t0 = 0;
  bool ok = true;
  for (;;) {
    const unsigned x = ld_relaxed_u32(a), y = ld_relaxed_u32(b), z = ld_relaxed_u32(c);
    if (min(x, min(y, z)) >= need) break;
    if (!t0) t0 = global_ns();
    if (*(volatile unsigned *)&micsa_flow_timeouts || global_ns() - t0 > micsa_flow_limit_ns) {
      ok = false;
      break;
    }
    __nanosleep(64);
  }
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
  return ok;
}

/* The lead thread's part: take a ticket, decode it into job[] (s, j, slab,
 * bx, row tile, group, walk) from the launch's constants in cst[] and wait
 * for the tile's dependencies. */
enum { C_GX, C_NSLAB, C_T, C_PER_HALF, C_PER_SAMPLE, C_YT, C_SMAJ, C_N };
__device__ __forceinline__ void dep_decode(const micsa_geo &g, const int *__restrict__ walk,
                                           const unsigned *cst, const unsigned u, unsigned *job) {
  const unsigned nslab = cst[C_NSLAB], T = cst[C_T], gx = cst[C_GX], ytiles = cst[C_YT];
  unsigned s, j, r2;
  if (cst[C_SMAJ]) {
    s = u / cst[C_PER_SAMPLE];
    const unsigned r = u % cst[C_PER_SAMPLE];
    j = r / cst[C_PER_HALF];
    r2 = r % cst[C_PER_HALF];
  } else {
    const unsigned per_j = (unsigned)g.ns * cst[C_PER_HALF], r = u % per_j;
    j = u / per_j;
    s = r / cst[C_PER_HALF];
    r2 = r % cst[C_PER_HALF];
  }
  const unsigned b = (r2 / T + j) % nslab, t = r2 % T;
  job[0] = s;
  job[1] = j;
  job[2] = b;
  job[3] = t % gx;
  job[4] = (t / gx) % ytiles;
  job[5] = t / (gx * ytiles);
  job[6] = (unsigned)__ldg(walk + s);
}
__device__ __forceinline__ void dep_take(const micsa_geo &g, const int *__restrict__ walk,
                                         unsigned *__restrict__ ctl, const unsigned *cst,
                                         unsigned *job) {
  dep_decode(g, walk, cst, atomicAdd(ctl, 1u), job);
}
/* ... and the lead thread's wait for the tile's dependencies */
__device__ __forceinline__ void dep_wait(const micsa_geo &g, unsigned *__restrict__ ctl,
                                         const unsigned *cst, const unsigned *job) {
  const unsigned s = job[0], j = job[1], b = job[2], nslab = cst[C_NSLAB], T = cst[C_T];
  if (j > 0 && !micsa_frozen(g, (int)s)) {
    const unsigned *c = ctl + 4 + s * nslab;
    if (!flow_wait3(c + (b == 0 ? nslab - 1 : b - 1), c + b, c + (b + 1 == nslab ? 0 : b + 1),
                    T * j + micsa_flow_need_offset))
      atomicAdd(&micsa_flow_timeouts, 1u);
  }
}

/* L2 prefetch of the demon words a thread of a sweep_block tile will read:
 * plane (p, ic) of sample s, rows as sweep_block derives them, z planes
 * [z0, z0 + n).  The demon planes are read and written by one half-sweep
 * only, so a dataflow tile can request them before its dependency wait. */
template <int VW>
__device__ __forceinline__ void prefetch_tile_demons(const micsa_geo &g, int p, int ic,
                                                     uint32_t s, uint32_t grp, uint32_t tile,
                                                     uint32_t bx, uint32_t z0, int n, int kwalk,
                                                     const uint32_t *d0, const uint32_t *d1) {
  const uint32_t L = g.L, Lh = g.Lh, W = g.W;
  const uint32_t y = tile * blockDim.y + threadIdx.y;
  if (y >= L) return;
  const uint32_t xa = 2 * (bx * blockDim.x + threadIdx.x);
  const int sh = ((p == 0) == (ic < 3)) ? kwalk : -kwalk;
  const int axis = ic < 3 ? ic : ic - 3;
  uint32_t drow = y * Lh + xa, zd = z0;
  if (axis == 0) {
    int xd = (int)xa - sh;
    xd += xd < 0 ? (int)Lh : (xd >= (int)Lh ? -(int)Lh : 0);
    drow = y * Lh + (uint32_t)xd;
  } else if (axis == 1) {
    int yd = (int)y - 2 * sh;
    yd += yd < 0 ? (int)L : (yd >= (int)L ? -(int)L : 0);
    drow = (uint32_t)yd * Lh + xa;
  } else {
    int t = (int)z0 - 2 * sh;
    t += t < 0 ? (int)L : (t >= (int)L ? -(int)L : 0);
    zd = (uint32_t)t;
  }
  const size_t base = ((size_t)(s * 2 + p) * g.nc + ic) * (size_t)g.P * W + grp * VW;
  const uint32_t plane = L * Lh;
  for (int t = 0; t < n; t++) {
    prefetch_l2(d0 + base + (size_t)(zd * plane + drow) * W);
    prefetch_l2(d1 + base + (size_t)(zd * plane + drow) * W);
    zd = (zd + 1 == L) ? 0 : zd + 1;
  }
}

/* The tile's values go through shared memory and are read where they are
 * used, so that none of them stays in a register across the sweep body
 * (which needs about all of the 64 registers of the 4-blocks budget). */
template <int VW, bool WIDE, int MINB, int BT = TPB, bool XS = false>
__global__ void __launch_bounds__(BT, MINB)
k_sweep_dep(const __grid_constant__ micsa_geo g, const int ytiles, const int G, const int zc,
            const int pd, const int smaj, const int pf, uint32_t *__restrict__ spin,
            uint32_t *__restrict__ d0,
            uint32_t *__restrict__ d1, const uint8_t *__restrict__ jb,
            const int *__restrict__ walk, unsigned *__restrict__ ctl) {
  /* the z loop unrolled once where two steps' registers do not fit: pairs
   * of two-word sites at 64 registers per thread (16-byte spills against 32
   * unrolled twice; L=160: 8.34 against 8.16 attempts/ps) and the shuffle
   * form (which spills unrolled twice at 80) */
  constexpr int UNR = (XS || (VW >= 2 && 65536 / (MINB * BT) <= 64)) ? 1 : 2;
  grid_dependency_sync();
  __shared__ unsigned cst[C_N];
  __shared__ unsigned job[8]; /* s, j, slab, bx, row tile, group, walk, last */
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  if (lead) {
    const unsigned gx = (unsigned)g.Lh / 2u / blockDim.x; /* blocks along x */
    const unsigned nslab = (unsigned)(g.L / zc);
    const unsigned T = gx * (unsigned)ytiles * (unsigned)G; /* tiles per slab */
    cst[C_GX] = gx;
    cst[C_NSLAB] = nslab;
    cst[C_T] = T;
    cst[C_YT] = (unsigned)ytiles;
    cst[C_PER_HALF] = nslab * T;
    cst[C_PER_SAMPLE] = (unsigned)(g.fit > 1 ? g.fit : 1) * 2u * (unsigned)g.nc * nslab * T;
    cst[C_SMAJ] = (unsigned)smaj;
    dep_take(g, walk, ctl, cst, job);
    if (pf <= 0) dep_wait(g, ctl, cst, job);
  }
  __syncthreads();
  /* half-sweep J of the launch is half-sweep J % 2nc of its iteration J / 2nc,
   * whose demons sit one walk step further per iteration */
  const unsigned per_it = 2u * (unsigned)g.nc, J = job[1];
  const unsigned jj = J % per_it;
  const int kwalk = (int)((job[6] + J / per_it) % (unsigned)g.Lh);
  if (pf > 0) {
    /* the tile's demon words are independent of the half-sweep before it:
     * on their way into L2 while the lead thread waits for the dependencies
     * (at most pf planes: the z loop's own prefetch takes over from there) */
    if (!micsa_frozen(g, (int)job[0]))
      prefetch_tile_demons<VW>(g, (int)(jj & 1u), (int)(jj >> 1), job[0], job[5], job[4],
                               job[3], job[2] * (unsigned)zc, pf < zc ? pf : zc, kwalk, d0, d1);
    if (lead) dep_wait(g, ctl, cst, job);
    __syncthreads();
  }
  {
    const unsigned s = job[0];
    if (!micsa_frozen(g, (int)s)) {
      micsa_tma none;
      sweep_block<VW, true, WIDE, false, true, 2, false, XS, UNR>(
          g, (int)(jj & 1u), (int)(jj >> 1), s, job[5], job[4], job[3], job[2] * (unsigned)zc,
          zc, pd, kwalk, spin, d0, d1, jb, nullptr, none);
    }
  }
  __syncthreads();
  if (lead) {
    __threadfence();
    atomicAdd(ctl + 4 + job[0] * cst[C_NSLAB] + job[2], 1u);
    __threadfence();
    job[7] = atomicAdd(ctl + 1, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (job[7]) { /* every other block has finished: reset for the next launch */
    const unsigned tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    const unsigned n = (unsigned)g.ns * cst[C_NSLAB];
    for (unsigned k = tid; k < n; k += nt) ctl[4 + k] = 0;
    if (lead) {
      ctl[0] = 0;
      ctl[1] = 0;
    }
  }
}

/* Persistent form of the dataflow sweep: a grid of the blocks that fit the
 * GPU at once, each looping over tickets.  A block takes its next ticket
 * while it computes the current tile (the atomic's round trip and the
 * decode leave the block's barrier path), releases the current tile's slab
 * counter, then waits for the next tile's dependencies.  Tickets are taken
 * in order by running blocks and a block holds at most one ticket it has
 * not started, which is larger than the one it works on; so the smallest
 * unfinished ticket always belongs to a block that is computing it, with
 * its dependencies (smaller tickets) done: the launch cannot stall.  Tiles,
 * order and results are those of k_sweep_dep. */
template <int VW, bool WIDE, int MINB>
__global__ void __launch_bounds__(TPB, MINB)
k_sweep_pdep(const __grid_constant__ micsa_geo g, const int ytiles, const int G, const int zc,
             const int pd, const int smaj, const unsigned total, uint32_t *__restrict__ spin,
             uint32_t *__restrict__ d0, uint32_t *__restrict__ d1,
             const uint8_t *__restrict__ jb, const int *__restrict__ walk,
             unsigned *__restrict__ ctl) {
  grid_dependency_sync();
  __shared__ unsigned cst[C_N];
  __shared__ unsigned job[2][8]; /* s, j, slab, bx, row tile, group, walk, valid */
  __shared__ unsigned last;
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  if (lead) {
    const unsigned gx = (unsigned)g.Lh / 2u / blockDim.x;
    const unsigned nslab = (unsigned)(g.L / zc);
    const unsigned T = gx * (unsigned)ytiles * (unsigned)G;
    cst[C_GX] = gx;
    cst[C_NSLAB] = nslab;
    cst[C_T] = T;
    cst[C_YT] = (unsigned)ytiles;
    cst[C_PER_HALF] = nslab * T;
    cst[C_PER_SAMPLE] = (unsigned)(g.fit > 1 ? g.fit : 1) * 2u * (unsigned)g.nc * nslab * T;
    cst[C_SMAJ] = (unsigned)smaj;
    const unsigned u = atomicAdd(ctl, 1u);
    job[0][7] = u < total;
    if (u < total) {
      dep_decode(g, walk, cst, u, job[0]);
      dep_wait(g, ctl, cst, job[0]);
    }
  }
  __syncthreads();
  const unsigned per_it = 2u * (unsigned)g.nc;
  for (int cur = 0; job[cur][7]; cur ^= 1) {
    unsigned un = 0;
    if (lead) un = atomicAdd(ctl, 1u); /* the next ticket, used after this tile */
    {
      const unsigned *jc = job[cur];
      const unsigned J = jc[1], jj = J % per_it, s = jc[0];
      const int kwalk = (int)((jc[6] + J / per_it) % (unsigned)g.Lh);
      if (!micsa_frozen(g, (int)s)) {
        micsa_tma none;
        sweep_block<VW, true, WIDE, false, true>(g, (int)(jj & 1u), (int)(jj >> 1), s, jc[5],
                                                 jc[4], jc[3], jc[2] * (unsigned)zc, zc, pd,
                                                 kwalk, spin, d0, d1, jb, nullptr, none);
      }
    }
    __syncthreads();
    if (lead) {
      __threadfence();
      atomicAdd(ctl + 4 + job[cur][0] * cst[C_NSLAB] + job[cur][2], 1u);
      unsigned *nx = job[cur ^ 1];
      nx[7] = un < total;
      if (un < total) {
        dep_decode(g, walk, cst, un, nx);
        dep_wait(g, ctl, cst, nx);
      }
    }
    __syncthreads();
  }
  if (lead) {
    __threadfence();
    last = atomicAdd(ctl + 1, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) { /* every other block has finished: reset for the next launch */
    const unsigned tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    const unsigned n = (unsigned)g.ns * cst[C_NSLAB];
    for (unsigned k = tid; k < n; k += nt) ctl[4 + k] = 0;
    if (lead) {
      ctl[0] = 0;
      ctl[1] = 0;
    }
  }
}

/* ------------------------------------------ mixed-lattice dataflow sweep */
/* One launch advances every sample of several contexts (groups) of
 * different L by one iteration: the dataflow sweep above, generalised to a
 * table of groups.  A ticket u falls in group gi when first[gi] <= u <
 * first[gi + 1]; inside the group it is decoded as in k_sweep_dep (sample,
 * half-sweep j, slab, tile; sample-major or half-sweep-major), and a tile of
 * half-sweep j on slab b waits until j-1 has finished slabs b-1, b, b+1 of
 * the same sample (the group's own counters).  The block is a fixed MTPB
 * threads mapped onto consecutive (word group, row, x/2 pair) units of the
 * slab -- rows of a z plane are contiguous, so a block's loads stay
 * coalesced at any L -- and each thread marches the group's zc planes.
 * A launch may carry several iterations (a.iters): half-sweep j of the
 * launch is half-sweep j % 2nc of iteration j / 2nc, and the same rule
 * orders it -- after j-1 on the neighbouring slabs, which transitively
 * covers the demon words the walk moves between iterations (two planes
 * along one axis) -- so the dependency wavefront runs on from one
 * iteration into the next without a drain of the GPU between them.
 * Where a slab plane has fewer units than a block has threads, one tile
 * takes the same slab of spt consecutive samples (a sample group, with its
 * own counters), so small lattices fill their blocks.  Tickets are only
 * taken for samples [0, ns_run) of each group (the running prefix); frozen
 * samples inside it are skipped. */
__global__ void __launch_bounds__(MTPB, 8)
k_walk_multi(const __grid_constant__ micsa_multi_args a) {
  const int gi = blockIdx.y, s = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= a.n) return;
  const micsa_mgroup &m = a.gr[gi];
  if (s < (int)m.ns_run && !micsa_frozen(m.g, s)) {
    int *w = m.walk + s;
    *w = (int)(((unsigned)*w + a.iters) % (unsigned)(m.g.L / 2));
  }
}

template <int VW, bool WIDE, int MINB>
__global__ void __launch_bounds__(MTPB, MINB)
k_sweep_multi(const __grid_constant__ micsa_multi_args a, unsigned *__restrict__ ctl) {
  grid_dependency_sync();
  __shared__ unsigned job[8]; /* group, sample group, j, slab, tile, last */
  /* the tile's group, copied out of the parameter table: read from shared
   * memory where used, so that none of it occupies registers */
  __shared__ micsa_mgroup m;
  if (threadIdx.x == 0) {
    const unsigned u = atomicAdd(ctl, 1u);
    int gi = 0;
    while (gi + 1 < a.n && u >= a.gr[gi + 1].first) gi++;
    m = a.gr[gi];
    /* j runs over the a.iters * 2nc half-sweeps of the launch */
    const unsigned r = u - m.first, per_half = m.nslab * m.T;
    unsigned sg, j, r2;
    if (a.smaj) {
      const unsigned per_sg = a.iters * 2u * (unsigned)m.g.nc * per_half;
      sg = r / per_sg;
      j = (r % per_sg) / per_half;
      r2 = r % per_half;
    } else {
      const unsigned per_j = m.nsg * per_half;
      j = r / per_j;
      sg = (r % per_j) / per_half;
      r2 = r % per_half;
    }
    const unsigned b = (r2 / m.T + j) % m.nslab;
    job[0] = (unsigned)gi;
    job[1] = sg;
    job[2] = j;
    job[3] = b;
    job[4] = r2 % m.T;
    if (j > 0) {
      const unsigned *c = ctl + 4 + m.cnt_off + sg * m.nslab;
      if (!flow_wait3(c + (b == 0 ? m.nslab - 1 : b - 1), c + b,
                      c + (b + 1 == m.nslab ? 0 : b + 1), m.T * j + micsa_flow_need_offset))
        atomicAdd(&micsa_flow_timeouts, 1u);
    }
  }
  __syncthreads();
  {
    /* the thread's unit of the tile: (sample of the group, word group, row, pair);
     * half-sweep j of the launch is half-sweep j % 2nc of iteration j / 2nc,
     * whose demons sit one walk step further per iteration */
    const unsigned J = job[2], per_it = 2u * (unsigned)m.g.nc;
    const unsigned it = J / per_it, j = J % per_it;
    const unsigned pairs = (unsigned)m.g.Lh / 2u, units = (unsigned)m.g.L * pairs;
    const unsigned uper = units * m.G;
    const unsigned v = job[4] * MTPB + threadIdx.x;
    const unsigned so = v / uper, w = v % uper;
    const unsigned s = job[1] * m.spt + so;
    if (so < m.spt && s < m.ns_run && !micsa_frozen(m.g, (int)s)) {
      const unsigned grp = w / units, un = w % units;
      const int kwalk = (int)(((unsigned)__ldg(m.walk + s) + it) % ((unsigned)m.g.L / 2u));
      micsa_tma none;
      sweep_block<VW, true, WIDE, false, true, 2, true>(
          m.g, (int)(j & 1u), (int)(j >> 1), s, grp, un / pairs, un % pairs,
          job[3] * (unsigned)m.zc, m.zc, m.pd, kwalk, m.spin, m.d0, m.d1, m.jb, nullptr, none);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctl + 4 + m.cnt_off + job[1] * m.nslab + job[3], 1u);
    __threadfence();
    job[5] = atomicAdd(ctl + 1, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (job[5]) { /* every other block has finished: reset for the next launch */
    for (unsigned k = threadIdx.x; k < a.ncnt; k += MTPB) ctl[4 + k] = 0;
    if (threadIdx.x == 0) {
      ctl[0] = 0;
      ctl[1] = 0;
    }
  }
}

/* ------------------------------------------- sweep with cp.async staging */
__device__ __forceinline__ void cp_async16(void *dst, const void *src, uint64_t pol) {
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;"
               ::"r"(smem_addr(dst)), "l"(src), "l"(pol) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src, uint64_t pol) {
  asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;"
               ::"r"(smem_addr(dst)), "l"(src), "l"(pol) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src, uint64_t pol) {
  asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;"
               ::"r"(smem_addr(dst)), "l"(src), "l"(pol) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int NPEND> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(NPEND) : "memory");
}

constexpr int ASYNC_ITEMS = 7; /* own, up, y+1, y-1, D0, D1, {x-neighbour word pair, couplings} */

/* The micSA half-sweep of k_sweep (VW = 2, one word group per site) with its
 * per-step operands double-buffered in shared memory: while a thread
 * computes z step t, its copies for step t+1 are in flight (cp.async), so
 * the latency of the next loads overlaps the arithmetic of this step.  Each
 * thread copies and reads only its own slots (item-major layout,
 * [stage][item][thread] x 16 bytes: conflict-free), waiting on its own copy
 * groups -- no barrier.  Prefetching a step is safe: a thread's own spins
 * and demon words are written only by that thread, the other colour and the
 * couplings are read-only during a half-sweep. */
template <int MINB>
__global__ void __launch_bounds__(TPB, MINB)
k_sweep_async(const micsa_geo g, const int p, const int ic, const int ytiles, const int zc,
              uint32_t *__restrict__ spin, uint32_t *__restrict__ d0,
              uint32_t *__restrict__ d1, const uint8_t *__restrict__ jb,
              const int *__restrict__ walk) {
  constexpr int VW = 2, N = 4;
  grid_dependency_sync();
  const uint32_t L = g.L, Lh = g.Lh, W = g.W; /* W == 2 */
  const uint32_t by = blockIdx.y;
  const uint32_t tile = by % ytiles, s = by / ytiles;
  /* the walk and the run flag are loaded together: one round trip */
  const int kwalk = __ldg(walk + s);
  if (micsa_frozen(g, (int)s)) return;
  const uint32_t y = tile * blockDim.y + threadIdx.y;
  if (y >= L) return;
  const uint32_t xa = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const uint32_t plane = L * Lh;
  const uint32_t z0 = blockIdx.z * zc;
  const uint32_t row = y * Lh + xa;
  const uint32_t rowN = (y + 1 == L) ? xa : row + Lh;
  const uint32_t rowS = (y == 0) ? row + (L - 1) * Lh : row - Lh;
  const uint32_t rowXp = (xa + 2 == Lh) ? row + 2 - Lh : row + 2;
  const uint32_t rowXm = (xa == 0) ? row + Lh - 1 : row - 1;
  const size_t P = (size_t)g.P;
  uint32_t *mine = spin + (size_t)(s * 2 + p) * P * W;
  const uint32_t *oth = spin + (size_t)(s * 2 + (p ^ 1)) * P * W;
  const uint8_t *jbp = jb + (size_t)(s * 2 + p) * P;
  const uint64_t keep = l2_keep(), strm = l2_stream();

  uint32_t drowA = row, drowB = row + 1, zd = z0;
  bool dpair = true;
  {
    const int k = kwalk;
    const int sh = ((p == 0) == (ic < 3)) ? k : -k;
    const int axis = ic < 3 ? ic : ic - 3;
    if (axis == 0) {
      int xd = (int)xa - sh;
      xd += xd < 0 ? (int)Lh : (xd >= (int)Lh ? -(int)Lh : 0);
      const int xe = (xd + 1 == (int)Lh) ? 0 : xd + 1;
      drowA = y * Lh + (uint32_t)xd;
      drowB = y * Lh + (uint32_t)xe;
      dpair = !(sh & 1);
    } else if (axis == 1) {
      int yd = (int)y - 2 * sh;
      yd += yd < 0 ? (int)L : (yd >= (int)L ? -(int)L : 0);
      drowA = (uint32_t)yd * Lh + xa;
      drowB = drowA + 1;
    } else {
      int t = (int)z0 - 2 * sh;
      t += t < 0 ? (int)L : (t >= (int)L ? -(int)L : 0);
      zd = (uint32_t)t;
    }
  }
  const size_t dbase = ((size_t)(s * 2 + p) * g.nc + ic) * P * W;
  uint32_t *q0b = d0 + dbase, *q1b = d1 + dbase;

  extern __shared__ __align__(16) uint4 sbuf[];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  auto slot = [&](int st, int item) -> uint4 * { return sbuf + (st * ASYNC_ITEMS + item) * TPB + tid; };
  /* the copies of z step t into stage t & 1 */
  auto issue = [&](uint32_t t) {
    const int st = (int)(t & 1);
    const uint32_t z = z0 + t, zo = z * plane, rowoff = (y + z + p) & 1;
    uint32_t zt = zd + t;
    zt -= zt >= L ? L : 0;
    cp_async16(slot(st, 0), mine + (zo + row) * W, keep);
    cp_async16(slot(st, 1), oth + ((z + 1 == L ? 0 : zo + plane) + row) * W, keep);
    cp_async16(slot(st, 2), oth + (zo + rowN) * W, keep);
    cp_async16(slot(st, 3), oth + (zo + rowS) * W, keep);
    const uint32_t sa = (zt * plane + drowA) * W;
    if (dpair) {
      cp_async16(slot(st, 4), q0b + sa, strm);
      cp_async16(slot(st, 5), q1b + sa, strm);
    } else {
      const uint32_t sb = (zt * plane + drowB) * W;
      cp_async8(slot(st, 4), q0b + sa, strm);
      cp_async8((uint8_t *)slot(st, 4) + 8, q0b + sb, strm);
      cp_async8(slot(st, 5), q1b + sa, strm);
      cp_async8((uint8_t *)slot(st, 5) + 8, q1b + sb, strm);
    }
    cp_async8(slot(st, 6), oth + (zo + (rowoff ? rowXp : rowXm)) * W, keep);
    const size_t jo = zo + row; /* the pair's two coupling bytes, in an aligned word */
    cp_async4((uint8_t *)slot(st, 6) + 8, jbp + (jo & ~(size_t)3), keep);
    cp_async_commit();
  };

  uint32_t vm[N], v0[N];
  hint<4>::ld_nc(oth + ((z0 == 0 ? L - 1 : z0 - 1) * plane + row) * W, vm, keep);
  hint<4>::ld_nc(oth + (z0 * plane + row) * W, v0, keep);
  issue(0);
  uint32_t zdd = zd;
  for (uint32_t t = 0; t < (uint32_t)zc; t++) {
    if (t + 1 < (uint32_t)zc) {
      issue(t + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const int st = (int)(t & 1);
    const uint32_t z = z0 + t, zo = z * plane, rowoff = (y + z + p) & 1;
    uint32_t own[N], up[N], vn[N], vs[N], a0[N], a1[N];
    {
      const uint4 o = *slot(st, 0), u = *slot(st, 1), n = *slot(st, 2), q = *slot(st, 3);
      const uint4 e0 = *slot(st, 4), e1 = *slot(st, 5);
      own[0] = o.x; own[1] = o.y; own[2] = o.z; own[3] = o.w;
      up[0] = u.x; up[1] = u.y; up[2] = u.z; up[3] = u.w;
      vn[0] = n.x; vn[1] = n.y; vn[2] = n.z; vn[3] = n.w;
      vs[0] = q.x; vs[1] = q.y; vs[2] = q.z; vs[3] = q.w;
      a0[0] = e0.x; a0[1] = e0.y; a0[2] = e0.z; a0[3] = e0.w;
      a1[0] = e1.x; a1[1] = e1.y; a1[2] = e1.z; a1[3] = e1.w;
    }
    const uint4 xj = *slot(st, 6);
    const uint32_t ext[VW] = {xj.x, xj.y};
    const uint32_t jb2 = (xj.z >> (8 * ((zo + row) & 3))) & 0xffffu;
#pragma unroll
    for (int site = 0; site < 2; site++) {
      const uint32_t jb6 = (jb2 >> (8 * site)) & 0xffu;
      const uint32_t mE = jmask(jb6, 0), mN = jmask(jb6, 1), mU = jmask(jb6, 2);
      const uint32_t mO = jmask(jb6, 3), mS = jmask(jb6, 4), mD = jmask(jb6, 5);
#pragma unroll
      for (int w = 0; w < VW; w++) {
        const int o = site * VW + w;
        const uint32_t cA = v0[w], cB = v0[VW + w], ex = ext[w];
        const uint32_t nE = site == 0 ? (rowoff ? cB : cA) : (rowoff ? ex : cB);
        const uint32_t nO = site == 0 ? (rowoff ? cA : ex) : (rowoff ? cB : cA);
        const uint32_t sw = own[o];
        const uint32_t f0 = xor3(sw, nE, mE), f1 = xor3(sw, vn[o], mN), f2 = xor3(sw, up[o], mU);
        const uint32_t f3 = xor3(sw, nO, mO), f4 = xor3(sw, vs[o], mS), f5 = xor3(sw, vm[o], mD);
        const uint32_t j1 = xor3(f0, f1, f2), j2 = maj3(f0, f1, f2);
        const uint32_t j3 = xor3(f3, f4, f5), j4 = maj3(f3, f4, f5);
        own[o] = sw ^ isi_update(j1, j2, j3, j4, a0[o], a1[o]);
      }
    }
    hint<4>::st(mine + (zo + row) * W, own, keep);
    const uint32_t sa = (zdd * plane + drowA) * W;
    if (dpair) {
      hint<4>::st(q0b + sa, a0, strm);
      hint<4>::st(q1b + sa, a1, strm);
    } else {
      const uint32_t sb = (zdd * plane + drowB) * W;
      const uint32_t x0[2] = {a0[0], a0[1]}, x1[2] = {a0[2], a0[3]};
      const uint32_t y0[2] = {a1[0], a1[1]}, y1[2] = {a1[2], a1[3]};
      hint<2>::st(q0b + sa, x0, strm);
      hint<2>::st(q0b + sb, x1, strm);
      hint<2>::st(q1b + sa, y0, strm);
      hint<2>::st(q1b + sb, y1, strm);
    }
#pragma unroll
    for (int w = 0; w < N; w++) {
      vm[w] = v0[w];
      v0[w] = up[w];
    }
    zdd = (zdd + 1 == L) ? 0 : zdd + 1;
  }
}

/* ------------------------------------- sweep with register-pipelined loads */
/* Operands of one z step of a thread's pair (k_sweep's loads). */
template <int VW> struct step_ops {
  uint32_t own[2 * VW], up[2 * VW], vn[2 * VW], vs[2 * VW], a0[2 * VW], a1[2 * VW], ext[VW];
  uint32_t jb2;
};

/* The micSA half-sweep of k_sweep with the loads of z step t+1 issued before
 * the arithmetic and stores of step t, so that a thread always has one step
 * of loads in flight while it computes.  Issuing them early is safe: a
 * thread's own spins and demon words are written only by that thread, and
 * the other colour and the couplings are read-only during a half-sweep. */
template <int VW, bool WIDE, int MINB>
__global__ void __launch_bounds__(TPB, MINB)
k_sweep_pipe(const micsa_geo g, const int p, const int ic, const int ytiles, const int G,
             const int zc, const int pd, uint32_t *__restrict__ spin, uint32_t *__restrict__ d0,
             uint32_t *__restrict__ d1, const uint8_t *__restrict__ jb,
             const int *__restrict__ walk) {
  constexpr int N = 2 * VW;
  using PR = pairs<VW, WIDE>;
  grid_dependency_sync();
  const uint32_t L = g.L, Lh = g.Lh, W = g.W;
  const uint32_t by = blockIdx.y;
  const uint32_t tile = by % ytiles, sg = by / ytiles;
  const uint32_t s = sg / G, grp = sg % G;
  /* the walk and the run flag are loaded together: one round trip */
  const int kwalk = __ldg(walk + s);
  if (micsa_frozen(g, (int)s)) return;
  const uint32_t y = tile * blockDim.y + threadIdx.y;
  if (y >= L) return;
  const uint32_t xa = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const uint32_t plane = L * Lh;
  const uint32_t z0 = blockIdx.z * zc;
  const uint32_t row = y * Lh + xa;
  const uint32_t rowN = (y + 1 == L) ? xa : row + Lh;
  const uint32_t rowS = (y == 0) ? row + (L - 1) * Lh : row - Lh;
  const uint32_t rowXp = (xa + 2 == Lh) ? row + 2 - Lh : row + 2;
  const uint32_t rowXm = (xa == 0) ? row + Lh - 1 : row - 1;
  const size_t P = (size_t)g.P;
  uint32_t *mine = spin + (size_t)(s * 2 + p) * P * W + grp * VW;
  const uint32_t *oth = spin + (size_t)(s * 2 + (p ^ 1)) * P * W + grp * VW;
  const uint8_t *jbp = jb + (size_t)(s * 2 + p) * P;
  const uint64_t keep = l2_keep(), strm = l2_stream();

  uint32_t drowA = row, drowB = row + 1, zd = z0;
  bool dpair = true;
  {
    const int k = kwalk;
    const int sh = ((p == 0) == (ic < 3)) ? k : -k;
    const int axis = ic < 3 ? ic : ic - 3;
    if (axis == 0) {
      int xd = (int)xa - sh;
      xd += xd < 0 ? (int)Lh : (xd >= (int)Lh ? -(int)Lh : 0);
      const int xe = (xd + 1 == (int)Lh) ? 0 : xd + 1;
      drowA = y * Lh + (uint32_t)xd;
      drowB = y * Lh + (uint32_t)xe;
      dpair = !(sh & 1);
    } else if (axis == 1) {
      int yd = (int)y - 2 * sh;
      yd += yd < 0 ? (int)L : (yd >= (int)L ? -(int)L : 0);
      drowA = (uint32_t)yd * Lh + xa;
      drowB = drowA + 1;
    } else {
      int t = (int)z0 - 2 * sh;
      t += t < 0 ? (int)L : (t >= (int)L ? -(int)L : 0);
      zd = (uint32_t)t;
    }
  }
  const size_t dbase = ((size_t)(s * 2 + p) * g.nc + ic) * P * W + grp * VW;
  uint32_t *q0b = d0 + dbase, *q1b = d1 + dbase;

  auto load = [&](uint32_t t, step_ops<VW> &o) {
    const uint32_t z = z0 + t, zo = z * plane, rowoff = (y + z + p) & 1;
    uint32_t zt = zd + t;
    zt -= zt >= L ? L : 0;
    PR::ld(mine + (zo + row) * W, W, o.own, keep);
    PR::ld_nc(oth + ((z + 1 == L ? 0 : zo + plane) + row) * W, W, o.up, keep);
    PR::ld_nc(oth + (zo + rowN) * W, W, o.vn, keep);
    PR::ld_nc(oth + (zo + rowS) * W, W, o.vs, keep);
    hint<VW>::ld_nc(oth + (zo + (rowoff ? rowXp : rowXm)) * W, o.ext, keep);
    o.jb2 = ld_u16_keep(jbp + zo + row, keep);
    const uint32_t sa = (zt * plane + drowA) * W;
    if (dpair) {
      PR::ld_na(q0b + sa, W, o.a0, strm);
      PR::ld_na(q1b + sa, W, o.a1, strm);
    } else {
      const uint32_t sb = (zt * plane + drowB) * W;
      uint32_t x0[VW], x1[VW], y0[VW], y1[VW];
      hint<VW>::ld_na(q0b + sa, x0, strm);
      hint<VW>::ld_na(q0b + sb, x1, strm);
      hint<VW>::ld_na(q1b + sa, y0, strm);
      hint<VW>::ld_na(q1b + sb, y1, strm);
#pragma unroll
      for (int w = 0; w < VW; w++) {
        o.a0[w] = x0[w]; o.a0[VW + w] = x1[w];
        o.a1[w] = y0[w]; o.a1[VW + w] = y1[w];
      }
    }
  };

  uint32_t vm[N], v0[N];
  PR::ld_nc(oth + ((z0 == 0 ? L - 1 : z0 - 1) * plane + row) * W, W, vm, keep);
  PR::ld_nc(oth + (z0 * plane + row) * W, W, v0, keep);
  step_ops<VW> cur;
  load(0, cur);
  uint32_t zdd = zd;
#pragma unroll 2
  for (uint32_t t = 0; t < (uint32_t)zc; t++) {
    step_ops<VW> nxt;
    if (t + 1 < (uint32_t)zc) load(t + 1, nxt);
    if (pd > 0 && t + (uint32_t)pd < (uint32_t)zc) {
      uint32_t zf = zdd + (uint32_t)pd;
      if (zf >= L) zf -= L;
      prefetch_l2(q0b + (zf * plane + drowA) * W);
      prefetch_l2(q1b + (zf * plane + drowA) * W);
    }
    const uint32_t z = z0 + t, zo = z * plane, rowoff = (y + z + p) & 1;
#pragma unroll
    for (int site = 0; site < 2; site++) {
      const uint32_t jb6 = (cur.jb2 >> (8 * site)) & 0xffu;
      const uint32_t mE = jmask(jb6, 0), mN = jmask(jb6, 1), mU = jmask(jb6, 2);
      const uint32_t mO = jmask(jb6, 3), mS = jmask(jb6, 4), mD = jmask(jb6, 5);
#pragma unroll
      for (int w = 0; w < VW; w++) {
        const int o = site * VW + w;
        const uint32_t cA = v0[w], cB = v0[VW + w], ex = cur.ext[w];
        const uint32_t nE = site == 0 ? (rowoff ? cB : cA) : (rowoff ? ex : cB);
        const uint32_t nO = site == 0 ? (rowoff ? cA : ex) : (rowoff ? cB : cA);
        const uint32_t sw = cur.own[o];
        const uint32_t f0 = xor3(sw, nE, mE), f1 = xor3(sw, cur.vn[o], mN), f2 = xor3(sw, cur.up[o], mU);
        const uint32_t f3 = xor3(sw, nO, mO), f4 = xor3(sw, cur.vs[o], mS), f5 = xor3(sw, vm[o], mD);
        const uint32_t j1 = xor3(f0, f1, f2), j2 = maj3(f0, f1, f2);
        const uint32_t j3 = xor3(f3, f4, f5), j4 = maj3(f3, f4, f5);
        cur.own[o] = sw ^ isi_update(j1, j2, j3, j4, cur.a0[o], cur.a1[o]);
      }
    }
    PR::st(mine + (zo + row) * W, W, cur.own, keep);
    const uint32_t sa = (zdd * plane + drowA) * W;
    if (dpair) {
      PR::st(q0b + sa, W, cur.a0, strm);
      PR::st(q1b + sa, W, cur.a1, strm);
    } else {
      const uint32_t sb = (zdd * plane + drowB) * W;
      uint32_t x0[VW], x1[VW], y0[VW], y1[VW];
#pragma unroll
      for (int w = 0; w < VW; w++) {
        x0[w] = cur.a0[w]; x1[w] = cur.a0[VW + w];
        y0[w] = cur.a1[w]; y1[w] = cur.a1[VW + w];
      }
      hint<VW>::st(q0b + sa, x0, strm);
      hint<VW>::st(q0b + sb, x1, strm);
      hint<VW>::st(q1b + sa, y0, strm);
      hint<VW>::st(q1b + sb, y1, strm);
    }
#pragma unroll
    for (int w = 0; w < N; w++) {
      vm[w] = v0[w];
      v0[w] = cur.up[w];
    }
    zdd = (zdd + 1 == L) ? 0 : zdd + 1;
    cur = nxt;
  }
}

/* ------------------------------------------------------ Philox + LUT bits */

/* Philox4x32-10 (Salmon et al., SC'11): 10 rounds, Weyl key schedule. */
__device__ __forceinline__ void philox10(uint32_t (&v)[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int rd = 0; rd < 10; rd++) {
    if (rd) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * v[0], hi0 = __umulhi(0xD2511F53u, v[0]);
    const uint32_t lo1 = 0xCD9E8D57u * v[2], hi1 = __umulhi(0xCD9E8D57u, v[2]);
    const uint32_t n0 = hi1 ^ v[1] ^ k0, n2 = hi0 ^ v[3] ^ k1;
    v[0] = n0; v[1] = lo1; v[2] = n2; v[3] = lo0;
  }
}

/* first threshold above the 64-bit uniform (hi, lo), with the 10-bit
 * prebisection table (main.cu:615-630) */
__device__ __forceinline__ uint32_t lut_bisect(uint32_t hi, uint32_t lo, const uint32_t *thr,
                                               const uint16_t *pre) {
#define MICSA_BELOW(ix) ((hi == thr[2 * (ix)]) ? (lo < thr[2 * (ix) + 1]) : (hi < thr[2 * (ix)]))
  uint32_t a = 255, b = 255;
  if (MICSA_BELOW(254)) {
    const uint32_t e = pre[hi >> 22];
    a = e & 255u;
    b = e >> 8;
  }
  /* a <= b (checked when the LUT is uploaded): at most 8 halvings */
  for (int step = 0; step < 8 && b - a > 1; step++) {
    const uint32_t mid = (a + b) >> 1;
    if (MICSA_BELOW(mid)) b = mid; else a = mid;
  }
  return MICSA_BELOW(a) ? a : b;
#undef MICSA_BELOW
}

/* one 32-bit word of Bernoulli bits from one Philox call, with the
 * reference's counter bump, post-mix and rotation (main.cu:597-644) */
__device__ __forceinline__ uint32_t heat_bath_word(uint32_t (&c)[4], uint32_t k0, uint32_t k1,
                                                   const uint32_t *thr, const uint16_t *pre) {
  uint32_t v[4] = {c[0], c[1], c[2], c[3]};
  philox10(v, k0, k1);
  c[0]++;
  const uint32_t hi = v[0] ^ v[2], lo = v[1] ^ v[3];
  uint32_t l[4];
  l[0] = ((v[1] << 17) | (v[0] >> 15)) ^ hi ^ ((hi << 21) | (lo >> 11));
  l[1] = ((v[0] << 17) | (v[1] >> 15)) ^ lo ^ (lo << 21);
  l[2] = (hi << 28) | (lo >> 4);
  l[3] = (lo << 28) | (hi >> 4);
  const uint32_t rot = (l[0] + v[1] + l[2] + v[3]) >> 27;
  uint32_t bb = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) bb |= lut_bisect(v[k], l[k], thr, pre) << (8 * k);
  return __funnelshift_l(bb, bb, rot);
}

/* Thread (h, r) = tid = h*nr + r, exactly the reference's thread id, key
 * (tid, keys[r]) and counter te[r] with z += tid; the three 64-bit words
 * (bit = block) are transposed in-warp to replica words of the 64 sites. */
__global__ void __launch_bounds__(TPB)
k_gen_rnd(const micsa_geo g, const int p, const uint32_t *__restrict__ te,
          const uint32_t *__restrict__ keys, const uint8_t *__restrict__ lut,
          uint32_t *__restrict__ rnd) {
  __shared__ uint32_t s_thr[512];
  __shared__ uint16_t s_pre[1024];
  const uint32_t *lw = reinterpret_cast<const uint32_t *>(lut);
  for (int t = threadIdx.x; t < 1024; t += TPB) {
    const uint32_t v = lw[t];
    if (t < 512) s_thr[t] = v;
    else {
      s_pre[2 * (t - 512)] = (uint16_t)(v & 0xffffu);
      s_pre[2 * (t - 512) + 1] = (uint16_t)(v >> 16);
    }
  }
  __syncthreads();
  const int64_t tid = (int64_t)blockIdx.x * TPB + threadIdx.x;
  if (tid >= g.H * g.nr) return; /* warp-uniform: H*nr is a multiple of 32 */
  const int lane = threadIdx.x & 31;
  const int r = (int)(tid % g.nr);
  const int64_t h = tid / g.nr;
  uint32_t c[4] = {te[4 * r], te[4 * r + 1], te[4 * r + 2] + (uint32_t)tid, te[4 * r + 3]};
  const uint32_t key1 = keys[r];
  uint32_t wd[6];
#pragma unroll
  for (int q = 0; q < 6; q++) wd[q] = heat_bath_word(c, (uint32_t)tid, key1, s_thr, s_pre);
  const site_xyz a = ref_site(g, p, h, lane), b = ref_site(g, p, h, lane + 32);
  const int64_t ia = ((int64_t)a.z * g.L + a.y) * g.Lh + (a.x >> 1);
  const int64_t ib = ((int64_t)b.z * g.L + b.y) * g.Lh + (b.x >> 1);
  const int w = r >> 5;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    /* 64-bit word k = (wd[2k] << 32) | wd[2k+1]; bit b = block b */
    const uint32_t lo = warp_transpose32(wd[2 * k + 1], lane);
    const uint32_t hi = warp_transpose32(wd[2 * k], lane);
    rnd[((int64_t)k * g.P + ia) * g.W + w] = lo;
    rnd[((int64_t)k * g.P + ib) * g.W + w] = hi;
  }
}

__global__ void k_walk_advance(const micsa_geo g, int *walk, int ns, int period) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < ns && !micsa_frozen(g, s)) {
    const int k = walk[s] + 1;
    walk[s] = (k == period) ? 0 : k;
  }
}

/* --------------------------------------------------- layout conversion */

/* Warp per (h, word w): lane l reads replica 32w+l of reference word h
 * (64 sites), the transpose gives lane l the replica word of block l and
 * block l+32. */
__global__ void __launch_bounds__(TPB)
k_from_ref(const micsa_geo g, const int p, const int ic, const int k,
           const uint64_t *__restrict__ ref, uint32_t *__restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (TPB / 32);
  for (int64_t wi = (int64_t)blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); wi < g.H * g.W;
       wi += nwarps) {
    const int64_t h = wi / g.W;
    const int w = (int)(wi % g.W);
    const uint64_t v = ref[h * g.nr + w * 32 + lane];
    const uint32_t lo = warp_transpose32((uint32_t)v, lane);
    const uint32_t hi = warp_transpose32((uint32_t)(v >> 32), lane);
    const site_xyz a = ref_site(g, p, h, lane), b = ref_site(g, p, h, lane + 32);
    dst[demon_slot(g, p, ic, k, a.x, a.y, a.z) * g.W + w] = lo;
    dst[demon_slot(g, p, ic, k, b.x, b.y, b.z) * g.W + w] = hi;
  }
}

/* Coupling words of one sample, J[(p*6 + d)*H + h] as CopyDataOnDevice
 * gathers them (main.cu:436-455), -> one bond byte per site (bit d = bond
 * in direction d).  The backward words of blocks on the lattice's low edge
 * along an axis are realigned first, by the block-edge rotation toward -x,
 * -y, -z that d_oneMCstepBN applies to them (RotateO/S/D, main.cu:732-742,
 * 910-927): the bit of block b receives the bit of block b-1 along the axis.
 * Thread per (p, h, bit). */
__device__ __forceinline__ uint64_t rot_back_word(int d, uint64_t v) {
  if (d == 3) { const uint64_t m = 0x8888888888888888ULL; return ((v & m) >> 3) | ((v & ~m) << 1); }
  if (d == 4) { const uint64_t m = 0xF000F000F000F000ULL; return ((v & m) >> 12) | ((v & ~m) << 4); }
  const uint64_t m = 0xFFFF000000000000ULL;
  return ((v & m) >> 48) | ((v & ~m) << 16);
}

__global__ void __launch_bounds__(TPB)
k_couplings_from_ref(const micsa_geo g, const uint64_t *__restrict__ J, uint8_t *__restrict__ jb) {
  const int64_t n = 2 * g.H * 64;
  const int m = g.L >> 2, mh = m >> 1;
  for (int64_t i = (int64_t)blockIdx.x * TPB + threadIdx.x; i < n; i += (int64_t)gridDim.x * TPB) {
    const int bit = (int)(i & 63);
    const int64_t ph = i >> 6;
    const int p = (int)(ph / g.H);
    const int64_t h = ph - (int64_t)p * g.H;
    const int64_t q = h / mh;
    const int bb = (int)(q % m), c = (int)(q / m);
    const int a = 2 * (int)(h % mh) + ((bb + c + p) & 1);
    const int edge[3] = {a == 0, bb == 0, c == 0};
    uint32_t v = 0;
#pragma unroll
    for (int d = 0; d < 6; d++) {
      uint64_t w = J[((int64_t)p * 6 + d) * g.H + h];
      if (d >= 3 && edge[d - 3]) w = rot_back_word(d, w);
      v |= (uint32_t)((w >> bit) & 1) << d;
    }
    const site_xyz s = ref_site(g, p, h, bit);
    jb[(int64_t)p * g.P + ((int64_t)s.z * g.L + s.y) * g.Lh + (s.x >> 1)] = (uint8_t)v;
  }
}

__global__ void __launch_bounds__(TPB)
k_to_ref(const micsa_geo g, const int p, const int ic, const int *__restrict__ walk,
         const int sample, const uint32_t *__restrict__ src, uint64_t *__restrict__ ref) {
  const int lane = threadIdx.x & 31;
  const int k = walk ? walk[sample] : 0;
  const int64_t nwarps = (int64_t)gridDim.x * (TPB / 32);
  for (int64_t wi = (int64_t)blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); wi < g.H * g.W;
       wi += nwarps) {
    const int64_t h = wi / g.W;
    const int w = (int)(wi % g.W);
    const site_xyz a = ref_site(g, p, h, lane), b = ref_site(g, p, h, lane + 32);
    const uint32_t lo = warp_transpose32(src[demon_slot(g, p, ic, k, a.x, a.y, a.z) * g.W + w], lane);
    const uint32_t hi = warp_transpose32(src[demon_slot(g, p, ic, k, b.x, b.y, b.z) * g.W + w], lane);
    ref[h * g.nr + w * 32 + lane] = (uint64_t)lo | ((uint64_t)hi << 32);
  }
}

/* ---------------------------------------------------------- measurement */

/* Per-replica counts of one lane, bit-sliced (bit r of every word belongs
 * to replica r of the lane's 32-replica word): a carry-save accumulator of
 * weights 1, 2, 4 and 8 (full adders as three-input LOP3s) in front of a
 * ripple counter of sixteens, so that adding a word costs about two logic
 * operations; one warp transpose per bit slice at the end turns the slices
 * into counts per replica.  Capacity: 1023 per lane and replica. */
constexpr int VC_HI = 6;
struct vcount {
  uint32_t ones = 0, twos = 0, fours = 0, eights = 0, hi[VC_HI] = {0, 0, 0, 0, 0, 0};
  static __device__ __forceinline__ void half(uint32_t &acc, uint32_t a, uint32_t &c) {
    c = acc & a;
    acc ^= a;
  }
  static __device__ __forceinline__ void full(uint32_t &acc, uint32_t a, uint32_t b, uint32_t &c) {
    c = maj3(acc, a, b);
    acc = xor3(acc, a, b);
  }
  __device__ __forceinline__ void ripple(uint32_t c) {
#pragma unroll
    for (int k = 0; k < VC_HI; k++) {
      const uint32_t t = hi[k] & c;
      hi[k] ^= c;
      c = t;
    }
  }
  /* a0..a3 with weight 1, b0..b3 with weight 2 (at most 12 per call) */
  __device__ __forceinline__ void add8(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                       uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
    uint32_t c1, c2, d1, d2, d3, e1, e2, f;
    full(ones, a0, a1, c1);
    full(ones, a2, a3, c2);
    full(twos, c1, c2, d1);
    full(twos, b0, b1, d2);
    full(twos, b2, b3, d3);
    full(fours, d1, d2, e1);
    half(fours, d3, e2);
    full(eights, e1, e2, f);
    ripple(f);
  }
  /* the bits of a count c = b0 + 2 b1 + 4 b2 (at most 7 per call) */
  __device__ __forceinline__ void add3(uint32_t b0, uint32_t b1, uint32_t b2) {
    uint32_t c1, c2, c3, c4;
    half(ones, b0, c1);
    full(twos, b1, c1, c2);
    full(fours, b2, c2, c3);
    half(eights, c3, c4);
    ripple(c4);
  }
  /* the warp's total for replica `lane` (all 32 lanes must call) */
  __device__ __forceinline__ unsigned long long reduce(int lane) const {
    unsigned long long t = __popc(warp_transpose32(ones, lane)) +
                           2ull * __popc(warp_transpose32(twos, lane)) +
                           4ull * __popc(warp_transpose32(fours, lane)) +
                           8ull * __popc(warp_transpose32(eights, lane));
#pragma unroll
    for (int k = 0; k < VC_HI; k++) t += (16ull << k) * __popc(warp_transpose32(hi[k], lane));
    return t;
  }
};

/* Adds v (lane l: the warp's total for replica l) of every warp of the block
 * into out[l]: one atomic per lane and block instead of one per warp.  All
 * threads of the block must call; buf holds TPB/32 * 32 entries. */
__device__ __forceinline__ void block_add(unsigned long long v, unsigned long long *buf,
                                          unsigned long long *out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  buf[warp * 32 + lane] = v;
  __syncthreads();
  if (warp == 0) {
    unsigned long long t = 0;
#pragma unroll
    for (int k = 0; k < TPB / 32; k++) t += buf[k * 32 + lane];
    atomicAdd(out + lane, t);
  }
  __syncthreads();
}

/* Unsatisfied bonds per replica, summed over the 6 bonds of every colour-0
 * site (each bond has exactly one colour-0 end).  blockIdx.y = word w,
 * blockIdx.z = sample; warps stride over chunks of 32 sites (at most 128
 * sites per lane: the launch sizes the grid for it).  Site offsets are
 * 32-bit (P*W < 2^32 is checked at creation). */
__global__ void __launch_bounds__(TPB)
k_energy(const micsa_geo g, const uint32_t *__restrict__ spin, const uint8_t *__restrict__ jb,
         unsigned long long *__restrict__ unsat) {
  __shared__ unsigned long long buf[TPB];
  const int s = blockIdx.z, w = blockIdx.y, lane = threadIdx.x & 31;
  if (micsa_frozen(g, s)) return;
  const uint32_t L = g.L, Lh = g.Lh, W = g.W, P = (uint32_t)g.P;
  const uint32_t *mine = spin + (size_t)(s * 2) * P * W + w;
  const uint32_t *oth = spin + (size_t)(s * 2 + 1) * P * W + w;
  const uint8_t *jbs = jb + (size_t)(s * 2) * P;
  vcount cnt;
  const uint32_t step = gridDim.x * TPB;
  for (uint32_t base = blockIdx.x * TPB + (threadIdx.x & ~31u); base < P; base += step) {
    const uint32_t i = base + lane; /* P is a multiple of 32: all lanes valid */
    const uint32_t xh = i % Lh, q = i / Lh;
    const uint32_t y = q % L, z = q / L;
    const uint32_t rowoff = (y + z) & 1;
    uint32_t xe = xh + rowoff; if (xe == Lh) xe = 0;
    const uint32_t xo = (xh + rowoff == 0) ? Lh - 1 : xh + rowoff - 1;
    const uint32_t yp = (y + 1 == L) ? 0 : y + 1, ym = (y == 0) ? L - 1 : y - 1;
    const uint32_t zp = (z + 1 == L) ? 0 : z + 1, zm = (z == 0) ? L - 1 : z - 1;
    const uint32_t row = z * L;
    const uint32_t sw = __ldg(mine + i * W);
    const uint32_t jbits = __ldg(jbs + i);
    const uint32_t f0 = sw ^ __ldg(oth + ((row + y) * Lh + xe) * W) ^ jmask(jbits, 0);
    const uint32_t f1 = sw ^ __ldg(oth + ((row + yp) * Lh + xh) * W) ^ jmask(jbits, 1);
    const uint32_t f2 = sw ^ __ldg(oth + ((zp * L + y) * Lh + xh) * W) ^ jmask(jbits, 2);
    const uint32_t f3 = sw ^ __ldg(oth + ((row + y) * Lh + xo) * W) ^ jmask(jbits, 3);
    const uint32_t f4 = sw ^ __ldg(oth + ((row + ym) * Lh + xh) * W) ^ jmask(jbits, 4);
    const uint32_t f5 = sw ^ __ldg(oth + ((zm * L + y) * Lh + xh) * W) ^ jmask(jbits, 5);
    /* bit-sliced sum of six bits: c = b0 + 2 b1 + 4 b2 */
    const uint32_t sa = xor3(f0, f1, f2), ca = maj3(f0, f1, f2);
    const uint32_t sb = xor3(f3, f4, f5), cb = maj3(f3, f4, f5);
    const uint32_t b0 = sa ^ sb, c0 = sa & sb;
    cnt.add3(b0, xor3(ca, cb, c0), maj3(ca, cb, c0));
  }
  block_add(cnt.reduce(lane), buf, unsat + (int64_t)s * g.nr + w * 32);
}

/* Demon energy per replica: blockIdx.y = (plane pi = p*nc + ic)*W + w. */
__global__ void __launch_bounds__(TPB)
k_demon_energy(const micsa_geo g, const uint32_t *__restrict__ d0, const uint32_t *__restrict__ d1,
               unsigned long long *__restrict__ dem) {
  const int s = blockIdx.z, lane = threadIdx.x & 31;
  if (micsa_frozen(g, s)) return;
  const int w = blockIdx.y % g.W, pi = blockIdx.y / g.W;
  const int64_t P = g.P, off = ((int64_t)s * 2 * g.nc + pi) * P * g.W + w;
  unsigned long long acc = 0;
  const int64_t step = (int64_t)gridDim.x * TPB;
  for (int64_t base = (int64_t)blockIdx.x * TPB + (threadIdx.x & ~31); base < P; base += step) {
    const int64_t i = base + lane;
    const uint32_t a = __ldcs(d0 + off + i * g.W), b = __ldcs(d1 + off + i * g.W);
    acc += __popc(warp_transpose32(a, lane)) + 2u * __popc(warp_transpose32(b, lane));
  }
  atomicAdd(dem + (int64_t)s * g.nr + w * 32 + lane, acc);
}

/* Demon energy with 16-byte loads, for W in {1, 2, 4}: a plane (sample s,
 * plane pi) is P*W consecutive words; component c of a 4-word vector at
 * word 4k is word w = c % W of its site (4 % W == 0).  A lane loads four
 * vectors of each demon array per trip (lane-contiguous, 512 bytes per warp
 * and load) and adds component c's words into the bit-sliced counter of
 * word c % W, D0 with weight 1 and D1 with weight 2; the counters are
 * transposed into per-replica counts once, at the end.  At most 16 trips
 * per lane (the launch sizes the grid for it) keep every counter within its
 * capacity.  blockIdx.y = s*2*nc + pi; blocks stride over the plane. */
template <int W>
__global__ void __launch_bounds__(TPB)
k_demon_energy_cs(const micsa_geo g, const uint32_t *__restrict__ d0,
                  const uint32_t *__restrict__ d1, unsigned long long *__restrict__ dem) {
  __shared__ unsigned long long buf[TPB];
  const int plane = blockIdx.y, s = plane / (2 * g.nc), lane = threadIdx.x & 31;
  if (micsa_frozen(g, s)) return;
  const uint32_t nvec = (uint32_t)(g.P * W / 4);
  const uint4 *a = (const uint4 *)(d0 + (int64_t)plane * g.P * W);
  const uint4 *b = (const uint4 *)(d1 + (int64_t)plane * g.P * W);
  vcount cnt[W];
  const uint32_t stride = gridDim.x * TPB * 4;
  for (uint32_t v0 = (blockIdx.x * TPB + (threadIdx.x & ~31u)) * 4; v0 < nvec; v0 += stride) {
    uint4 x[4], y[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint32_t v = v0 + k * 32 + lane;
      x[k] = v < nvec ? __ldcs(a + v) : make_uint4(0, 0, 0, 0);
      y[k] = v < nvec ? __ldcs(b + v) : make_uint4(0, 0, 0, 0);
    }
    cnt[0].add8(x[0].x, x[1].x, x[2].x, x[3].x, y[0].x, y[1].x, y[2].x, y[3].x);
    cnt[1 % W].add8(x[0].y, x[1].y, x[2].y, x[3].y, y[0].y, y[1].y, y[2].y, y[3].y);
    cnt[2 % W].add8(x[0].z, x[1].z, x[2].z, x[3].z, y[0].z, y[1].z, y[2].z, y[3].z);
    cnt[3 % W].add8(x[0].w, x[1].w, x[2].w, x[3].w, y[0].w, y[1].w, y[2].w, y[3].w);
  }
#pragma unroll
  for (int w = 0; w < W; w++) block_add(cnt[w].reduce(lane), buf, dem + (int64_t)s * g.nr + w * 32);
}

/* Overlap and C4 of the replica pairs (2k, 2k+1): with t = s(x) ^ s(x'),
 * bit 2k of t ^ (t >> 1) is d_x xor d_x', d = a xor b the pair difference.
 * blockIdx.y = axis*nd + dist (dist 0 also yields q via x' = x and the
 * second pass below), blockIdx.z = s*W + w.  Sites in natural order. */
__global__ void __launch_bounds__(TPB)
k_overlap(const micsa_geo g, const uint32_t *__restrict__ spin, unsigned long long *__restrict__ qd,
          unsigned long long *__restrict__ c4d) {
  const int nd = g.L / 2 + 1;
  const int axis = blockIdx.y / nd, dist = blockIdx.y % nd;
  const int s = blockIdx.z / g.W, w = blockIdx.z % g.W, lane = threadIdx.x & 31;
  if (micsa_frozen(g, s)) return;
  const int L = g.L, Lh = g.Lh, W = g.W;
  const int64_t P = g.P, V = 2 * P;
  const uint32_t *sp = spin + (int64_t)(s * 2) * P * W + w;
  unsigned long long acc = 0, accq = 0;
  const bool want_q = (axis == 0 && dist == 0);
  const int64_t step = (int64_t)gridDim.x * TPB;
  for (int64_t base = (int64_t)blockIdx.x * TPB + (threadIdx.x & ~31); base < V; base += step) {
    const int64_t n = base + lane; /* V is a multiple of 32 */
    const int x = (int)(n % L);
    const int64_t q = n / L;
    const int y = (int)(q % L), z = (int)(q / L);
    int x2 = x, y2 = y, z2 = z;
    if (axis == 0) { x2 += dist; if (x2 >= L) x2 -= L; }
    else if (axis == 1) { y2 += dist; if (y2 >= L) y2 -= L; }
    else { z2 += dist; if (z2 >= L) z2 -= L; }
    const uint32_t s1 = __ldg(sp + ((int64_t)((x + y + z) & 1) * P + ((int64_t)z * L + y) * Lh + (x >> 1)) * W);
    const uint32_t s2 = __ldg(sp + ((int64_t)((x2 + y2 + z2) & 1) * P + ((int64_t)z2 * L + y2) * Lh + (x2 >> 1)) * W);
    const uint32_t t = s1 ^ s2;
    acc += __popc(warp_transpose32(t ^ (t >> 1), lane));
    if (want_q) accq += __popc(warp_transpose32(s1 ^ (s1 >> 1), lane));
  }
  if (!(lane & 1)) {
    const int k = w * 16 + (lane >> 1);
    atomicAdd(c4d + (((int64_t)s * (g.nr / 2) + k) * 3 + axis) * nd + dist, acc);
    if (want_q) atomicAdd(qd + (int64_t)s * (g.nr / 2) + k, accq);
  }
}

/* Sweep launches with programmatic dependent launch (g.pdl): the next
 * half-sweep's blocks are scheduled while this one drains and wait in
 * griddepcontrol.wait (the kernels' first statement after the trigger) until
 * it has completed and its writes are visible -- the same ordering as a plain
 * launch, without the launch gap between the two grids. */
template <typename... KArgs, typename... Args>
cudaError_t launch_sweep(const micsa_geo &g, void (*k)(KArgs...), dim3 grid, dim3 block,
                         size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t c = {};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = smem;
  c.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = g.pdl ? 1 : 0;
  c.attrs = at;
  c.numAttrs = 1;
  return cudaLaunchKernelEx(&c, k, args...);
}

inline int blocks_for(int64_t n, int per_block) {
  int64_t b = (n + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > 2147483647LL) b = 2147483647LL;
  return (int)b;
}

} /* namespace */

/* ------------------------------------------------------------ launchers */

/* tile of the sweep for this L: tx pairs along x/2 (the largest power of two
 * <= 32 dividing L/4, L/4 even) x ty rows, ty*tx = TPB threads */
/* Block shape of the sweeps: tx threads along x (two x/2 positions each) by
 * ty rows.  Default: the largest power of two up to 32 dividing L/4.  Whole
 * rows (wide, when L/4 is not already that and fits a block): a row's demon
 * words are then read as one run, so the x translation of the demon walk
 * shifts one run instead of misaligning several short ones. */
static void sweep_tile(int L, int wide, int *tx, int *ty, int S = 2) {
  const int cols = L / 2 / S; /* threads a row needs */
  int x = 32;
  while (cols % x) x >>= 1;
  if (wide && cols <= TPB / 2) x = cols;
  *tx = x;
  *ty = TPB / x;
}

template <int VW>
static cudaError_t sweep_vw(const micsa_geo &g, int p, int ic, bool micsa, uint32_t *spin,
                            uint32_t *d0, uint32_t *d1, const uint8_t *jb, const int *walk,
                            const uint32_t *rnd, const micsa_tma *tm, cudaStream_t st) {
  const int G = g.W / VW;
  int tx, ty;
  sweep_tile(g.L, g.tw, &tx, &ty);
  const int ytiles = (g.L + ty - 1) / ty;
  /* z chunk per thread: long columns at large L, more threads at small L */
  const int zc = g.zc > 0 ? g.zc : ((g.L >= 128 && g.L % 16 == 0) ? 16 : (g.L >= 48 ? 8 : 2));
  dim3 block(tx, ty);
  dim3 grid(g.Lh / 2 / tx, ytiles * g.ns * G, g.L / zc);
  /* blocks per SM the register allocation is made for: the default (3, or
   * 2 for 4-word vectors), or occ = 4 (at most 64 registers, VW <= 2) */
  constexpr int B0 = VW == 4 ? 2 : 3, B1 = VW == 4 ? 2 : 4;
  /* TMA-staged demon tiles: one word group per site, whole row tiles, at
   * most 4 planes per block (shared memory 2*zc tiles + zc barriers) */
  const bool tma = micsa && tm && tm->ok && g.tma && G == 1 && g.L % ty == 0 && zc <= 4 &&
                   tm->ty == ty && tm->box_w >= 2 * tx * VW;
  const size_t smem = tma ? (size_t)2 * zc * ty * tm->box_w * 4 + (size_t)zc * 8 : 0;
  if (VW == 2 && micsa && g.async && G == 1 && !tma) {
    const size_t sb = (size_t)2 * ASYNC_ITEMS * TPB * 16;
    cudaError_t e;
    if (g.occ == 4) {
      if ((e = cudaFuncSetAttribute(k_sweep_async<B1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sb)) != cudaSuccess) return e;
      if ((e = launch_sweep(g, k_sweep_async<B1>, grid, block, sb, st, g, p, ic, ytiles, zc, spin, d0,
                            d1, jb, walk)) != cudaSuccess) return e;
    } else {
      if ((e = cudaFuncSetAttribute(k_sweep_async<B0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sb)) != cudaSuccess) return e;
      if ((e = launch_sweep(g, k_sweep_async<B0>, grid, block, sb, st, g, p, ic, ytiles, zc, spin, d0,
                            d1, jb, walk)) != cudaSuccess) return e;
    }
    return cudaGetLastError();
  }
  if (micsa && g.pipe && !tma) {
    /* register budgets: 2 blocks per SM (128 registers; always for 4-word
     * vectors) or 3 (85) */
    const bool b2 = g.occ == 2 || VW == 4;
    if (G == 1)
      return b2 ? launch_sweep(g, k_sweep_pipe<VW, true, 2>, grid, block, 0, st, g, p, ic, ytiles, G,
                               zc, g.pd, spin, d0, d1, jb, walk)
                : launch_sweep(g, k_sweep_pipe<VW, true, 3>, grid, block, 0, st, g, p, ic, ytiles, G,
                               zc, g.pd, spin, d0, d1, jb, walk);
    return b2 ? launch_sweep(g, k_sweep_pipe<VW, false, 2>, grid, block, 0, st, g, p, ic, ytiles, G, zc,
                             g.pd, spin, d0, d1, jb, walk)
              : launch_sweep(g, k_sweep_pipe<VW, false, 3>, grid, block, 0, st, g, p, ic, ytiles, G, zc,
                             g.pd, spin, d0, d1, jb, walk);
  }
  micsa_tma none;
  const micsa_tma &t = tm ? *tm : none;
  if constexpr (VW == 1) {
    if (micsa && g.quad && G == 1 && !tma) { /* four one-word sites per thread */
      int qx, qy;
      sweep_tile(g.L, g.tw, &qx, &qy, 4);
      const int qyt = (g.L + qy - 1) / qy;
      const dim3 qgrid(g.Lh / 4 / qx, qyt * g.ns, g.L / zc);
      const cudaError_t e = g.occ == 4
          ? launch_sweep(g, k_sweep<1, true, true, B1, false, 4>, qgrid, dim3(qx, qy), 0, st, g, p, ic,
                         qyt, G, zc, g.pd, spin, d0, d1, jb, walk, rnd, t)
          : launch_sweep(g, k_sweep<1, true, true, B0, false, 4>, qgrid, dim3(qx, qy), 0, st, g, p, ic,
                         qyt, G, zc, g.pd, spin, d0, d1, jb, walk, rnd, t);
      return e != cudaSuccess ? e : cudaGetLastError();
    }
  }
#define MICSA_SWEEP(M, WD, B, T)                                                                  \
  do {                                                                                            \
    if (T && smem > 48 * 1024) {                                                                  \
      const cudaError_t e_ = cudaFuncSetAttribute(k_sweep<VW, M, WD, B, T>,                       \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                                  (int)smem);                                     \
      if (e_ != cudaSuccess) return e_;                                                           \
    }                                                                                             \
    const cudaError_t l_ = launch_sweep(g, k_sweep<VW, M, WD, B, T>, grid, block, smem, st, g, p, \
                                        ic, ytiles, G, zc, g.pd, spin, d0, d1, jb, walk, rnd, t);  \
    if (l_ != cudaSuccess) return l_;                                                             \
  } while (0)
  if (G == 1) {
    if (micsa) {
      if (tma) { if (g.occ == 4) MICSA_SWEEP(true, true, B1, true); else MICSA_SWEEP(true, true, B0, true); }
      else { if (g.occ == 4) MICSA_SWEEP(true, true, B1, false); else MICSA_SWEEP(true, true, B0, false); }
    } else {
      MICSA_SWEEP(false, true, B0, false);
    }
  } else {
    if (micsa) { if (g.occ == 4) MICSA_SWEEP(true, false, B1, false); else MICSA_SWEEP(true, false, B0, false); }
    else MICSA_SWEEP(false, false, B0, false);
  }
#undef MICSA_SWEEP
  return cudaGetLastError();
}

/* the dataflow sweep: one block per tile, or (g.pers) the persistent form
 * with as many blocks as fit the GPU at once */
template <int VW, bool WIDE, int MINB>
static cudaError_t sweep_flow_k(const micsa_geo &g, int smaj, int ytiles, int G, int zc,
                                dim3 block, int64_t tiles, uint32_t *spin, uint32_t *d0,
                                uint32_t *d1, const uint8_t *jb, const int *walk, unsigned *ctl,
                                cudaStream_t st) {
  if (g.pers) {
    int dev = 0, nsm = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_pdep<VW, WIDE, MINB>,
                                                        (int)(block.x * block.y), 0);
    if (e != cudaSuccess) return e;
    int64_t nb = (int64_t)nsm * (per > 0 ? per : 1);
    if (nb > tiles) nb = tiles;
    return launch_sweep(g, k_sweep_pdep<VW, WIDE, MINB>, dim3((unsigned)nb), block, 0, st, g,
                        ytiles, G, zc, g.pd, smaj, (unsigned)tiles, spin, d0, d1, jb, walk, ctl);
  }
  if (g.half) /* half-height tiles: the same registers per thread, twice the blocks per SM */
    return launch_sweep(g, k_sweep_dep<VW, WIDE, 2 * MINB, TPB / 2>, dim3((unsigned)tiles), block,
                        0, st, g, ytiles, G, zc, g.pd, smaj, g.pf, spin, d0, d1, jb, walk, ctl);
  if (g.xs) /* the x halo by warp shuffle */
    return launch_sweep(g, k_sweep_dep<VW, WIDE, MINB, TPB, true>, dim3((unsigned)tiles), block,
                        0, st, g, ytiles, G, zc, g.pd, smaj, g.pf, spin, d0, d1, jb, walk, ctl);
  return launch_sweep(g, k_sweep_dep<VW, WIDE, MINB>, dim3((unsigned)tiles), block, 0, st, g,
                      ytiles, G, zc, g.pd, smaj, g.pf, spin, d0, d1, jb, walk, ctl);
}

template <int VW>
static cudaError_t sweep_flow_vw(const micsa_geo &g, int smaj, uint32_t *spin, uint32_t *d0,
                                 uint32_t *d1, const uint8_t *jb, const int *walk, unsigned *ctl,
                                 cudaStream_t st) {
  const int G = g.W / VW;
  int tx, ty;
  sweep_tile(g.L, g.tw, &tx, &ty);
  if (g.half && !g.pers) ty = ty / 2 > 0 ? ty / 2 : 1; /* blocks of tx x ty/2 threads */
  const int ytiles = (g.L + ty - 1) / ty;
  const int zc = g.zc > 0 ? g.zc : 4;
  if (g.L % zc) return cudaErrorInvalidValue;
  const int64_t tiles = (int64_t)(g.fit > 1 ? g.fit : 1) * g.ns * 2 * g.nc * (g.L / zc) *
                        (g.Lh / 2 / tx) * ytiles * G;
  if (tiles >= (1LL << 31)) return cudaErrorInvalidValue; /* 32-bit tickets */
  const dim3 block(tx, ty);
  constexpr int B0 = VW == 4 ? 2 : 3, B1 = VW == 4 ? 2 : 4;
  if (G == 1)
    return g.occ == 4 ? sweep_flow_k<VW, true, B1>(g, smaj, ytiles, G, zc, block, tiles, spin, d0,
                                                   d1, jb, walk, ctl, st)
                      : sweep_flow_k<VW, true, B0>(g, smaj, ytiles, G, zc, block, tiles, spin, d0,
                                                   d1, jb, walk, ctl, st);
  return g.occ == 4 ? sweep_flow_k<VW, false, B1>(g, smaj, ytiles, G, zc, block, tiles, spin, d0,
                                                  d1, jb, walk, ctl, st)
                    : sweep_flow_k<VW, false, B0>(g, smaj, ytiles, G, zc, block, tiles, spin, d0,
                                                  d1, jb, walk, ctl, st);
}

cudaError_t micsa_launch_sweep_flow(const micsa_geo &g, int sample_major, uint32_t *spin,
                                    uint32_t *d0, uint32_t *d1, const uint8_t *jb,
                                    const int *walk, unsigned *ctl, cudaStream_t st) {
  cudaError_t e;
  if (g.W % 4 == 0) e = sweep_flow_vw<4>(g, sample_major, spin, d0, d1, jb, walk, ctl, st);
  else if (g.W % 2 == 0) e = sweep_flow_vw<2>(g, sample_major, spin, d0, d1, jb, walk, ctl, st);
  else e = sweep_flow_vw<1>(g, sample_major, spin, d0, d1, jb, walk, ctl, st);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t micsa_flow_timeout_count(unsigned *n) {
  return cudaMemcpyFromSymbol(n, micsa_flow_timeouts, sizeof(unsigned));
}

cudaError_t micsa_flow_timeout_clear() {
  const unsigned zero = 0;
  return cudaMemcpyToSymbol(micsa_flow_timeouts, &zero, sizeof(unsigned));
}

cudaError_t micsa_flow_set_waits(unsigned long long limit_ns, unsigned need_offset,
                                 cudaStream_t st) {
  cudaError_t e = cudaMemcpyToSymbolAsync(micsa_flow_limit_ns, &limit_ns, sizeof limit_ns, 0,
                                          cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbolAsync(micsa_flow_need_offset, &need_offset, sizeof need_offset, 0,
                                cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st); /* the host values are on this stack */
  return e;
}

cudaError_t micsa_make_tma(const micsa_geo &g, const uint32_t *d0, const uint32_t *d1,
                           micsa_tma *out) {
  memset(out, 0, sizeof *out);
  if (g.W != 1 && g.W != 2 && g.W != 4) return cudaSuccess;
  typedef CUresult (*encode_t)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                               const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                               const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                               CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return cudaSuccess; /* no staged sweep; not an error */
  }
  int tx, ty;
  sweep_tile(g.L, 0, &tx, &ty);
  const cuuint64_t row = (cuuint64_t)g.Lh * g.W; /* words per (plane, y) row */
  /* the tile plus 4 words (16 bytes) for a start rounded down, at most a row */
  int box_w = 2 * tx * g.W + 4;
  if (box_w > (int)row) box_w = (int)row;
  if (box_w > 256 || ty > 256 || box_w % 4 || ty > g.L) return cudaSuccess;
  const cuuint64_t dims[3] = {row, (cuuint64_t)g.L, (cuuint64_t)g.L * g.ns * 2 * g.nc};
  const cuuint64_t strides[2] = {row * 4, row * 4 * (cuuint64_t)g.L};
  const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)ty, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const uint32_t *base[2] = {d0, d1};
  for (int k = 0; k < 2; k++) {
    const CUresult r = ((encode_t)fn)((CUtensorMap *)out->map[k], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3,
                                      (void *)base[k], dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaSuccess;
  }
  out->box_w = box_w;
  out->ty = ty;
  out->ok = 1;
  return cudaSuccess;
}

static cudaError_t sweep_any(const micsa_geo &g, int p, int ic, bool micsa, uint32_t *spin,
                             uint32_t *d0, uint32_t *d1, const uint8_t *jb, const int *walk,
                             const uint32_t *rnd, const micsa_tma *tm, cudaStream_t st) {
  if (g.W % 4 == 0) return sweep_vw<4>(g, p, ic, micsa, spin, d0, d1, jb, walk, rnd, tm, st);
  if (g.W % 2 == 0) return sweep_vw<2>(g, p, ic, micsa, spin, d0, d1, jb, walk, rnd, tm, st);
  return sweep_vw<1>(g, p, ic, micsa, spin, d0, d1, jb, walk, rnd, tm, st);
}

cudaError_t micsa_launch_sweep_micsa(const micsa_geo &g, int p, int ic, uint32_t *spin,
                                     uint32_t *d0, uint32_t *d1, const uint8_t *jb,
                                     const int *walk, const micsa_tma *tm, cudaStream_t st) {
  return sweep_any(g, p, ic, true, spin, d0, d1, jb, walk, nullptr, tm, st);
}

cudaError_t micsa_launch_sweep_metropolis(const micsa_geo &g, int p, uint32_t *spin,
                                          const uint8_t *jb, const uint32_t *rnd,
                                          cudaStream_t st) {
  return sweep_any(g, p, 0, false, spin, nullptr, nullptr, jb, nullptr, rnd, nullptr, st);
}

cudaError_t micsa_launch_gen_rnd(const micsa_geo &g, int p, const uint32_t *te,
                                 const uint32_t *keys, const uint8_t *lut, uint32_t *rnd,
                                 cudaStream_t st) {
  k_gen_rnd<<<blocks_for(g.H * g.nr, TPB), TPB, 0, st>>>(g, p, te, keys, lut, rnd);
  return cudaGetLastError();
}

cudaError_t micsa_launch_walk_advance(const micsa_geo &g, int *walk, cudaStream_t st) {
  k_walk_advance<<<(g.ns + 127) / 128, 128, 0, st>>>(g, walk, g.ns, g.L / 2);
  return cudaGetLastError();
}

cudaError_t micsa_launch_from_ref(const micsa_geo &g, int p, int ic, int k, const uint64_t *ref,
                                  uint32_t *dst, cudaStream_t st) {
  k_from_ref<<<blocks_for(g.H * g.W, TPB / 32), TPB, 0, st>>>(g, p, ic, k, ref, dst);
  return cudaGetLastError();
}

cudaError_t micsa_launch_couplings_from_ref(const micsa_geo &g, const uint64_t *J, uint8_t *jb,
                                            cudaStream_t st) {
  k_couplings_from_ref<<<blocks_for(2 * g.H * 64, TPB), TPB, 0, st>>>(g, J, jb);
  return cudaGetLastError();
}

cudaError_t micsa_launch_to_ref(const micsa_geo &g, int p, int ic, const int *walk, int sample,
                                const uint32_t *src, uint64_t *ref, cudaStream_t st) {
  k_to_ref<<<blocks_for(g.H * g.W, TPB / 32), TPB, 0, st>>>(g, p, ic, walk, sample, src, ref);
  return cudaGetLastError();
}

static int measure_blocks(int64_t sites, int64_t slices) {
  /* enough blocks to fill the GPU, never more than one per 32-site chunk */
  int64_t want = (4 * 152 + slices - 1) / slices;
  int64_t maxb = (sites + TPB - 1) / TPB;
  if (want > maxb) want = maxb;
  return want < 1 ? 1 : (int)want;
}

cudaError_t micsa_launch_energy(const micsa_geo &g, const uint32_t *spin, const uint8_t *jb,
                                unsigned long long *unsat, cudaStream_t st) {
  /* at most 128 sites per lane: the counters hold 1023 per replica */
  int bx = measure_blocks(g.P, (int64_t)g.W * g.ns);
  const int64_t need = (g.P + (int64_t)TPB * 128 - 1) / ((int64_t)TPB * 128);
  if (bx < need) bx = (int)need;
  dim3 grid(bx, g.W, g.ns);
  k_energy<<<grid, TPB, 0, st>>>(g, spin, jb, unsat);
  return cudaGetLastError();
}

cudaError_t micsa_launch_demon_energy(const micsa_geo &g, const uint32_t *d0, const uint32_t *d1,
                                      unsigned long long *dem, cudaStream_t st) {
  if (g.W == 1 || g.W == 2 || g.W == 4) {
    /* at most 16 trips of 4 vectors per lane (counter capacity) */
    const int64_t planes = (int64_t)2 * g.nc * g.ns, nvec = g.P * g.W / 4;
    const int64_t bx = (nvec + (int64_t)TPB * 4 * 16 - 1) / ((int64_t)TPB * 4 * 16);
    const dim3 grid((unsigned)(bx < 1 ? 1 : bx), (unsigned)planes);
    if (g.W == 1) k_demon_energy_cs<1><<<grid, TPB, 0, st>>>(g, d0, d1, dem);
    else if (g.W == 2) k_demon_energy_cs<2><<<grid, TPB, 0, st>>>(g, d0, d1, dem);
    else k_demon_energy_cs<4><<<grid, TPB, 0, st>>>(g, d0, d1, dem);
    return cudaGetLastError();
  }
  dim3 grid(measure_blocks(g.P, (int64_t)2 * g.nc * g.W * g.ns), 2 * g.nc * g.W, g.ns);
  k_demon_energy<<<grid, TPB, 0, st>>>(g, d0, d1, dem);
  return cudaGetLastError();
}

cudaError_t micsa_launch_overlap(const micsa_geo &g, const uint32_t *spin, unsigned long long *qd,
                                 unsigned long long *c4d, cudaStream_t st) {
  const int nd = g.L / 2 + 1;
  dim3 grid(measure_blocks(2 * g.P, (int64_t)3 * nd * g.W * g.ns), 3 * nd, g.ns * g.W);
  k_overlap<<<grid, TPB, 0, st>>>(g, spin, qd, c4d);
  return cudaGetLastError();
}

int micsa_sweep_wide_differs(int L, int sites) {
  int a, b, c, d;
  sweep_tile(L, 0, &a, &b, sites);
  sweep_tile(L, 1, &c, &d, sites);
  return a != c;
}

int micsa_sweep_zc_candidates(int L, int *out, int max) {
  int n = 0;
  for (int zc = 1; zc <= 64 && zc <= L && n < max; zc <<= 1)
    if (L % zc == 0) out[n++] = zc;
  return n;
}

/* ------------------------------------------------------- demon refresh */
/* One refresh (InitWalkers, ini.c:712-781) drawn on the device.  A warp
 * owns 32 replica streams (w*32 + lane) of one sample and one segment of
 * wps CPUwalker words; rec holds each stream's start state grouped by warp,
 * rec[(grp*REFRESH_REC + k)*32 + lane], grp = j*W + w (layout of
 * micsa_stream_record).  The lane jumps its generators to draw m = seg*64*wps:
 *   lagged Fibonacci  x_{m-61+t} = sum_i fib[i] E[i+t] for t < 55, then the
 *                     recurrence gives x_{m-6} .. x_{m-1};
 *   congruential      z -> lcg[0] z + lcg[1];
 *   xoshiro           s -> q(T) s = sum of T^i s over the bits i of q.
 * Each word is then 64 draws with the PR ring in registers (ring slot = draw
 * index mod 64, constant after unrolling), and four warp transposes turn the
 * 32 streams' words into device words of the sites (walk translation 0). */
constexpr int REFRESH_REC = 120;
constexpr uint64_t REFRESH_LCG_A = 3202034522624059733ULL; /* random_generator.h:66 */


__device__ __forceinline__ uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

__device__ __forceinline__ void xoshiro_step(uint64_t &s0, uint64_t &s1, uint64_t &s2,
                                             uint64_t &s3) {
  const uint64_t t = s1 << 17;
  s2 ^= s0;
  s3 ^= s1;
  s1 ^= s2;
  s0 ^= s3;
  s2 ^= t;
  s3 = rotl64(s3, 45);
}

template <int MINB>
__global__ void __launch_bounds__(64, MINB)
k_refresh(const micsa_geo g, const int first, const int count, const int64_t nwords,
          const int wps, const int64_t nseg, const uint64_t *__restrict__ rec,
          const uint64_t *__restrict__ lcg, const uint64_t *__restrict__ xoq,
          const uint64_t *__restrict__ fib, const uint64_t t0, const uint64_t t1,
          const uint64_t t2, uint32_t *__restrict__ dem0, uint32_t *__restrict__ dem1) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (warp >= (int64_t)count * g.W * nseg) return; /* whole warps only */
  const int64_t seg = warp % nseg, grp = warp / nseg;
  const int w = (int)(grp % g.W), j = (int)(grp / g.W);
  const uint64_t *R = rec + grp * REFRESH_REC * 32 + lane;

  uint64_t ring[64];
  if (seg == 0) {
#pragma unroll
    for (int t = 0; t < 61; t++) ring[3 + t] = R[t * 32];
  } else {
#pragma unroll
    for (int t = 0; t < 55; t++) ring[3 + t] = 0;
    const uint64_t *c = fib + seg * 55;
    const uint64_t *E = R + 6 * 32;
    for (int i = 0; i < 55; i++) {
      const uint64_t ci = c[i];
#pragma unroll
      for (int t = 0; t < 55; t++) ring[3 + t] += ci * E[(i + t) * 32];
    }
#pragma unroll
    for (int k = 0; k < 6; k++) ring[58 + k] = ring[34 + k] + ring[3 + k];
  }
  uint64_t z = lcg[2 * seg] * R[115 * 32] + lcg[2 * seg + 1];
  uint64_t s0 = R[116 * 32], s1 = R[117 * 32], s2 = R[118 * 32], s3 = R[119 * 32];
  if (seg != 0) {
    uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int qw = 0; qw < 4; qw++) {
      uint64_t bits = xoq[4 * seg + qw];
      for (int b = 0; b < 64; b++, bits >>= 1) {
        if (bits & 1) { a0 ^= s0; a1 ^= s1; a2 ^= s2; a3 ^= s3; }
        xoshiro_step(s0, s1, s2, s3);
      }
    }
    s0 = a0; s1 = a1; s2 = a2; s3 = a3;
  }

  const int64_t i0 = seg * wps;
  const int64_t i1 = i0 + wps < nwords ? i0 + wps : nwords;
  const int sample = first + j;
  /* Where the two sites of this lane's bits (lane, lane + 32) of word i live
   * at walk 0: word i = pi*H + h is colour p = pi / nc, plane ic = pi % nc,
   * MSC word h = a2 + mh*(bb + m*c); the site of bit b is x = (b&3)*m + a
   * (a = 2*a2 + parity, so x/2 = (b&3)*mh + a2), y = ((b>>2)&3)*m + bb,
   * z = (b>>4)*m + c (ini.c:317-337), stored at (z*L + y)*Lh + x/2.  That
   * splits into a lane part and a warp-uniform word part, the latter
   * stepped along with i instead of divided out per word. */
  const int m = g.L >> 2, mh = m >> 1;
  const int64_t slab = (int64_t)m * g.L * g.Lh; /* one block step in z */
  const int64_t lane_a = ((int64_t)(lane >> 4) * slab) + (int64_t)((lane >> 2) & 3) * m * g.Lh +
                         (int64_t)(lane & 3) * mh;
  const int64_t lane_b = lane_a + 2 * slab;
  int64_t pi = i0 / g.H;
  int64_t hrem = i0 % g.H;
  int a2 = (int)(hrem % mh), bb = (int)((hrem / mh) % m), c = (int)(hrem / ((int64_t)mh * m));
  int64_t base = ((int64_t)sample * 2 * g.nc + pi) * g.P * g.W + w;
  for (int64_t i = i0; i < i1; i++) {
    uint64_t d0 = 0, d1 = 0;
#pragma unroll
    for (int b = 0; b < 64; b++) {
      const uint64_t xo_out = rotl64(s0 + s3, 23) + s0;
      xoshiro_step(s0, s1, s2, s3);
      const uint64_t xn = ring[(b - 24) & 63] + ring[(b - 55) & 63];
      const uint64_t pr = xn ^ ring[(b - 61) & 63];
      ring[b] = xn;
      z = z * REFRESH_LCG_A + 1;
      const uint64_t e = (z + pr) + xo_out;
      const uint32_t a0 = e < t0, a1 = e < t1, a2 = e < t2;
      d0 |= (uint64_t)(a0 ^ a1 ^ a2) << b;
      d1 |= (uint64_t)((a0 & a1) | (a0 & a2) | (a1 & a2)) << b;
    }
    const uint32_t lo0 = warp_transpose32((uint32_t)d0, lane);
    const uint32_t hi0 = warp_transpose32((uint32_t)(d0 >> 32), lane);
    const uint32_t lo1 = warp_transpose32((uint32_t)d1, lane);
    const uint32_t hi1 = warp_transpose32((uint32_t)(d1 >> 32), lane);
    const int64_t word = ((int64_t)c * g.L + bb) * g.Lh + a2;
    const int64_t oa = base + (word + lane_a) * g.W;
    const int64_t ob = base + (word + lane_b) * g.W;
    dem0[oa] = lo0;
    dem0[ob] = hi0;
    dem1[oa] = lo1;
    dem1[ob] = hi1;
    if (++a2 == mh) {
      a2 = 0;
      if (++bb == m) {
        bb = 0;
        if (++c == m) { /* next (colour, plane) */
          c = 0;
          base += g.P * g.W;
        }
      }
    }
  }
}

cudaError_t micsa_launch_refresh(const micsa_geo &g, int first, int count, int64_t nwords,
                                 int wps, int64_t nseg, const uint64_t *rec, const uint64_t *lcg,
                                 const uint64_t *xoq, const uint64_t *fib, const uint64_t thr[3],
                                 uint32_t *dem0, uint32_t *dem1, cudaStream_t st) {
  const int64_t warps = (int64_t)count * g.W * nseg;
  const unsigned blocks = (unsigned)((warps + 1) / 2);
  /* registers for 6 blocks (12 warps) per SM: 168, with a small spill */
  if (g.occ == 1)
    k_refresh<1><<<blocks, 64, 0, st>>>(g, first, count, nwords, wps, nseg, rec, lcg, xoq, fib,
                                        thr[0], thr[1], thr[2], dem0, dem1);
  else
    k_refresh<6><<<blocks, 64, 0, st>>>(g, first, count, nwords, wps, nseg, rec, lcg, xoq, fib,
                                        thr[0], thr[1], thr[2], dem0, dem1);
  return cudaGetLastError();
}

/* --------------------------------------------- resident small lattices */
/* At L <= 16 one sample's spins, coupling bytes and demon planes of one
 * 32-replica word -- 2P*4 + 2P + 2*(2*nc*P*4) bytes, 216 KB at L=16, nc=6 --
 * fit in one block's shared memory.  Block (w, s) copies them in, runs n
 * iterations (2*nc half-sweeps with a barrier after each, the demon walk as
 * the translation k -> k+1 mod L/2, as in the other kernels) and copies them
 * back; HBM is touched only at the ends.  The per-site arithmetic is
 * k_sweep's; shared memory has no coalescing constraint, so a thread takes
 * one site at a time.  The walk counter is only read here: the caller
 * advances it by n afterwards. */
template <int L>
struct resident_cfg {
  static constexpr int P = L * L * L / 2, Lh = L / 2;
  static constexpr int TPB = P < 512 ? P : 512;
};

template <int L>
__global__ void __launch_bounds__(resident_cfg<L>::TPB)
k_resident(const micsa_geo g, const int n, uint32_t *__restrict__ spin,
           uint32_t *__restrict__ d0, uint32_t *__restrict__ d1, const uint8_t *__restrict__ jb,
           const int *__restrict__ walk) {
  constexpr int P = resident_cfg<L>::P, Lh = resident_cfg<L>::Lh, TPB = resident_cfg<L>::TPB;
  extern __shared__ uint4 smem_raw[];
  const int w = blockIdx.x, s = blockIdx.y, W = g.W, nc = g.nc;
  if (micsa_frozen(g, s)) return;
  uint32_t *sp = (uint32_t *)smem_raw; /* [2][P] */
  uint32_t *sd0 = sp + 2 * P;          /* [2][nc][P] */
  uint32_t *sd1 = sd0 + 2 * nc * P;
  uint8_t *sj = (uint8_t *)(sd1 + 2 * nc * P); /* [2][P] */
  const size_t sbase = (size_t)s * 2 * P, dbase = (size_t)s * 2 * nc * P;
  for (int i = threadIdx.x; i < 2 * P; i += TPB) {
    sp[i] = spin[(sbase + i) * W + w];
    sj[i] = jb[sbase + i];
  }
  for (int i = threadIdx.x; i < 2 * nc * P; i += TPB) {
    sd0[i] = d0[(dbase + i) * W + w];
    sd1[i] = d1[(dbase + i) * W + w];
  }
  int k = walk[s];
  __syncthreads();
  for (int it = 0; it < n; it++) {
    for (int ic = 0; ic < nc; ic++) {
      const int axis = ic < 3 ? ic : ic - 3;
      for (int p = 0; p < 2; p++) {
        const int sh = ((p == 0) == (ic < 3)) ? k : -k; /* demon shift, units of 2 sites */
        const uint32_t *oth = sp + (p ^ 1) * P;
        uint32_t *mine = sp + p * P;
        uint32_t *q0 = sd0 + (p * nc + ic) * P, *q1 = sd1 + (p * nc + ic) * P;
        const uint8_t *jp = sj + p * P;
#pragma unroll
        for (int i = threadIdx.x; i < P; i += TPB) {
          const int xh = i % Lh, y = (i / Lh) % L, z = i / (Lh * L);
          const int rowoff = (y + z + p) & 1;
          int xe = xh + rowoff; if (xe == Lh) xe = 0;
          int xo = xh + rowoff - 1; if (xo < 0) xo = Lh - 1;
          const int yp = (y + 1) & (L - 1), ym = (y - 1) & (L - 1);
          const int zp = (z + 1) & (L - 1), zm = (z - 1) & (L - 1);
          const int row = (z * L + y) * Lh;
          const uint32_t sw = mine[i];
          const uint32_t jb6 = jp[i];
          const uint32_t f0 = sw ^ oth[row + xe] ^ jmask(jb6, 0);
          const uint32_t f1 = sw ^ oth[(z * L + yp) * Lh + xh] ^ jmask(jb6, 1);
          const uint32_t f2 = sw ^ oth[(zp * L + y) * Lh + xh] ^ jmask(jb6, 2);
          const uint32_t f3 = sw ^ oth[row + xo] ^ jmask(jb6, 3);
          const uint32_t f4 = sw ^ oth[(z * L + ym) * Lh + xh] ^ jmask(jb6, 4);
          const uint32_t f5 = sw ^ oth[(zm * L + y) * Lh + xh] ^ jmask(jb6, 5);
          const uint32_t j1 = xor3(f0, f1, f2), j2 = maj3(f0, f1, f2);
          const uint32_t j3 = xor3(f3, f4, f5), j4 = maj3(f3, f4, f5);
          int slot;
          if (axis == 0) slot = row + ((xh - sh) & (Lh - 1));
          else if (axis == 1) slot = (z * L + ((y - 2 * sh) & (L - 1))) * Lh + xh;
          else slot = (((z - 2 * sh) & (L - 1)) * L + y) * Lh + xh;
          uint32_t D0 = q0[slot], D1 = q1[slot];
          const uint32_t flip = isi_update(j1, j2, j3, j4, D0, D1);
          q0[slot] = D0;
          q1[slot] = D1;
          mine[i] = sw ^ flip;
        }
        __syncthreads();
      }
    }
    k = (k + 1 == Lh) ? 0 : k + 1;
  }
  for (int i = threadIdx.x; i < 2 * P; i += TPB) spin[(sbase + i) * W + w] = sp[i];
  for (int i = threadIdx.x; i < 2 * nc * P; i += TPB) {
    d0[(dbase + i) * W + w] = sd0[i];
    d1[(dbase + i) * W + w] = sd1[i];
  }
}

__global__ void k_walk_add(const micsa_geo g, int *walk, int ns, int n, int period) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < ns && !micsa_frozen(g, s)) walk[s] = (int)(((int64_t)walk[s] + n) % period);
}

cudaError_t micsa_launch_walk_add(const micsa_geo &g, int *walk, int n, cudaStream_t st) {
  k_walk_add<<<(g.ns + 127) / 128, 128, 0, st>>>(g, walk, g.ns, n, g.L / 2);
  return cudaGetLastError();
}

size_t micsa_resident_smem(int L, int nc) {
  if (L != 8 && L != 16) return 0;
  const size_t P = (size_t)L * L * L / 2;
  return 2 * P * 4 + 2 * P + 2 * (2 * (size_t)nc * P * 4);
}

template <int L>
static cudaError_t resident_l(const micsa_geo &g, int n, uint32_t *spin, uint32_t *d0,
                              uint32_t *d1, const uint8_t *jb, int *walk, cudaStream_t st) {
  const size_t bytes = micsa_resident_smem(L, g.nc);
  cudaError_t e = cudaFuncSetAttribute(k_resident<L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes);
  if (e != cudaSuccess) return e;
  k_resident<L><<<dim3(g.W, g.ns), resident_cfg<L>::TPB, bytes, st>>>(g, n, spin, d0, d1, jb, walk);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_walk_add<<<(g.ns + 127) / 128, 128, 0, st>>>(g, walk, g.ns, n, g.L / 2);
  return cudaGetLastError();
}

cudaError_t micsa_launch_resident(const micsa_geo &g, int n, uint32_t *spin, uint32_t *d0,
                                  uint32_t *d1, const uint8_t *jb, int *walk, cudaStream_t st) {
  if (g.L == 8) return resident_l<8>(g, n, spin, d0, d1, jb, walk, st);
  if (g.L == 16) return resident_l<16>(g, n, spin, d0, d1, jb, walk, st);
  return cudaErrorInvalidValue;
}

cudaError_t micsa_launch_sweep_multi(const micsa_multi_args &a, int occ, unsigned *ctl,
                                     cudaStream_t st) {
  if (a.n < 1 || a.n > MICSA_MULTI_MAX || a.total == 0) return cudaErrorInvalidValue;
  const int W = a.gr[0].g.W;
  for (int i = 1; i < a.n; i++)
    if (a.gr[i].g.W != W) return cudaErrorInvalidValue;
  const dim3 grid(a.total), block(MTPB);
  /* the word vector of one site: 4, 2 or 1 words; one group of them (WIDE)
   * when it is all of a site's words */
  if (W % 4 == 0) {
    if (W == 4) k_sweep_multi<4, true, 4><<<grid, block, 0, st>>>(a, ctl);
    else k_sweep_multi<4, false, 4><<<grid, block, 0, st>>>(a, ctl);
  } else if (W % 2 == 0) {
    if (W == 2) {
      if (occ == 8) k_sweep_multi<2, true, 8><<<grid, block, 0, st>>>(a, ctl);
      else if (occ == 5) k_sweep_multi<2, true, 5><<<grid, block, 0, st>>>(a, ctl);
      else k_sweep_multi<2, true, 6><<<grid, block, 0, st>>>(a, ctl);
    } else {
      k_sweep_multi<2, false, 6><<<grid, block, 0, st>>>(a, ctl);
    }
  } else {
    if (occ == 8) k_sweep_multi<1, true, 8><<<grid, block, 0, st>>>(a, ctl);
    else k_sweep_multi<1, true, 6><<<grid, block, 0, st>>>(a, ctl);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  unsigned maxns = 1;
  for (int i = 0; i < a.n; i++) maxns = a.gr[i].ns_run > maxns ? a.gr[i].ns_run : maxns;
  k_walk_multi<<<dim3((maxns + MTPB - 1) / MTPB, a.n), MTPB, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t micsa_tma_timeout_count(unsigned *n) {
  return cudaMemcpyFromSymbol(n, micsa_tma_timeouts, sizeof(unsigned));
}
