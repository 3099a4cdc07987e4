/*
 * Lattice initialisation, reference-layout packing, demon draws, Philox
 * counters and measurement arithmetic of the micSA drop-in.  Each function
 * reproduces the cited part of IsidoroGlez/micSA-EA-MC PROGRAM/.
 */
#include "micsa_host.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* binary128 arithmetic for the demon thresholds: __float128 + libquadmath
 * on x86-64, the native IEEE quad `long double` on AArch64 (both evaluate
 * exp with the same ldbl-128 algorithm). */
#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 micsa_quad;
#define MICSA_QEXP expq
#define MICSA_QPOW powq
#define MICSA_Q(x) x##Q
#elif defined(__aarch64__) && (__LDBL_MANT_DIG__ == 113)
typedef long double micsa_quad;
#define MICSA_QEXP expl
#define MICSA_QPOW powl
#define MICSA_Q(x) x##L
#else
#error "binary128 arithmetic is required for the demon thresholds"
#endif

int64_t micsa_half_words(int L) {
  int64_t m = L / 4;
  return m * m * m / 2;
}

/* Inverse of the packing index of packing_u (ini.c:317-337). */
void micsa_msc_site(int L, int p, int64_t h, int bit, int *x, int *y, int *z) {
  const int m = L / 4, mh = m / 2;
  int a2 = (int)(h % mh);
  int b = (int)((h / mh) % m);
  int c = (int)(h / ((int64_t)mh * m));
  int a = 2 * a2 + ((b + c + p) & 1);
  int bx = bit & 3, by = (bit >> 2) & 3, bz = bit >> 4;
  *x = bx * m + a;
  *y = by * m + b;
  *z = bz * m + c;
}

/* packing_u (ini.c:301-345). */
void micsa_pack_spins(int L, int nr, const uint8_t *uu, uint64_t *even,
                      uint64_t *odd) {
  const int m = L / 4;
  const int64_t V = (int64_t)L * L * L, H = micsa_half_words(L);
  memset(even, 0, sizeof(uint64_t) * H * nr);
  memset(odd, 0, sizeof(uint64_t) * H * nr);
  for (int r = 0; r < nr; r++) {
    const uint8_t *u = uu + (int64_t)r * V;
    int64_t site = 0;
    for (int z = 0; z < L; z++)
      for (int y = 0; y < L; y++)
        for (int x = 0; x < L; x++, site++) {
          int bit = x / m + 4 * (y / m) + 16 * (z / m);
          int64_t h = ((x % m) + (int64_t)m * (y % m) + (int64_t)m * m * (z % m)) / 2;
          uint64_t *w = ((x ^ y ^ z) & 1) ? odd : even;
          w[h * nr + r] |= (uint64_t)(u[site] & 1) << bit;
        }
  }
}

/* unpacking_u (ini.c:347-395). */
void micsa_unpack_spins(int L, int nr, const uint64_t *even,
                        const uint64_t *odd, uint8_t *uu) {
  const int64_t V = (int64_t)L * L * L, H = micsa_half_words(L);
  for (int p = 0; p < 2; p++) {
    const uint64_t *w = p ? odd : even;
    for (int64_t h = 0; h < H; h++)
      for (int bit = 0; bit < 64; bit++) {
        int x, y, z;
        micsa_msc_site(L, p, h, bit, &x, &y, &z);
        int64_t site = x + (int64_t)L * y + (int64_t)L * L * z;
        for (int r = 0; r < nr; r++)
          uu[(int64_t)r * V + site] = (uint8_t)((w[h * nr + r] >> bit) & 1);
      }
  }
}

/* packing_J (ini.c:521-578).  The backward-direction word of a site holds
 * each bond at the bit of the site that OWNS the bond (the -x neighbour),
 * which for a neighbour across a block edge is a different block; the sweep
 * compensates by xoring before rotating (main.cu:913-923). */
void micsa_pack_couplings(int L, const uint8_t *Jx, const uint8_t *Jy,
                          const uint8_t *Jz, uint64_t *J) {
  const int m = L / 4;
  const int64_t H = micsa_half_words(L);
  memset(J, 0, sizeof(uint64_t) * 12 * H);
  int64_t site = 0;
  for (int z = 0; z < L; z++)
    for (int y = 0; y < L; y++)
      for (int x = 0; x < L; x++, site++) {
        int a = x % m, b = y % m, c = z % m;
        int bit = x / m + 4 * (y / m) + 16 * (z / m);
        int p = (a + b + c) & 1;
        int64_t msc = a + (int64_t)m * b + (int64_t)m * m * c;
        int64_t nb[3] = {((a + 1) % m) + (int64_t)m * b + (int64_t)m * m * c,
                         a + (int64_t)m * ((b + 1) % m) + (int64_t)m * m * c,
                         a + (int64_t)m * b + (int64_t)m * m * ((c + 1) % m)};
        const uint8_t jv[3] = {Jx[site], Jy[site], Jz[site]};
        for (int d = 0; d < 3; d++) {
          uint64_t v = (uint64_t)(jv[d] & 1) << bit;
          J[(int64_t)(p * 6 + d) * H + msc / 2] |= v;
          J[(int64_t)((1 - p) * 6 + d + 3) * H + nb[d] / 2] |= v;
        }
      }
}

/* Init_u (ini.c:275-299): MAXNSAMPLES draws per (replica, site), of which
 * the ones whose index is in list_samples are kept. */
int micsa_init_spins(micsa_prc_t *random_u, int L, int nr, int maxnsamples,
                     const int *list_samples, int nbits, uint8_t *uu) {
  const int64_t V = (int64_t)L * L * L;
  int *ls = (int *)calloc((size_t)maxnsamples + 1, sizeof(int));
  if (!ls) return -1;
  for (int i = 0; i < nbits && i < maxnsamples; i++) ls[i] = list_samples[i];
  for (int r = 0; r < nr; r++)
    for (int64_t site = 0; site < V; site++) {
      int i = 0;
      for (int ib = 0; ib < maxnsamples; ib++) {
        uint64_t v = micsa_prc_next(random_u);
        if (i <= maxnsamples && ib == ls[i]) {
          if (i < nbits) uu[((int64_t)i * nr + r) * V + site] = (uint8_t)(v >> 63);
          i++;
        }
      }
      if (i != nbits) { free(ls); return -1; }
    }
  free(ls);
  return 0;
}

/* Init_J, -DJANUS branch (ini.c:457-471). */
int micsa_init_couplings_janus(uint64_t seed, int L, uint8_t *Jx, uint8_t *Jy,
                               uint8_t *Jz) {
  micsa_janus_t g;
  micsa_janus_seed(&g, seed);
  const int64_t V = (int64_t)L * L * L;
  int count = 0;
  for (int64_t s = 0; s < V; s++) {
    Jx[s] = (uint8_t)(micsa_janus_next(&g) >> 63); count += Jx[s];
    Jy[s] = (uint8_t)(micsa_janus_next(&g) >> 63); count += Jy[s];
    Jz[s] = (uint8_t)(micsa_janus_next(&g) >> 63); count += Jz[s];
  }
  return count;
}

/* get_thresholds (ini.c:680-710): P(D=k) ~ exp(-4 beta k), k = 0..3,
 * thresholds 2^64 * P(D>=3), P(D>=2), P(D>=1), truncated. */
void micsa_thresholds(double beta, uint64_t thr[3]) {
  micsa_quad qb = (micsa_quad)beta;
  micsa_quad f = MICSA_QEXP(MICSA_Q(-4.0) * qb);
  micsa_quad prob[4], norm, acc[3];
  prob[0] = MICSA_Q(1.0);
  norm = prob[0];
  for (int i = 1; i < 4; i++) {
    prob[i] = prob[i - 1] * f;
    norm += prob[i];
  }
  for (int i = 0; i < 4; i++) prob[i] /= norm;
  acc[0] = prob[3];
  acc[1] = prob[2] + acc[0];
  acc[2] = prob[1] + acc[1];
  for (int i = 0; i < 3; i++)
    thr[i] = (uint64_t)(MICSA_Q(18446744073709551616.0) * acc[i]);
}

/* prepara_LUT (input/LUT/preparation.c:265-388): 256 cumulative 64-bit
 * thresholds for a byte whose 8 bits are independently 1 with probability
 * e^{-4 beta}, and a 1024-entry table of (first, last) candidate index for
 * each value of the top 10 bits of a uniform.  out: 4096 bytes. */
void micsa_build_lut(double beta, void *out) {
  micsa_quad qb = (micsa_quad)beta;
  micsa_quad p0 = MICSA_Q(1.0) - MICSA_QEXP(MICSA_Q(-4.0) * qb);
  micsa_quad p1 = MICSA_QEXP(MICSA_Q(-4.0) * qb);
  uint64_t caso[9], cum[256];
  for (int i = 0; i < 9; i++)
    caso[i] = (uint64_t)(MICSA_Q(18446744073709551616.0) * (MICSA_QPOW(p0, 8 - i) * MICSA_QPOW(p1, i)));
  cum[0] = caso[0];
  for (int i = 1; i < 255; i++) cum[i] = cum[i - 1] + caso[__builtin_popcount(i)];
  cum[255] = ~0ULL;
  uint32_t *w = (uint32_t *)out;
  for (int i = 0; i < 256; i += 2) {
    w[2 * i + 0] = (uint32_t)(cum[i] >> 32);
    w[2 * i + 1] = (uint32_t)cum[i];
    w[2 * i + 2] = (uint32_t)(cum[i + 1] >> 32);
    w[2 * i + 3] = (uint32_t)cum[i + 1];
  }
  uint32_t lo[1024], hi[1024];
  const uint64_t tail = (1ULL << 54) - 1;
  for (uint64_t m = 0; m < 1024; m++) {
    uint64_t t = m << 54;
    int i = 0;
    while (i < 256 && !(t < cum[i])) i++;
    lo[m] = (uint32_t)(i > 255 ? 255 : i);
    t |= tail;
    i = 0;
    while (i < 256 && !(t < cum[i])) i++;
    hi[m] = (uint32_t)(i > 255 ? 255 : i);
  }
  for (int i = 0; i < 1024; i += 8)
    for (int j = 0; j < 4; j++)
      w[512 + i / 2 + j] = lo[i + 2 * j] | (hi[i + 2 * j] << 8) | (lo[i + 2 * j + 1] << 16) |
                           (hi[i + 2 * j + 1] << 24);
}

/* InitWalkers (ini.c:751-778) for one replica stream. */
void micsa_draw_demons(micsa_prc_t *prc, micsa_xoshiro_t *xo,
                       const uint64_t thr[3], int L, int nr, int nc, int r,
                       uint64_t *w0, uint64_t *w1) {
  const int64_t nw = 2 * micsa_half_words(L) * nc;
  micsa_prc_t a = *prc;
  micsa_xoshiro_t b = *xo;
  const uint64_t t0 = thr[0], t1 = thr[1], t2 = thr[2];
  for (int64_t i = 0; i < nw; i++) {
    uint64_t d0 = 0, d1 = 0;
    for (int bit = 0; bit < 64; bit++) {
      micsa_xoshiro_next(&b);
      micsa_prc_next(&a);
      uint64_t e = a.out + b.out;
      uint64_t v = (uint64_t)(e < t0) + (uint64_t)(e < t1) + (uint64_t)(e < t2);
      d0 |= (v & 1ULL) << bit;
      d1 |= ((v >> 1) & 1ULL) << bit;
    }
    w0[i * nr + r] = d0;
    w1[i * nr + r] = d1;
  }
  *prc = a;
  *xo = b;
}

typedef struct {
  micsa_prc_t *prc;
  micsa_xoshiro_t *xo;
  const uint64_t *thr;
  int L, nr, nc, r0, r1;
  uint64_t *w0, *w1;
} demon_job;

static void *demon_worker(void *arg) {
  demon_job *j = (demon_job *)arg;
  for (int r = j->r0; r < j->r1; r++)
    micsa_draw_demons(&j->prc[r], &j->xo[r], j->thr, j->L, j->nr, j->nc, r,
                      j->w0, j->w1);
  return NULL;
}

int micsa_draw_demons_all(micsa_prc_t *prc, micsa_xoshiro_t *xo,
                          const uint64_t thr[3], int L, int nr, int nc,
                          uint64_t *w0, uint64_t *w1, int nthreads) {
  enum { MAXT = 256 };
  if (nthreads < 1) nthreads = 1;
  if (nthreads > nr) nthreads = nr;
  if (nthreads > MAXT) nthreads = MAXT;
  pthread_t tid[MAXT];
  int spawned[MAXT];
  demon_job job[MAXT];
  for (int t = 0; t < nthreads; t++) {
    job[t] = (demon_job){prc, xo, thr, L, nr, nc,
                         (int)((int64_t)nr * t / nthreads),
                         (int)((int64_t)nr * (t + 1) / nthreads), w0, w1};
    /* the last share runs on the calling thread, as does any share whose
     * thread could not be started */
    spawned[t] = t < nthreads - 1 &&
                 pthread_create(&tid[t], NULL, demon_worker, &job[t]) == 0;
    if (!spawned[t]) demon_worker(&job[t]);
  }
  int rc = 0;
  for (int t = 0; t < nthreads; t++)
    if (spawned[t]) rc |= pthread_join(tid[t], NULL);
  return rc ? -1 : 0;
}

/* _fill_bits (include/fill_bits.h:47-68): 52 entropy bits per replica are
 * spread over the 128-bit Philox counter around the iteration number
 * (15 bits in x, 25 in y), the colour, 2 bits of internal call counter,
 * 19 bits of thread index (z) and 14 bits of job id (w). */
void micsa_fill_bits(micsa_prc_t *prc, micsa_xoshiro_t *xo, int nr,
                     uint64_t iter, int parity, uint32_t jobid, uint32_t *te) {
  for (int r = 0; r < nr; r++) {
    micsa_xoshiro_next(&xo[r]);
    micsa_prc_next(&prc[r]);
    uint64_t e = (prc[r].out + xo[r].out) >> (64 - 52);
    uint32_t x = (uint32_t)(((iter & 32767ULL) << 3) | (((uint64_t)parity & 1ULL) << 2));
    uint32_t y = (uint32_t)(iter >> 15);
    x |= (uint32_t)((e & 0x3FFFULL) << 18);
    e >>= 14;
    y |= (uint32_t)((e & 0x7FULL) << 25);
    e >>= 7;
    uint32_t z = (uint32_t)((e & 0x1FFFULL) << 19);
    e >>= 13;
    uint32_t w = (uint32_t)(e << 14) | jobid;
    te[4 * r + 0] = x;
    te[4 * r + 1] = y;
    te[4 * r + 2] = z;
    te[4 * r + 3] = w;
  }
}

/* Measures (med.c:270-309 of the energy part), same operation order. */
void micsa_energy_stats(const int32_t *e_spin, int nr, int L, double *mean,
                        double *std) {
  const double V = (double)((int64_t)L * L * L);
  double a = 0, s = 0;
  for (int r = 0; r < nr; r++) {
    double v = ((double)(-e_spin[r])) / V;
    a += v;
    s += v * v;
  }
  a /= (double)nr;
  s /= (double)nr;
  s -= a * a;
  s /= (double)nr - 1;
  *mean = a;
  *std = sqrt(s);
}

void micsa_demon_stats(const uint64_t *e_demon, int nr, int L, int nc,
                       double *mean, double *std) {
  const double V = (double)((int64_t)L * L * L);
  double a = 0, s = 0;
  for (int r = 0; r < nr; r++) {
    double v = ((double)e_demon[r]) / (V * nc);
    a += v;
    s += v * v;
  }
  a /= (double)nr;
  s /= (double)nr;
  s -= a * a;
  s /= (double)nr - 1;
  *mean = a;
  *std = sqrt(s);
}

/* Correlation lengths from C4 by the integral estimators of the Janus
 * collaboration (Belletti et al., Phys. Rev. Lett. 101, 157201 (2008)):
 * I_k = sum_{r < r_cut} r^k C4(r), xi_{k,k+1} = I_{k+1} / I_k, with C4(r)
 * the pair- and axis-averaged correlation normalised by V.  Far from the
 * origin C4(r) is noise, and summing it with weights r^k swamps the
 * estimate; the Janus analyses (Belletti et al., J. Stat. Phys. 135, 1121
 * (2009)) therefore stop the integrals where C4 falls below a few times its
 * statistical error.  Here the error of C4(r) is the standard error over the
 * replica pairs (each pair's axis average is one estimate, pairs being
 * independent), and r_cut is the first r >= 1 with C4(r) < kappa * err(r)
 * (kappa > 0 and at least two pairs), capped at rmax + 1 when rmax > 0.
 * kappa = 0 and rmax = 0 sum the whole range 0 .. L/2. */
void micsa_correlation_lengths(int L, int npairs, const int64_t *c4, double kappa, int rmax,
                               double *C4r, double *err, double *xi12, double *xi23, int *rcut) {
  const int nd = L / 2 + 1;
  const double V = (double)L * L * L;
  int cut = nd;
  if (rmax > 0 && rmax + 1 < cut) cut = rmax + 1;
  double I1 = 0, I2 = 0, I3 = 0;
  for (int d = 0; d < nd; d++) {
    double s = 0, s2 = 0;
    for (int k = 0; k < npairs; k++) {
      double pk = 0;
      for (int a = 0; a < 3; a++) pk += (double)c4[((int64_t)k * 3 + a) * nd + d];
      pk /= 3.0 * V;
      s += pk;
      s2 += pk * pk;
    }
    const double c = s / (double)npairs;
    double e = 0;
    if (npairs > 1) {
      const double var = (s2 - s * c) / (double)(npairs - 1);
      e = var > 0 ? sqrt(var / (double)npairs) : 0;
    }
    if (C4r) C4r[d] = c;
    if (err) err[d] = e;
    if (d >= 1 && d < cut && kappa > 0 && npairs > 1 && c < kappa * e) cut = d;
    if (d < cut) {
      const double r = (double)d;
      I1 += r * c;
      I2 += r * r * c;
      I3 += r * r * r * c;
    }
  }
  if (rcut) *rcut = cut;
  if (xi12) *xi12 = I1 != 0 ? I2 / I1 : 0;
  if (xi23) *xi23 = I2 != 0 ? I3 / I2 : 0;
}
