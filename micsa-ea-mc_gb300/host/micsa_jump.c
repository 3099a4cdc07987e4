/*
 * Jump-ahead of the demon-refresh streams (InitWalkers, ini.c:712-781).
 *
 * One refresh draws M = 64 * 2*H*nc values from each replica's stream pair
 * (PR+congruential, xoshiro256++).  The draws are sequential in the
 * reference; here a stream is cut into segments of S draws and the state at
 * the start of each segment is reached by jumping:
 *
 *  - congruential z -> A z + 1: o steps compose to z -> m z + a (doubling);
 *  - lagged Fibonacci x_n = x_{n-24} + x_{n-55} (mod 2^64), output
 *    x_n ^ x_{n-61}: with E[k] = x_{-55+k}, the value x_{-55+t+j} equals
 *    sum_i c_i E[i+j] for X^t = sum_i c_i X^i mod (X^55 - X^31 - 1), since
 *    X^t -> x_{-55+t} is linear and respects the recurrence;
 *  - xoshiro256's state map T is GF(2)-linear with a characteristic
 *    polynomial p of degree 256 (found here by Berlekamp-Massey on one
 *    state bit); T^o s = q(T) s for q = X^o mod p.
 * These are the standard jump constructions for linear generators (e.g.
 * Haramoto et al., "Efficient jump ahead for F2-linear random number
 * generators", 2008); every table is computed here, none is embedded.
 */
#include "micsa_jump.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define R MICSA_FIB_R
#define LAG_A 24
#define LAG_O 61

/* ------------------------------------------------------ congruential */
static void lcg_compose(uint64_t m1, uint64_t a1, uint64_t m2, uint64_t a2, uint64_t *m,
                        uint64_t *a) {
  /* (z -> m1 z + a1) after (z -> m2 z + a2) */
  *m = m1 * m2;
  *a = m1 * a2 + a1;
}

void micsa_lcg_jump(uint64_t o, uint64_t *mult, uint64_t *add) {
  uint64_t m = 1, a = 0, bm = MICSA_LCG_A, ba = 1;
  while (o) {
    if (o & 1) lcg_compose(bm, ba, m, a, &m, &a);
    lcg_compose(bm, ba, bm, ba, &bm, &ba);
    o >>= 1;
  }
  *mult = m;
  *add = a;
}

/* ---------------------------------------------------- lagged Fibonacci */
/* c <- a * b mod (X^55 - X^31 - 1) over Z/2^64 */
static void fib_mulmod(const uint64_t *a, const uint64_t *b, uint64_t *c) {
  uint64_t t[2 * R - 1];
  memset(t, 0, sizeof t);
  for (int i = 0; i < R; i++) {
    if (!a[i]) continue;
    for (int j = 0; j < R; j++) t[i + j] += a[i] * b[j];
  }
  /* X^k = X^(k-24) + X^(k-55) for k >= 55, highest first */
  for (int k = 2 * R - 2; k >= R; k--) {
    t[k - LAG_A] += t[k];
    t[k - R] += t[k];
  }
  memcpy(c, t, sizeof(uint64_t) * R);
}

void micsa_fib_jump(uint64_t t, uint64_t c[R]) {
  uint64_t base[R], acc[R];
  memset(acc, 0, sizeof acc);
  acc[0] = 1;
  memset(base, 0, sizeof base);
  base[1] = 1; /* X */
  while (t) {
    if (t & 1) fib_mulmod(acc, base, acc);
    fib_mulmod(base, base, base);
    t >>= 1;
  }
  memcpy(c, acc, sizeof acc);
}

/* --------------------------------------------------------- xoshiro256 */
static void xo_step(uint64_t s[4]) {
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = micsa_rotl64(s[3], 45);
}

static int bit_of(const uint64_t *v, int i) { return (int)((v[i >> 6] >> (i & 63)) & 1); }

/* Berlekamp-Massey over GF(2) on 512 terms of bit 0 of s[0]; the result is
 * the minimal polynomial of T when that has degree 256 (T's characteristic
 * polynomial is primitive, so every non-zero state gives it). */
void micsa_xoshiro_charpoly(uint64_t p[5]) {
  enum { N = 512, WORDS = 9 };
  uint8_t seq[N];
  uint64_t s[4] = {0x9E3779B97F4A7C15ULL, 0xBF58476D1CE4E5B9ULL, 0x94D049BB133111EBULL, 1};
  for (int k = 0; k < N; k++) {
    seq[k] = (uint8_t)(s[0] & 1);
    xo_step(s);
  }
  /* connection polynomials as bit vectors, C(X) = 1 + c1 X + ... */
  uint64_t C[WORDS] = {1}, B[WORDS] = {1}, T[WORDS];
  int Lc = 0, m = 1;
  for (int n = 0; n < N; n++) {
    int d = seq[n];
    for (int i = 1; i <= Lc; i++) d ^= bit_of(C, i) & seq[n - i];
    if (!d) {
      m++;
      continue;
    }
    memcpy(T, C, sizeof T);
    /* C ^= X^m B */
    for (int i = WORDS * 64 - 1; i >= m; i--)
      if (bit_of(B, i - m)) C[i >> 6] ^= 1ULL << (i & 63);
    if (2 * Lc <= n) {
      Lc = n + 1 - Lc;
      memcpy(B, T, sizeof B);
      m = 1;
    } else {
      m++;
    }
  }
  /* characteristic polynomial = X^Lc C(1/X): reverse the coefficients */
  memset(p, 0, 5 * sizeof(uint64_t));
  for (int i = 0; i <= Lc; i++)
    if (bit_of(C, i)) p[(Lc - i) >> 6] |= 1ULL << ((Lc - i) & 63);
  if (Lc != 256) memset(p, 0, 5 * sizeof(uint64_t)); /* flagged to the caller by p[4] == 0 */
}

/* c <- a * b mod p (GF(2), 256-bit residues) */
static void xo_mulmod(const uint64_t a[4], const uint64_t b[4], const uint64_t p[5],
                      uint64_t c[4]) {
  uint64_t t[8] = {0};
  for (int i = 0; i < 256; i++) {
    if (!bit_of(a, i)) continue;
    const int w = i >> 6, sh = i & 63;
    for (int k = 0; k < 4; k++) {
      t[w + k] ^= b[k] << sh;
      if (sh) t[w + k + 1] ^= b[k] >> (64 - sh);
    }
  }
  for (int i = 510; i >= 256; i--) {
    if (!bit_of(t, i)) continue;
    const int off = i - 256, w = off >> 6, sh = off & 63;
    for (int k = 0; k < 5 && w + k < 8; k++) {
      t[w + k] ^= p[k] << sh;
      if (sh && w + k + 1 < 8) t[w + k + 1] ^= p[k] >> (64 - sh);
    }
  }
  memcpy(c, t, 4 * sizeof(uint64_t));
}

static uint64_t XO_P[5];
static pthread_once_t xo_p_once = PTHREAD_ONCE_INIT;
static void xo_p_init(void) { micsa_xoshiro_charpoly(XO_P); }

static const uint64_t *xo_poly(void) {
  pthread_once(&xo_p_once, xo_p_init);
  return XO_P;
}

void micsa_xoshiro_jump_poly(uint64_t o, uint64_t q[4]) {
  const uint64_t *p = xo_poly();
  uint64_t acc[4] = {1, 0, 0, 0}, base[4] = {2, 0, 0, 0};
  while (o) {
    if (o & 1) xo_mulmod(acc, base, p, acc);
    xo_mulmod(base, base, p, base);
    o >>= 1;
  }
  memcpy(q, acc, sizeof acc);
}

void micsa_xoshiro_apply(const uint64_t q[4], uint64_t s[4]) {
  uint64_t acc[4] = {0, 0, 0, 0}, cur[4] = {s[0], s[1], s[2], s[3]};
  for (int i = 0; i < 256; i++) {
    if (bit_of(q, i))
      for (int k = 0; k < 4; k++) acc[k] ^= cur[k];
    xo_step(cur);
  }
  memcpy(s, acc, sizeof acc);
}

/* ----------------------------------------------------------- streams */
static int lags_ok(const micsa_prc_t *u) {
  return (unsigned char)(u->ip - u->ip1) == LAG_A && (unsigned char)(u->ip - u->ip2) == R &&
         (unsigned char)(u->ip - u->ip3) == LAG_O;
}

int micsa_stream_record(const micsa_prc_t *prc, const micsa_xoshiro_t *xo,
                        uint64_t rec[MICSA_STREAM_REC]) {
  if (!lags_ok(prc)) return -1;
  for (int j = 0; j < LAG_O; j++) /* x_{-61+j} sits LAG_O - j slots behind ip */
    rec[j] = prc->ira[(unsigned char)(prc->ip - (LAG_O - j))];
  uint64_t *E = rec + (LAG_O - R);
  for (int k = R; k < 2 * R - 1; k++) E[k] = E[k - LAG_A] + E[k - R];
  rec[115] = prc->zseed;
  for (int k = 0; k < 4; k++) rec[116 + k] = xo->s[k];
  return 0;
}

/* Advance by n draws using precomputed jumps: fib = X^(n-202), lcg = the
 * congruential map of n-1 steps, q = X^(n-1) mod p.  n > 512. */
static void advance_with(micsa_prc_t *prc, micsa_xoshiro_t *xo, uint64_t n, const uint64_t *fib,
                         const uint64_t lcg[2], const uint64_t q[4]) {
  uint64_t rec[MICSA_STREAM_REC];
  micsa_stream_record(prc, xo, rec);
  const uint64_t *E = rec + (LAG_O - R);
  /* x_{n-257} .. x_{n-2}: the ring after n-1 steps */
  uint64_t v[256];
  for (int j = 0; j < R; j++) {
    uint64_t a = 0;
    for (int i = 0; i < R; i++) a += fib[i] * E[i + j];
    v[j] = a;
  }
  for (int j = R; j < 256; j++) v[j] = v[j - LAG_A] + v[j - R];
  const unsigned char ip0 = prc->ip;
  for (int j = 0; j < 256; j++) /* x_k lives in slot ip0 + k */
    prc->ira[(unsigned char)(ip0 + (n - 257) + (uint64_t)j)] = v[j];
  const unsigned char d = (unsigned char)(n - 1);
  prc->ip = (unsigned char)(prc->ip + d);
  prc->ip1 = (unsigned char)(prc->ip1 + d);
  prc->ip2 = (unsigned char)(prc->ip2 + d);
  prc->ip3 = (unsigned char)(prc->ip3 + d);
  prc->zseed = lcg[0] * prc->zseed + lcg[1];
  micsa_xoshiro_apply(q, xo->s);
  /* the last step runs as written, which also sets pr, out and t */
  micsa_prc_next(prc);
  micsa_xoshiro_next(xo);
}

void micsa_streams_advance(micsa_prc_t *prc, micsa_xoshiro_t *xo, uint64_t n) {
  if (n <= 512 || !lags_ok(prc)) {
    for (uint64_t k = 0; k < n; k++) {
      micsa_prc_next(prc);
      micsa_xoshiro_next(xo);
    }
    return;
  }
  uint64_t fib[R], lcg[2], q[4];
  micsa_fib_jump(n - 202, fib);
  micsa_lcg_jump(n - 1, &lcg[0], &lcg[1]);
  micsa_xoshiro_jump_poly(n - 1, q);
  advance_with(prc, xo, n, fib, lcg, q);
}

void micsa_streams_advance_plan(const micsa_refresh_plan *plan, micsa_prc_t *prc,
                                micsa_xoshiro_t *xo) {
  const uint64_t n = 64 * (uint64_t)plan->nwords;
  if (n <= 512)
    micsa_streams_advance(prc, xo, n);
  else
    advance_with(prc, xo, n, plan->adv_fib, plan->adv_lcg, plan->adv_xo);
}

/* ------------------------------------------------------------- plans */
int micsa_refresh_plan_make(int64_t nwords, int64_t words_per_seg, micsa_refresh_plan *plan) {
  memset(plan, 0, sizeof *plan);
  if (nwords < 1 || words_per_seg < 1) return -1;
  if (!xo_poly()[4]) return -1;
  const int64_t nseg = (nwords + words_per_seg - 1) / words_per_seg;
  const uint64_t S = 64 * (uint64_t)words_per_seg, M = 64 * (uint64_t)nwords;
  plan->nwords = nwords;
  plan->words_per_seg = words_per_seg;
  plan->nseg = nseg;
  plan->lcg = (uint64_t *)malloc(sizeof(uint64_t) * 2 * nseg);
  plan->xo = (uint64_t *)malloc(sizeof(uint64_t) * 4 * nseg);
  plan->fib = (uint64_t *)calloc((size_t)(R * nseg), sizeof(uint64_t));
  if (!plan->lcg || !plan->xo || !plan->fib) {
    micsa_refresh_plan_free(plan);
    return -1;
  }
  uint64_t sm, sa, qS[4], fS[R];
  micsa_lcg_jump(S, &sm, &sa);
  micsa_xoshiro_jump_poly(S, qS);
  micsa_fib_jump(S, fS);
  plan->lcg[0] = 1;
  plan->lcg[1] = 0;
  memset(plan->xo, 0, 4 * sizeof(uint64_t));
  plan->xo[0] = 1;
  if (nseg > 1) micsa_fib_jump(S - 6, plan->fib + R);
  for (int64_t g = 1; g < nseg; g++) {
    lcg_compose(sm, sa, plan->lcg[2 * (g - 1)], plan->lcg[2 * (g - 1) + 1], &plan->lcg[2 * g],
                &plan->lcg[2 * g + 1]);
    xo_mulmod(plan->xo + 4 * (g - 1), qS, xo_poly(), plan->xo + 4 * g);
    if (g > 1) fib_mulmod(plan->fib + R * (g - 1), fS, plan->fib + R * g);
  }
  if (M > 512) {
    micsa_lcg_jump(M - 1, &plan->adv_lcg[0], &plan->adv_lcg[1]);
    micsa_xoshiro_jump_poly(M - 1, plan->adv_xo);
    micsa_fib_jump(M - 202, plan->adv_fib);
  }
  return 0;
}

void micsa_refresh_plan_free(micsa_refresh_plan *plan) {
  free(plan->lcg);
  free(plan->xo);
  free(plan->fib);
  plan->lcg = plan->xo = plan->fib = NULL;
}

/* What one GPU lane does for segment g (k_refresh in micsa_refresh.cu). */
void micsa_draw_segment(const micsa_refresh_plan *plan, int64_t g,
                        const uint64_t rec[MICSA_STREAM_REC], const uint64_t thr[3], int nr,
                        int r, uint64_t *w0, uint64_t *w1) {
  uint64_t ring[64];
  const uint64_t *E = rec + (LAG_O - R);
  if (g == 0) {
    for (int j = 0; j < LAG_O; j++) ring[3 + j] = rec[j];
  } else {
    const uint64_t *c = plan->fib + R * g;
    for (int j = 0; j < R; j++) {
      uint64_t a = 0;
      for (int i = 0; i < R; i++) a += c[i] * E[i + j];
      ring[3 + j] = a;
    }
    for (int k = 0; k < LAG_O - R; k++) ring[3 + R + k] = ring[3 + R + k - LAG_A] + ring[3 + k];
  }
  uint64_t z = plan->lcg[2 * g] * rec[115] + plan->lcg[2 * g + 1];
  uint64_t s[4] = {rec[116], rec[117], rec[118], rec[119]};
  micsa_xoshiro_apply(plan->xo + 4 * g, s);
  int64_t i1 = (g + 1) * plan->words_per_seg;
  if (i1 > plan->nwords) i1 = plan->nwords;
  for (int64_t i = g * plan->words_per_seg; i < i1; i++) {
    uint64_t d0 = 0, d1 = 0;
    for (int b = 0; b < 64; b++) {
      const uint64_t xo_out = micsa_rotl64(s[0] + s[3], 23) + s[0];
      xo_step(s);
      const uint64_t xn = ring[(b - LAG_A) & 63] + ring[(b - R) & 63];
      const uint64_t pr = xn ^ ring[(b - LAG_O) & 63];
      ring[b] = xn;
      z = z * MICSA_LCG_A + 1;
      const uint64_t e = (z + pr) + xo_out;
      const int a0 = e < thr[0], a1 = e < thr[1], a2 = e < thr[2];
      d0 |= (uint64_t)(a0 ^ a1 ^ a2) << b;
      d1 |= (uint64_t)((a0 & a1) | (a0 & a2) | (a1 & a2)) << b;
    }
    w0[i * nr + r] = d0;
    w1[i * nr + r] = d1;
  }
}
