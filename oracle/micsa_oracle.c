/*
 * micsa_oracle.c -- TEST INFRASTRUCTURE ONLY (see micsa_oracle.h).
 *
 * Scalar-CPU restatement of the reference device path, written for
 * clarity: every kernel thread of the reference becomes one iteration of a
 * plain loop over (word h, replica r).  Each function names the reference
 * lines it follows.
 */
#include "micsa_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static int64_t half_words(int L) {
  int64_t m = L / 4;
  return m * m * m / 2;
}

/* ---- block-edge rotations (main.cu:706-742) ----
 * Bit b = bx + 4*by + 16*bz of a word is block (bx,by,bz).  Rotation "E"
 * moves block bx+1 into bx (the +x neighbour of the last column of block bx
 * is the first column of block bx+1); "O" is its inverse; N/S and U/D do
 * the same along y and z. */
static uint64_t rot_e(uint64_t v) {
  const uint64_t m = 0x1111111111111111ULL;
  return ((v & m) << 3) | ((v & ~m) >> 1);
}
static uint64_t rot_o(uint64_t v) {
  const uint64_t m = 0x8888888888888888ULL;
  return ((v & m) >> 3) | ((v & ~m) << 1);
}
static uint64_t rot_n(uint64_t v) {
  const uint64_t m = 0x000F000F000F000FULL;
  return ((v & m) << 12) | ((v & ~m) >> 4);
}
static uint64_t rot_s(uint64_t v) {
  const uint64_t m = 0xF000F000F000F000ULL;
  return ((v & m) >> 12) | ((v & ~m) << 4);
}
static uint64_t rot_u(uint64_t v) {
  const uint64_t m = 0x000000000000FFFFULL;
  return ((v & m) << 48) | ((v & ~m) >> 16);
}
static uint64_t rot_d(uint64_t v) {
  const uint64_t m = 0xFFFF000000000000ULL;
  return ((v & m) >> 48) | ((v & ~m) << 16);
}
typedef uint64_t (*rot_fn)(uint64_t);
static const rot_fn ROT[6] = {rot_e, rot_n, rot_u, rot_o, rot_s, rot_d};
/* rotation applied to the word that moves the opposite way (main.cu:1128-1176) */
static const rot_fn ROT_BACK[6] = {rot_o, rot_s, rot_d, rot_e, rot_n, rot_u};

/* The tables follow from coordinates: colour-p word h is the MSC site
 * (a,b,c) with h = (a + m*b + m*m*c)/2 and (a+b+c)&1 == p. */
void oracle_tables(int L, int32_t *neig, uint8_t *rot) {
  const int m = L / 4, mh = m / 2;
  const int64_t H = half_words(L);
  for (int p = 0; p < 2; p++)
    for (int64_t h = 0; h < H; h++) {
      int a2 = (int)(h % mh), b = (int)((h / mh) % m), c = (int)(h / ((int64_t)mh * m));
      int a = 2 * a2 + ((b + c + p) & 1);
      int na[6] = {(a + 1) % m, a, a, (a + m - 1) % m, a, a};
      int nb[6] = {b, (b + 1) % m, b, b, (b + m - 1) % m, b};
      int nc[6] = {c, c, (c + 1) % m, c, c, (c + m - 1) % m};
      int wrap[6] = {a == m - 1, b == m - 1, c == m - 1, a == 0, b == 0, c == 0};
      uint8_t r = 0;
      for (int d = 0; d < 6; d++) {
        int64_t msc = na[d] + (int64_t)m * nb[d] + (int64_t)m * m * nc[d];
        neig[(p * 6 + d) * H + h] = (int32_t)(msc / 2);
        if (wrap[d]) r |= (uint8_t)(1u << d);
      }
      rot[p * H + h] = r;
    }
}

typedef struct {
  int L;
  int64_t H;
  int32_t *neig;
  uint8_t *rot;
} tables_t;

static int make_tables(int L, tables_t *t) {
  t->L = L;
  t->H = half_words(L);
  t->neig = (int32_t *)malloc(sizeof(int32_t) * 12 * t->H);
  t->rot = (uint8_t *)malloc(2 * t->H);
  if (!t->neig || !t->rot) return -1;
  oracle_tables(L, t->neig, t->rot);
  return 0;
}
static void free_tables(tables_t *t) {
  free(t->neig);
  free(t->rot);
}

/* ISI demon algebra (main.cu:1037-1074): returns the flip mask and
 * updates D = D0 + 2*D1 in place. */
static uint64_t isi(uint64_t j1, uint64_t j2, uint64_t j3, uint64_t j4,
                    uint64_t *D0p, uint64_t *D1p) {
  uint64_t D0 = *D0p, D1 = *D1p;
  uint64_t x13 = j1 ^ j3, x24 = j2 ^ j4;
  uint64_t sub = (x24 & (~j1 & ~j3)) | (~j2 & ~j4);
  uint64_t s0 = ~x13;
  uint64_t s1 = ~x24 & (x13 | (s0 & ~(j1 ^ j2)));
  s1 = (~sub & s1) | (sub & (s1 ^ s0));
  uint64_t n0 = D0 ^ s0, k1 = D0 & s0, k2 = D1 ^ s1, n1 = k1 ^ k2, k3 = D1 & s1;
  uint64_t carry = (k3 | (k2 & k1)) ^ sub;
  uint64_t flip = ~carry;
  *D0p = (flip & n0) | (~flip & D0);
  *D1p = (flip & n1) | (~flip & D1);
  return flip;
}

uint64_t oracle_isi_word(uint64_t j1, uint64_t j2, uint64_t j3, uint64_t j4,
                         uint64_t *D0, uint64_t *D1) {
  return isi(j1, j2, j3, j4, D0, D1);
}

/* Body of d_oneMCstepBN_multisample (main.cu:899-1078) for one word. */
static void sweep_word(const tables_t *t, int nr, int p, int64_t h, int r,
                       const uint64_t *J, uint64_t *mine, const uint64_t *other,
                       uint64_t *d0, uint64_t *d1, const uint64_t *rand) {
  const int64_t H = t->H;
  const int32_t *ng = t->neig + (int64_t)p * 6 * H;
  const uint64_t *Jp = J + (int64_t)p * 6 * H;
  const uint64_t s = mine[h * nr + r];
  uint64_t n[6];
  for (int d = 0; d < 6; d++) {
    n[d] = other[(int64_t)ng[d * H + h] * nr + r];
    /* backward bonds sit at the owner's bit: xor before rotating */
    if (d >= 3) n[d] ^= Jp[d * H + h];
    if (t->rot[p * H + h] & (1u << d)) n[d] = ROT[d](n[d]);
  }
  uint64_t f0 = s ^ Jp[0 * H + h] ^ n[0];
  uint64_t f1 = s ^ Jp[1 * H + h] ^ n[1];
  uint64_t f2 = s ^ Jp[2 * H + h] ^ n[2];
  uint64_t f3 = n[3] ^ s, f4 = n[4] ^ s, f5 = n[5] ^ s;
  /* bit-sliced unsatisfied-bond counts j1+2*j2 (dirs 0-2), j3+2*j4 (3-5) */
  uint64_t j1 = f0 ^ f1 ^ f2;
  uint64_t j2 = (f0 & f1) ^ ((f0 ^ f1) & f2);
  uint64_t j3 = f3 ^ f4 ^ f5;
  uint64_t j4 = (f3 & f4) ^ ((f3 ^ f4) & f5);
  uint64_t flip;
  if (rand) {
    /* Metropolis against Bernoulli(e^{-4b k}) words (main.cu:945-957) */
    const int64_t stride = H * nr;
    uint64_t b0 = rand[h * nr + r];
    uint64_t b1 = rand[stride + h * nr + r] & b0;
    uint64_t b2 = rand[2 * stride + h * nr + r] & b1;
    uint64_t id2 = b1, id1 = (b0 ^ b1) | b2, j24 = j2 | j4;
    flip = (j1 & j3 & id1) | ((j24 | id2) & (j1 | j3 | id1)) | ((j2 & j4) | (j24 & id2));
  } else {
    /* microcanonical demon update, ISI algebra (main.cu:1037-1074) */
    flip = isi(j1, j2, j3, j4, &d0[h * nr + r], &d1[h * nr + r]);
  }
  mine[h * nr + r] = s ^ flip;
}

static void half_sweep_t(const tables_t *t, int nr, int nc, int p, int ic,
                         const uint64_t *J, uint64_t *even, uint64_t *odd,
                         uint64_t *w0, uint64_t *w1, const uint64_t *rand,
                         int r0, int r1) {
  const int64_t H = t->H;
  uint64_t *mine = p ? odd : even;
  const uint64_t *other = p ? even : odd;
  uint64_t *d0 = w0 ? w0 + ((int64_t)p * nc + ic) * H * nr : NULL;
  uint64_t *d1 = w1 ? w1 + ((int64_t)p * nc + ic) * H * nr : NULL;
  for (int64_t h = 0; h < H; h++)
    for (int r = r0; r < r1; r++) sweep_word(t, nr, p, h, r, J, mine, other, d0, d1, rand);
}

void oracle_half_sweep(int L, int nr, int nc, int p, int ic, const uint64_t *J,
                       uint64_t *even, uint64_t *odd, uint64_t *w0,
                       uint64_t *w1, const uint64_t *rand, int r0, int r1) {
  tables_t t;
  if (make_tables(L, &t)) return;
  half_sweep_t(&t, nr, nc, p, ic, J, even, odd, w0, w1, rand, r0, r1);
  free_tables(&t);
}

/* d_Walk (main.cu:1084-1193): the demon of colour-p word h on plane ic is
 * swapped with the one of its ic-neighbour (other colour), realigned across
 * block edges.  Launched for p = 0 then p = 1. */
static void walk_t(const tables_t *t, int nr, int nc, uint64_t *w0,
                   uint64_t *w1, int r0, int r1) {
  const int64_t H = t->H;
  for (int p = 0; p < 2; p++)
    for (int ic = 0; ic < nc; ic++) {
      uint64_t *a0 = w0 + ((int64_t)p * nc + ic) * H * nr;
      uint64_t *a1 = w1 + ((int64_t)p * nc + ic) * H * nr;
      uint64_t *b0 = w0 + ((int64_t)(1 - p) * nc + ic) * H * nr;
      uint64_t *b1 = w1 + ((int64_t)(1 - p) * nc + ic) * H * nr;
      const int32_t *ng = t->neig + ((int64_t)p * 6 + ic) * H;
      for (int64_t h = 0; h < H; h++) {
        const int wrap = (t->rot[p * H + h] >> ic) & 1;
        const int64_t n = ng[h];
        for (int r = r0; r < r1; r++) {
          uint64_t c0 = a0[h * nr + r], c1 = a1[h * nr + r];
          uint64_t s0 = b0[n * nr + r], s1 = b1[n * nr + r];
          if (wrap) {
            s0 = ROT[ic](s0);
            s1 = ROT[ic](s1);
            c0 = ROT_BACK[ic](c0);
            c1 = ROT_BACK[ic](c1);
          }
          a0[h * nr + r] = s0;
          a1[h * nr + r] = s1;
          b0[n * nr + r] = c0;
          b1[n * nr + r] = c1;
        }
      }
    }
}

void oracle_walk(int L, int nr, int nc, uint64_t *w0, uint64_t *w1, int r0,
                 int r1) {
  tables_t t;
  if (make_tables(L, &t)) return;
  walk_t(&t, nr, nc, w0, w1, r0, r1);
  free_tables(&t);
}

typedef struct {
  const tables_t *t;
  int nr, nc, r0, r1;
  const uint64_t *J;
  uint64_t *even, *odd, *w0, *w1;
} iter_job;

static void *iter_worker(void *arg) {
  iter_job *j = (iter_job *)arg;
  for (int ic = 0; ic < j->nc; ic++)
    for (int p = 0; p < 2; p++)
      half_sweep_t(j->t, j->nr, j->nc, p, ic, j->J, j->even, j->odd, j->w0,
                   j->w1, NULL, j->r0, j->r1);
  walk_t(j->t, j->nr, j->nc, j->w0, j->w1, j->r0, j->r1);
  return NULL;
}

/* Replicas never interact, so a replica range can run a whole iteration
 * on its own thread. */
void oracle_micsa_iteration(int L, int nr, int nc, const uint64_t *J,
                            uint64_t *even, uint64_t *odd, uint64_t *w0,
                            uint64_t *w1, int nthreads) {
  enum { MAXT = 256 };
  tables_t t;
  if (make_tables(L, &t)) return;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > nr) nthreads = nr;
  if (nthreads > MAXT) nthreads = MAXT;
  pthread_t tid[MAXT];
  int spawned[MAXT];
  iter_job job[MAXT];
  for (int k = 0; k < nthreads; k++) {
    job[k] = (iter_job){&t, nr, nc, nr * k / nthreads, nr * (k + 1) / nthreads,
                        J, even, odd, w0, w1};
    spawned[k] = k < nthreads - 1 &&
                 pthread_create(&tid[k], NULL, iter_worker, &job[k]) == 0;
    if (!spawned[k]) iter_worker(&job[k]);
  }
  for (int k = 0; k < nthreads; k++)
    if (spawned[k]) pthread_join(tid[k], NULL);
  free_tables(&t);
}

/* ---- Philox4x32-10 with the reference's post-mix and LUT bisection ---- */
static uint32_t umulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * b) >> 32);
}

/* _philox_4x32_10 (main.cu:562-595): 10 rounds, 9 key bumps. */
static void philox(uint32_t v[4], uint32_t k0, uint32_t k1) {
  for (int round = 0; round < 10; round++) {
    if (round) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t lo0 = 0xD2511F53u * v[0], hi0 = umulhi32(0xD2511F53u, v[0]);
    uint32_t lo1 = 0xCD9E8D57u * v[2], hi1 = umulhi32(0xCD9E8D57u, v[2]);
    uint32_t n0 = hi1 ^ v[1] ^ k0, n2 = hi0 ^ v[3] ^ k1;
    v[0] = n0;
    v[1] = lo1;
    v[2] = n2;
    v[3] = lo0;
  }
}

/* _bisection (main.cu:615-630): index n of the first threshold above the
 * 64-bit uniform (msb, lsb), via a 10-bit prebisection table.  The
 * thresholds are the LUT's 256 (x = high, y = low) pairs. */
static uint32_t bisect(uint32_t msb, uint32_t lsb, const uint32_t *thr,
                       const uint16_t *pre) {
#define BELOW(i) ((msb == thr[2 * (i)]) ? (lsb < thr[2 * (i) + 1]) : (msb < thr[2 * (i)]))
  uint32_t lo, hi;
  if (BELOW(254)) {
    uint16_t e = pre[msb >> (32 - 10)];
    lo = e & 255u;
    hi = e >> 8;
  } else {
    lo = hi = 255;
  }
  while (hi - lo > 1) {
    uint32_t mid = (hi + lo) >> 1;
    if (BELOW(mid))
      hi = mid;
    else
      lo = mid;
  }
  return BELOW(lo) ? lo : hi;
#undef BELOW
}

/* _get_rnd_word (main.cu:597-644): one Philox call -> four 64-bit
 * uniforms -> four bytes of Bernoulli bits -> rotated 32-bit word. */
static uint32_t rnd_word(uint32_t ctr[4], uint32_t k0, uint32_t k1,
                         const uint32_t *thr, const uint16_t *pre) {
  uint32_t v[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox(v, k0, k1);
  ctr[0]++;
  uint32_t hi = v[0] ^ v[2], lo = v[1] ^ v[3], l[4];
  l[0] = ((v[1] << 17) | (v[0] >> 15)) ^ hi ^ ((hi << 21) | (lo >> 11));
  l[1] = ((v[0] << 17) | (v[1] >> 15)) ^ lo ^ (lo << 21);
  l[2] = (hi << 28) | (lo >> 4);
  l[3] = (lo << 28) | (hi >> 4);
  uint32_t rot = (l[0] + v[1] + l[2] + v[3]) >> 27;
  uint32_t bb = 0;
  for (int k = 0; k < 4; k++) bb |= bisect(v[k], l[k], thr, pre) << (8 * k);
  return rot ? (bb << rot) | (bb >> (32 - rot)) : bb;
}

static void lut_unpack(const void *lut, uint32_t *thr, uint16_t *pre) {
  /* s_lut_heat_bath (header.h:113-116): 128 uint4 thresholds = 256
   * (high, low) uint32 pairs, then 128 uint4 = 1024 uint16 (min | max<<8) */
  memcpy(thr, lut, 2048);
  memcpy(pre, (const char *)lut + 2048, 2048);
}

/* d_gen_rndbits_cuda (main.cu:647-702) with NBETAS = 1. */
void oracle_gen_rndbits(int L, int nr, const uint32_t *te, const uint32_t *keys,
                        const void *lut, uint64_t *out) {
  uint32_t thr[512];
  uint16_t pre[1024];
  lut_unpack(lut, thr, pre);
  const int64_t H = half_words(L), n = H * nr;
  for (int64_t tid = 0; tid < n; tid++) {
    int r = (int)(tid % nr);
    uint32_t c[4] = {te[4 * r], te[4 * r + 1], te[4 * r + 2] + (uint32_t)tid, te[4 * r + 3]};
    uint64_t w[3];
    for (int k = 0; k < 3; k++) {
      uint64_t hi = rnd_word(c, (uint32_t)tid, keys[r], thr, pre);
      uint64_t lo = rnd_word(c, (uint32_t)tid, keys[r], thr, pre);
      w[k] = (hi << 32) | lo;
    }
    for (int k = 0; k < 3; k++) out[k * n + tid] = w[k];
  }
}

void oracle_metropolis_iteration(int L, int nr, const uint64_t *J,
                                 uint64_t *even, uint64_t *odd,
                                 const uint32_t *te0, const uint32_t *te1,
                                 const uint32_t *keys, const void *lut) {
  const int64_t n = half_words(L) * nr;
  uint64_t *rnd = (uint64_t *)malloc(sizeof(uint64_t) * 3 * n);
  if (!rnd) return;
  oracle_gen_rndbits(L, nr, te0, keys, lut, rnd);
  oracle_half_sweep(L, nr, 1, 0, 0, J, even, odd, NULL, NULL, rnd, 0, nr);
  oracle_gen_rndbits(L, nr, te1, keys, lut, rnd);
  oracle_half_sweep(L, nr, 1, 1, 0, J, even, odd, NULL, NULL, rnd, 0, nr);
  free(rnd);
}

/* d_computeEne (main.cu:745-815) on the even colour: each of the 6 bonds
 * of every even site counted once; h_Ener = 6*64*H - 2*unsatisfied. */
void oracle_energy(int L, int nr, const uint64_t *J, const uint64_t *even,
                   const uint64_t *odd, int32_t *ener) {
  tables_t t;
  if (make_tables(L, &t)) return;
  const int64_t H = t.H;
  for (int r = 0; r < nr; r++) {
    int64_t un = 0;
    for (int64_t h = 0; h < H; h++) {
      const uint64_t s = even[h * nr + r];
      for (int d = 0; d < 6; d++) {
        uint64_t n = odd[(int64_t)t.neig[d * H + h] * nr + r];
        uint64_t f;
        if (d < 3) {
          if (t.rot[h] & (1u << d)) n = ROT[d](n);
          f = s ^ J[d * H + h] ^ n;
        } else {
          n ^= J[d * H + h];
          if (t.rot[h] & (1u << d)) n = ROT[d](n);
          f = n ^ s;
        }
        un += __builtin_popcountll(f);
      }
    }
    ener[r] = (int32_t)(6 * 64 * H - 2 * un);
  }
  free_tables(&t);
}

/* Measure_Energy_Clerics (med.c:55-83). */
void oracle_demon_energy(int L, int nr, int nc, const uint64_t *w0,
                         const uint64_t *w1, uint64_t *ener) {
  const int64_t nw = 2 * half_words(L) * nc;
  for (int r = 0; r < nr; r++) {
    uint64_t e = 0;
    for (int64_t i = 0; i < nw; i++)
      e += (uint64_t)__builtin_popcountll(w0[i * nr + r]) +
           2ULL * (uint64_t)__builtin_popcountll(w1[i * nr + r]);
    ener[r] = e;
  }
}

/* ---- scalar rendering ---- */

/* With u unsatisfied bonds a flip changes the spin energy by 12 - 4u; the
 * demon (energy 4*D, D = 0..3) pays it: accepted iff 0 <= D + u - 3 <= 3. */
int oracle_scalar_rule(int unsatisfied, int demon, int *flip) {
  int d = demon + unsatisfied - 3;
  *flip = d >= 0 && d <= 3;
  return *flip ? d : demon;
}

void oracle_overlap_c4(int L, int nr, const uint8_t *uu, int64_t *q,
                       int64_t *c4) {
  const int64_t V = (int64_t)L * L * L;
  const int nd = L / 2 + 1;
  uint8_t *dq = (uint8_t *)malloc((size_t)V);
  if (!dq) return;
  for (int k = 0; k < nr / 2; k++) {
    const uint8_t *a = uu + (int64_t)(2 * k) * V, *b = uu + (int64_t)(2 * k + 1) * V;
    int64_t diff = 0;
    for (int64_t s = 0; s < V; s++) {
      dq[s] = (a[s] ^ b[s]) & 1;
      diff += dq[s];
    }
    if (q) q[k] = V - 2 * diff;
    if (!c4) continue;
    for (int axis = 0; axis < 3; axis++)
      for (int d = 0; d < nd; d++) {
        int64_t x_ = 0;
        for (int z = 0; z < L; z++)
          for (int y = 0; y < L; y++)
            for (int x = 0; x < L; x++) {
              int xs = x, ys = y, zs = z;
              if (axis == 0) xs = (x + d) % L;
              if (axis == 1) ys = (y + d) % L;
              if (axis == 2) zs = (z + d) % L;
              x_ += dq[x + (int64_t)L * y + (int64_t)L * L * z] ^
                    dq[xs + (int64_t)L * ys + (int64_t)L * L * zs];
            }
        c4[((int64_t)k * 3 + axis) * nd + d] = V - 2 * x_;
      }
  }
  free(dq);
}

/* calculate_scalar_energy (med.c:85-114): 3V - 2 * unsatisfied bonds. */
int32_t oracle_scalar_energy(int L, const uint8_t *u, const uint8_t *Jx,
                             const uint8_t *Jy, const uint8_t *Jz) {
  int64_t e = 0;
  for (int z = 0; z < L; z++)
    for (int y = 0; y < L; y++)
      for (int x = 0; x < L; x++) {
        int64_t s = x + (int64_t)L * y + (int64_t)L * L * z;
        int64_t sx = (x + 1) % L + (int64_t)L * y + (int64_t)L * L * z;
        int64_t sy = x + (int64_t)L * ((y + 1) % L) + (int64_t)L * L * z;
        int64_t sz = x + (int64_t)L * y + (int64_t)L * L * ((z + 1) % L);
        e += (u[s] ^ Jx[s] ^ u[sx]) + (u[s] ^ Jy[s] ^ u[sy]) + (u[s] ^ Jz[s] ^ u[sz]);
      }
  int64_t V = (int64_t)L * L * L;
  return (int32_t)(3 * V - 2 * e);
}

/* packing_J (ini.c:521-578): coupling of site (x,y,z) along +d goes to bit
 * bx + 4*by + 16*bz of the site's own forward word d and of its
 * +d neighbour's backward word d+3 (ini.c:553-564); rows are then taken per
 * colour in word order (viciniB/N, ini.c:569-575), which here is msc/2. */
void oracle_pack_couplings(int L, const uint8_t *Jx, const uint8_t *Jy,
                           const uint8_t *Jz, uint64_t *J) {
  const int m = L / 4;
  const int64_t H = half_words(L);
  const uint8_t *Jd[3] = {Jx, Jy, Jz};
  memset(J, 0, sizeof(uint64_t) * 12 * H);
  for (int z = 0; z < L; z++)
    for (int y = 0; y < L; y++)
      for (int x = 0; x < L; x++) {
        const int64_t site = x + (int64_t)L * y + (int64_t)L * L * z;
        const int a = x % m, b = y % m, c = z % m;
        const uint64_t bit = (uint64_t)(x / m + 4 * (y / m) + 16 * (z / m));
        const int p = (a + b + c) & 1;
        for (int d = 0; d < 3; d++) {
          const int na = d == 0 ? (a + 1) % m : a, nb = d == 1 ? (b + 1) % m : b,
                    nc = d == 2 ? (c + 1) % m : c;
          const int64_t own = (a + (int64_t)m * b + (int64_t)m * m * c) / 2;
          const int64_t nbr = (na + (int64_t)m * nb + (int64_t)m * m * nc) / 2;
          const uint64_t v = (uint64_t)(Jd[d][site] & 1) << bit;
          J[(int64_t)(p * 6 + d) * H + own] |= v;
          J[(int64_t)((p ^ 1) * 6 + d + 3) * H + nbr] |= v;
        }
      }
}
