/*
 * micsa_host.h -- host side of the micSA drop-in: the random-number streams,
 * seed fan-out, lattice initialisation, demon draws and the Philox counter
 * layout that decide, bit for bit, what the GPU sweeps consume.
 *
 * Everything here follows IsidoroGlez/micSA-EA-MC (PROGRAM/); each function
 * cites the reference file:line whose behaviour it reproduces.  The structs
 * that the reference writes raw into checkpoint files keep the reference's
 * byte layout (sizes are asserted in micsa_rng.c).
 */
#ifndef MICSA_HOST_H
#define MICSA_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parisi-Rapuano lagged Fibonacci (lags 24, 55, output xor lag 61) plus a
 * 64-bit congruential generator; same 2080-byte layout as
 * s_aleatorio_HQ_64bits (include/random_generator.h:28-36). */
typedef struct {
  uint64_t ira[256];
  uint64_t pr;
  uint64_t zseed;
  uint64_t out;
  unsigned char ip, ip1, ip2, ip3;
  unsigned char pad[4];
} micsa_prc_t;

/* xoshiro256++ (Blackman & Vigna); same 48-byte layout as s_xoshiro256pp
 * (include/random_generator.h:39-44). */
typedef struct {
  uint64_t s[4];
  uint64_t t;
  uint64_t out;
} micsa_xoshiro_t;

/* 24-bit subtract-with-borrow generator with luxury decimation (389 steps
 * per output), used only to seed the others (random_generator.cu:27-91). */
typedef struct {
  uint32_t x[256];
  int borrow;
  unsigned char ip, ip1, ip2;
} micsa_luxury_t;

/* Janus coupling generator: PR + congruential, summed
 * (random_generator.h:72-86, random_generator.cu:238-256). */
typedef struct {
  uint64_t ira[256];
  uint64_t zseed;
  unsigned char ip, ip1, ip2, ip3;
} micsa_janus_t;

#define MICSA_LCG_A 3202034522624059733ULL

static inline uint64_t micsa_rotl64(uint64_t x, int k) {
  return (x << k) | (x >> (64 - k));
}

/* One step of _actualiza_aleatorio_HQ_escalar (random_generator.h:62-67). */
static inline uint64_t micsa_prc_next(micsa_prc_t *u) {
  u->ira[u->ip] = u->ira[u->ip1] + u->ira[u->ip2];
  u->pr = u->ira[u->ip] ^ u->ira[u->ip3];
  u->zseed = u->zseed * MICSA_LCG_A + 1;
  u->out = u->zseed + u->pr;
  u->ip++; u->ip1++; u->ip2++; u->ip3++;
  return u->out;
}

/* One step of _actualiza_xoshiro256pp (random_generator.h:50-59). */
static inline uint64_t micsa_xoshiro_next(micsa_xoshiro_t *u) {
  u->out = micsa_rotl64(u->s[0] + u->s[3], 23) + u->s[0];
  u->t = u->s[1] << 17;
  u->s[2] ^= u->s[0];
  u->s[3] ^= u->s[1];
  u->s[1] ^= u->s[2];
  u->s[0] ^= u->s[3];
  u->s[2] ^= u->t;
  u->s[3] = micsa_rotl64(u->s[3], 45);
  return u->out;
}

/* HIRANDOM (random_generator.h:83-85). */
static inline uint64_t micsa_janus_next(micsa_janus_t *g) {
  uint64_t v = g->ira[g->ip1] + g->ira[g->ip2];
  g->ira[g->ip] = v;
  uint64_t pr = v ^ g->ira[g->ip3];
  g->ip++; g->ip1++; g->ip2++; g->ip3++;
  g->zseed = g->zseed * MICSA_LCG_A + 1;
  return pr + g->zseed;
}

/* ---- seeding (random_generator.cu) ---- */
uint64_t micsa_check_seed(uint64_t seed);                          /* :11-16 */
void micsa_luxury_seed(micsa_luxury_t *g, uint64_t seed);          /* :27-55 */
uint32_t micsa_luxury_next(micsa_luxury_t *g);                     /* :57-75 */
uint64_t micsa_luxury_u64(micsa_luxury_t *g);                      /* :77-91 */
void micsa_init_cpu_generators(micsa_prc_t *prc, micsa_xoshiro_t *xo,
                               uint32_t *key, uint64_t seed);      /* :94-158 */
void micsa_init_rand_hq(micsa_prc_t *prc, uint64_t seed);          /* :160-200 */
void micsa_seeds_from_one(uint64_t *seed, uint64_t *out, int n);   /* :202-234 */
void micsa_janus_seed(micsa_janus_t *g, uint64_t seed);            /* :238-256 */

/* ---- lattice geometry (ini.c:119-258, 301-395) ----
 * Sites are (x,y,z), 0 <= x,y,z < L, L a multiple of 8.  The reference's
 * multispin-coded (MSC) form cuts the lattice into 4x4x4 blocks of side L/4;
 * one 64-bit word holds the 64 sites that share the in-block coordinate
 * (a,b,c), bit = bx + 4*by + 16*bz.  Words are split by the colour
 * (a+b+c)&1 ("bianchi" = 0, "neri" = 1) and h = (a + (L/4)*b + (L/4)^2*c)/2
 * indexes a colour half of H = (L/4)^3/2 words. */
int64_t micsa_half_words(int L);                                   /* H */
/* real site of (colour p, word h, bit) */
void micsa_msc_site(int L, int p, int64_t h, int bit, int *x, int *y, int *z);
/* packing_u (ini.c:301-345): uu[r*V + site] (site = x + L*y + L*L*z) ->
 * even/odd words [H][nr] */
void micsa_pack_spins(int L, int nr, const uint8_t *uu, uint64_t *even,
                      uint64_t *odd);
/* unpacking_u (ini.c:347-395) */
void micsa_unpack_spins(int L, int nr, const uint64_t *even,
                        const uint64_t *odd, uint8_t *uu);
/* packing_J (ini.c:521-578): per-site bonds Jx,Jy,Jz (to +x,+y,+z) ->
 * J[(p*6 + d)*H + h], d = E,N,U,O,S,D as in viciniB/N[h].J[d] */
void micsa_pack_couplings(int L, const uint8_t *Jx, const uint8_t *Jy,
                          const uint8_t *Jz, uint64_t *J);

/* ---- model initialisation (ini.c) ---- */
/* Init_u (ini.c:275-299): spins of nbits samples, uu[ibit][r][site] */
int micsa_init_spins(micsa_prc_t *random_u, int L, int nr, int maxnsamples,
                     const int *list_samples, int nbits, uint8_t *uu);
/* Init_J under -DJANUS (ini.c:457-471): returns the number of J=1 bonds */
int micsa_init_couplings_janus(uint64_t seed, int L, uint8_t *Jx,
                               uint8_t *Jy, uint8_t *Jz);
/* get_thresholds (ini.c:680-710), computed in binary128 */
void micsa_thresholds(double beta, uint64_t thr[3]);
/* LUT builder (input/LUT/preparation.c:265-388): 4096-byte s_lut_heat_bath */
void micsa_build_lut(double beta, void *out);
/* InitWalkers (ini.c:712-781) for ONE replica stream: fills words
 * w[i*nr + r], i = 0 .. 2*H*nc-1, of the CPUwalker0/1 layout */
void micsa_draw_demons(micsa_prc_t *prc, micsa_xoshiro_t *xo,
                       const uint64_t thr[3], int L, int nr, int nc, int r,
                       uint64_t *w0, uint64_t *w1);
/* All nr streams of one sample in parallel threads (the streams are
 * independent, so the result equals the reference's serial loop). */
int micsa_draw_demons_all(micsa_prc_t *prc, micsa_xoshiro_t *xo,
                          const uint64_t thr[3], int L, int nr, int nc,
                          uint64_t *w0, uint64_t *w1, int nthreads);
/* _fill_bits (include/fill_bits.h:47-68): advances the nr Metropolis
 * streams once and writes the Philox counters te[r*4 + {x,y,z,w}] */
void micsa_fill_bits(micsa_prc_t *prc, micsa_xoshiro_t *xo, int nr,
                     uint64_t iter, int parity, uint32_t jobid, uint32_t *te);

/* ---- measurement arithmetic (med.c:3-53, io.c:395-462) ---- */
/* mean and sample std of -E/V over replicas, in the reference's operation
 * order; e_spin[r] are the integer energies h_Ener */
void micsa_energy_stats(const int32_t *e_spin, int nr, int L, double *mean,
                        double *std);
/* mean and std of the demon energy per site per demon */
void micsa_demon_stats(const uint64_t *e_demon, int nr, int L, int nc,
                       double *mean, double *std);

/* ---- observables beyond the reference ----
 * c4[(k*3 + axis)*(L/2+1) + d] of npairs replica pairs (micsa_measure's
 * layout for one sample) -> C4r[d] (pair- and axis-averaged, / V), err[d]
 * (its standard error over the pairs) and the integral-estimator
 * correlation lengths xi12, xi23 summed over r < *rcut: the first r >= 1
 * where C4r < kappa * err (kappa > 0), at most rmax + 1 (rmax > 0); kappa =
 * rmax = 0 sums the whole range.  C4r, err and rcut may be NULL. */
#define MICSA_XI_KAPPA 3.0 /* the cut-off the driver's evol_xi.txt uses */
void micsa_correlation_lengths(int L, int npairs, const int64_t *c4, double kappa, int rmax,
                               double *C4r, double *err, double *xi12, double *xi23, int *rcut);

#ifdef __cplusplus
}
#endif
#endif
