/*
 * Seeding generators of the micSA drop-in.  Reproduces, in behaviour and
 * output bits, PROGRAM/src/random_generator.cu of IsidoroGlez/micSA-EA-MC.
 * The reference keeps the Luescher generator and the Janus generator in
 * globals; here each lives in a caller-owned struct so that independent
 * samples and threads never share state.
 */
#include "micsa_host.h"

#include <stdio.h>
#include <string.h>

_Static_assert(sizeof(micsa_prc_t) == 2080, "s_aleatorio_HQ_64bits layout");
_Static_assert(sizeof(micsa_xoshiro_t) == 48, "s_xoshiro256pp layout");

/* comprueba_semilla / lee_urandom (random_generator.cu:11-26): a zero seed
 * means "draw one from /dev/urandom". */
uint64_t micsa_check_seed(uint64_t seed) {
  if (seed) return seed;
  uint64_t v = 0;
  FILE *f = fopen("/dev/urandom", "rb");
  if (f) {
    if (fread(&v, sizeof v, 1, f) != 1) v = 0;
    fclose(f);
  }
  return v;
}

/* Init_luxury (random_generator.cu:27-55). */
void micsa_luxury_seed(micsa_luxury_t *g, uint64_t seed) {
  memset(g, 0, sizeof *g);
  g->ip = 128;
  g->ip1 = (unsigned char)(128 - 10);
  g->ip2 = (unsigned char)(128 - 24);
  for (int i = 0; i < 1111; i++) seed = seed * MICSA_LCG_A + 1;
  for (int j = g->ip2; j < g->ip; j++) {
    uint64_t v = 0;
    for (int i = 0; i < 3; i++) {
      seed = seed * MICSA_LCG_A + 1;
      v |= (seed >> 56) << (8 * i);
    }
    g->x[j] = (uint32_t)v;
  }
  seed = seed * MICSA_LCG_A + 1;
  g->borrow = (int)(seed >> 63);
  for (int i = 0; i < 1111; i++) (void)micsa_luxury_next(g);
}

/* luxury (random_generator.cu:57-75): 389 subtract-with-borrow steps, then
 * the slot AFTER the last one written is returned (as the reference does). */
uint32_t micsa_luxury_next(micsa_luxury_t *g) {
  for (int i = 0; i < 389; i++) {
    int32_t d = (int32_t)(g->x[g->ip1] - g->x[g->ip2] - (uint32_t)g->borrow);
    g->x[g->ip] = (uint32_t)(d + 16777216) & 16777215u;
    g->borrow = (d < 0) ? 1 : 0;
    g->ip++; g->ip1++; g->ip2++;
  }
  return g->x[g->ip];
}

/* Luescher_PRNG (random_generator.cu:77-91): top byte of 8 outputs. */
uint64_t micsa_luxury_u64(micsa_luxury_t *g) {
  uint64_t v = 0;
  for (int j = 0; j < 8; j++) v |= ((uint64_t)micsa_luxury_next(g) >> 16) << (8 * j);
  return v;
}

/* Inicia_generadores_CPU (random_generator.cu:94-158). */
void micsa_init_cpu_generators(micsa_prc_t *prc, micsa_xoshiro_t *xo,
                               uint32_t *key, uint64_t seed) {
  micsa_luxury_t g;
  micsa_prc_t s;
  memset(&s, 0, sizeof s);
  micsa_luxury_seed(&g, micsa_check_seed(seed));
  for (int i = 0; i < 1111; i++) (void)micsa_luxury_next(&g);
  s.zseed = micsa_luxury_u64(&g);
  for (int k = 128 - 61; k < 128; k++) s.ira[k] = micsa_luxury_u64(&g);
  s.ip = 128;
  s.ip1 = 128 - 24;
  s.ip2 = 128 - 55;
  s.ip3 = 128 - 61;
  for (int i = 0; i < 2222; i++) (void)micsa_prc_next(&s);
  *prc = s;

  uint64_t st[4] = {0, 0, 0, 0};
  while (!(st[0] | st[1] | st[2] | st[3])) {
    for (int j = 0; j < 4; j++) {
      st[j] = 0;
      for (int i = 0; i < 64; i++)
        st[j] |= (((uint64_t)micsa_luxury_next(&g) >> 23) & 1ULL) << i;
    }
  }
  memset(xo, 0, sizeof *xo);
  for (int j = 0; j < 4; j++) xo->s[j] = st[j];

  uint32_t k32 = 0;
  for (int i = 0; i < 32; i++) k32 |= ((micsa_luxury_next(&g) >> 23) & 1u) << i;
  *key = k32;
}

/* Init_Rand_HQ_64bits (random_generator.cu:160-200). */
void micsa_init_rand_hq(micsa_prc_t *prc, uint64_t seed) {
  micsa_prc_t s;
  memset(&s, 0, sizeof s);
  s.zseed = micsa_check_seed(seed);
  for (int i = 0; i < 111; i++) s.zseed = s.zseed * MICSA_LCG_A + 1;
  for (int k = 128 - 61; k < 128; k++) {
    s.ira[k] = 0;
    for (int i = 0; i < 8; i++) {
      s.zseed = s.zseed * MICSA_LCG_A + 1;
      s.ira[k] |= (s.zseed >> 56) << (8 * i);
    }
  }
  s.ip = 128;
  s.ip1 = 128 - 24;
  s.ip2 = 128 - 55;
  s.ip3 = 128 - 61;
  for (int i = 0; i < 1111; i++) {
    s.ira[s.ip] = s.ira[s.ip1] + s.ira[s.ip2];
    s.ip++; s.ip1++; s.ip2++; s.ip3++;
  }
  for (int i = 0; i < 1111; i++) (void)micsa_prc_next(&s);
  *prc = s;
}

/* generate_seeds_from_one (random_generator.cu:202-234).  The reference
 * overwrites its random draw with a constant before choosing how many
 * outputs to skip, so the skip is always 109; the discarded draw is kept. */
void micsa_seeds_from_one(uint64_t *seed, uint64_t *out, int n) {
  micsa_luxury_t g;
  *seed = micsa_check_seed(*seed);
  micsa_luxury_seed(&g, *seed);
  for (int i = 0; i < 1109; i++) (void)micsa_luxury_next(&g);
  for (int k = 0; k < n; k++) {
    (void)micsa_luxury_u64(&g);
    uint32_t sel = (uint32_t)((MICSA_LCG_A + 1) >> 61);
    int skip = sel == 0 ? 709 : sel == 1 ? 109 : sel == 2 ? 1373 : 2099;
    for (int i = 0; i < skip; i++) (void)micsa_luxury_next(&g);
    uint64_t v = micsa_luxury_u64(&g);
    out[k] = v * 6364136223846793005ULL + 14426950408889634071ULL;
  }
}

/* ini_random (random_generator.cu:238-256). */
void micsa_janus_seed(micsa_janus_t *g, uint64_t seed) {
  memset(g, 0, sizeof *g);
  g->zseed = seed;
  for (int i = 0; i < 11; i++) g->zseed = g->zseed * MICSA_LCG_A + 1;
  g->ip = 128;
  g->ip1 = 128 - 24;
  g->ip2 = 128 - 55;
  g->ip3 = 128 - 61;
  for (int i = g->ip3; i < g->ip; i++) {
    g->zseed = g->zseed * MICSA_LCG_A + 1;
    g->ira[i] = g->zseed;
  }
  for (int i = 0; i < 1111; i++) {
    uint64_t v = g->ira[g->ip1] + g->ira[g->ip2];
    g->ira[g->ip] = v;
    g->ip++; g->ip1++; g->ip2++; g->ip3++;
  }
}
