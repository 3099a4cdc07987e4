/*
 * File formats and run control of the micSA drop-in driver: the reference's
 * input files, output directory tree, measurement files, seed files,
 * checkpoints and lock/error files (PROGRAM/src/io.c, timing.c).
 * Binary records keep the reference's byte layout so that files move
 * between the two programs.
 */
#ifndef MICSA_IO_H
#define MICSA_IO_H

#include <stdint.h>
#include <stdio.h>

#include "micsa_host.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MICSA_MAXSTR 1024

/* s_data (header.h:98-111) with the replica count known at run time */
typedef struct {
  unsigned long long maxtime, now;
  int ntimes, nterm, nc, nr, l, flag;
  uint64_t seed_J, seed_u;
  uint64_t *seed_MC; /* nr entries */
} micsa_data;

/* icds (header.h:69-78): 40 bytes on disk */
typedef struct {
  unsigned int first, isample, Nrep, NUM_WALKERS_PER_SITE, Lv, t;
  unsigned long long seed;
  double beta;
} micsa_icds;

/* read_input (io.c:464-502): path line, 2 ULL, 6 int, 2 + nr seeds; a short
 * file repeats its last line, as fgets into an unchanged buffer does.
 * Returns 0 or -1 with msg filled. */
int micsa_read_input(const char *name, char *dir, micsa_data *d, char *msg, size_t n);
void micsa_free_data(micsa_data *d);
/* print_data (io.c:518-532) */
void micsa_print_data(FILE *f, const micsa_data *d);
/* read_betas (io.c:534-558), NBETAS = 1 */
int micsa_read_beta(const char *name, double *beta, char *msg, size_t n);
/* read_lut (io.c:561-591): beta check, then the 4096-byte table */
int micsa_read_lut(const char *name, double beta, void *lut, char *msg, size_t n);
/* read_list_times (io.c:626-655); *times malloc'd */
int micsa_read_times(const char *name, int ntimes, unsigned long long **times, char *msg,
                     size_t n);
/* read_list_samples (io.c:593-624) */
int micsa_read_samples(const char *name, int nbits, int *list, char *msg, size_t n);

/* binary record sizes (io.c:23-26, 260-262) */
int64_t micsa_conf_bytes(int L, int nr);
int64_t micsa_walkers_bytes(int L, int nr, int nc);
/* serialise s_data exactly as fwrite(&data, sizeof(s_data)) does */
int micsa_write_data_record(FILE *f, const micsa_data *d);
int micsa_read_data_record(FILE *f, micsa_data *d);

/* write one conf.<t> record (io.c:17-96): data, beta, the replica's
 * Metropolis streams, permutation byte, spins 1 bit/site (x fastest, LSB
 * first), energy */
int micsa_write_conf_record(FILE *f, const micsa_data *d, double beta,
                            const micsa_prc_t *prc, const micsa_xoshiro_t *xo,
                            const uint8_t *u, int L, int32_t energy);
/* compact_dump (io.c:1125-1145): 8 sites per byte, LSB first */
void micsa_pack_bits(const uint8_t *u, int64_t n, uint8_t *out);
void micsa_unpack_bits(const uint8_t *in, int64_t n, uint8_t *u);

/* timing.c:3-33: prints "<s>s (<ps per spin-flip attempt> ps/s, <cpu%>%): " */
void micsa_measure_time(int L, int nr, int nbits, int nc, unsigned long long t);
/* timing.c:35-58: 1 when the next block would exceed max_time seconds */
int micsa_check_time(unsigned long long max_time, unsigned long long dt0,
                     unsigned long long dt1);

#ifdef __cplusplus
}
#endif
#endif
