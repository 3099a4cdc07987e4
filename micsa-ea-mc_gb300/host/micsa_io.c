/*
 * Input parsing, binary records and timing of the micSA drop-in
 * (reference: PROGRAM/src/io.c and PROGRAM/src/timing.c).
 */
#include "micsa_io.h"

#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static int err(char *msg, size_t n, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, n, fmt, ap);
  va_end(ap);
  return -1;
}

int micsa_read_input(const char *name, char *dir, micsa_data *d, char *msg, size_t n) {
  FILE *f = fopen(name, "r");
  if (!f) return err(msg, n, "Error: No file %s\n", name);
  char line[MICSA_MAXSTR + 1] = {0};
  memset(d, 0, sizeof *d);
  if (!fgets(line, MICSA_MAXSTR, f)) line[0] = 0;
  dir[0] = 0;
  sscanf(line, "%1023s", dir);
  unsigned long long *ull[2] = {&d->maxtime, &d->now};
  for (int j = 0; j < 2; j++) {
    if (!fgets(line, MICSA_MAXSTR, f)) { /* keep the previous line */ }
    sscanf(line, "%llu", ull[j]);
  }
  int *ints[6] = {&d->ntimes, &d->nterm, &d->nc, &d->nr, &d->l, &d->flag};
  for (int j = 0; j < 6; j++) {
    if (!fgets(line, MICSA_MAXSTR, f)) { /* keep the previous line */ }
    sscanf(line, "%u", (unsigned *)ints[j]);
  }
  if (d->nr <= 0 || d->nr > 4096) {
    fclose(f);
    return err(msg, n, "d.nr = %d is not a usable replica count\n", d->nr);
  }
  d->seed_MC = (uint64_t *)calloc((size_t)d->nr, sizeof(uint64_t));
  if (!d->seed_MC) {
    fclose(f);
    return err(msg, n, "out of memory\n");
  }
  for (int j = 0; j < 2 + d->nr; j++) {
    if (!fgets(line, MICSA_MAXSTR, f)) { /* keep the previous line */ }
    unsigned long long v = 0;
    if (j == 0) v = d->seed_J; else if (j == 1) v = d->seed_u; else v = d->seed_MC[j - 2];
    sscanf(line, "%llu", &v);
    if (j == 0) d->seed_J = v; else if (j == 1) d->seed_u = v; else d->seed_MC[j - 2] = v;
  }
  fclose(f);
  if (d->nterm < 0 || d->nc < 0 || d->ntimes < 0)
    return err(msg, n, "Bad data input\n");
  return 0;
}

void micsa_free_data(micsa_data *d) {
  free(d->seed_MC);
  d->seed_MC = NULL;
}

void micsa_print_data(FILE *f, const micsa_data *d) {
  fprintf(f, "maxtime      %16llu\n", d->maxtime);
  fprintf(f, "now          %16llu\n", d->now);
  fprintf(f, "ntimes       %16d\n", d->ntimes);
  fprintf(f, "nterm        %16d\n", d->nterm);
  fprintf(f, "nr           %16d\n", d->nr);
  fprintf(f, "nc           %16d\n", d->nc);
  fprintf(f, "L            %16d\n", d->l & 0xffff);
  fprintf(f, "M            %16d\n", d->l >> 16);
  fprintf(f, "flag         %16d\n", d->flag);
  fprintf(f, "seed_J       %016llx\n", (unsigned long long)d->seed_J);
  fprintf(f, "seed_u       %016llx\n", (unsigned long long)d->seed_u);
  for (int r = 0; r < d->nr; r++)
    fprintf(f, "seed_MC[%d]   %016llx\n", r, (unsigned long long)d->seed_MC[r]);
}

int micsa_read_beta(const char *name, double *beta, char *msg, size_t n) {
  FILE *f = fopen(name, "rt");
  if (!f) return err(msg, n, "File %s doesn't exist.\n", name);
  if (fscanf(f, "%lf ", beta) == EOF) {
    fclose(f);
    return err(msg, n, "File %s only has %d lines (it needs %d)\n", name, 0, 1);
  }
  double dummy;
  if (fscanf(f, "%lf", &dummy) != EOF) fprintf(stderr, "More lines in file %s\n", name);
  fclose(f);
  return 0;
}

int micsa_read_lut(const char *name, double beta, void *lut, char *msg, size_t n) {
  FILE *f = fopen(name, "rb");
  if (!f) return err(msg, n, "Problems opening %s\n", name);
  double b = 0;
  if (fread(&b, sizeof b, 1, f) != 1) {
    fclose(f);
    return err(msg, n, "Problems reading betas\n");
  }
  if (fabs(beta - b) > 1e-14) {
    fclose(f);
    snprintf(msg, n, "betas[0]=%.14g from the beta file, betas[0]=%.14g from %s\n", beta, b, name);
    return -1;
  }
  if (fread(lut, 4096, 1, f) != 1) {
    fclose(f);
    return err(msg, n, "Problems reading lut_heat_bath\n");
  }
  fclose(f);
  return 0;
}

int micsa_read_times(const char *name, int ntimes, unsigned long long **times, char *msg,
                     size_t n) {
  *times = (unsigned long long *)malloc(sizeof(unsigned long long) * (ntimes > 0 ? ntimes : 1));
  if (!*times) return err(msg, n, "Problems allocating memory for list_times\n");
  FILE *f = fopen(name, "rt");
  if (!f) return err(msg, n, "File %s doesn't exist.\n", name);
  for (int i = 0; i < ntimes; i++)
    if (fscanf(f, "%llu ", &(*times)[i]) == EOF) {
      fclose(f);
      return err(msg, n, "File %s only has %d lines (it needs %d)\n", name, i, ntimes);
    }
  unsigned long long dummy;
  if (fscanf(f, "%llu", &dummy) != EOF) fprintf(stderr, "More lines in file %s\n", name);
  fclose(f);
  for (int i = 0; i + 1 < ntimes; i++)
    if ((*times)[i] >= (*times)[i + 1])
      return err(msg, n, "List of times must be sorted!\n");
  return 0;
}

int micsa_read_samples(const char *name, int nbits, int *list, char *msg, size_t n) {
  if (!name || !name[0]) {
    for (int i = 0; i < nbits; i++) list[i] = i;
  } else {
    FILE *f = fopen(name, "rt");
    if (!f) return err(msg, n, "File %s doesn't exist.\n", name);
    for (int i = 0; i < nbits; i++)
      if (fscanf(f, "%d ", &list[i]) == EOF) {
        fclose(f);
        return err(msg, n, "File %s only has %d lines (it needs %d)\n", name, i, nbits);
      }
    int dummy;
    if (fscanf(f, "%d", &dummy) != EOF) fprintf(stderr, "More lines in file %s\n", name);
    fclose(f);
  }
  for (int i = 0; i + 1 < nbits; i++)
    if (list[i] >= list[i + 1]) return err(msg, n, "List of samples must be sorted!\n");
  return 0;
}

static int64_t data_record_bytes(int nr) { return 40 + 8 * (2 + (int64_t)nr); }

int64_t micsa_conf_bytes(int L, int nr) {
  const int64_t V = (int64_t)L * L * L;
  return data_record_bytes(nr) + 8 + (int64_t)sizeof(micsa_prc_t) +
         (int64_t)sizeof(micsa_xoshiro_t) + 1 + V / 8 + 4;
}

int64_t micsa_walkers_bytes(int L, int nr, int nc) {
  const int64_t H = micsa_half_words(L);
  return 40 + (int64_t)nr * ((int64_t)sizeof(micsa_prc_t) + (int64_t)sizeof(micsa_xoshiro_t)) +
         4 * 8 * H * nr * nc;
}

int micsa_write_data_record(FILE *f, const micsa_data *d) {
  int32_t ints[6] = {d->ntimes, d->nterm, d->nc, d->nr, d->l, d->flag};
  uint64_t s2[2] = {d->seed_J, d->seed_u};
  int ok = fwrite(&d->maxtime, 8, 1, f) == 1 && fwrite(&d->now, 8, 1, f) == 1 &&
           fwrite(ints, 4, 6, f) == 6 && fwrite(s2, 8, 2, f) == 2 &&
           fwrite(d->seed_MC, 8, (size_t)d->nr, f) == (size_t)d->nr;
  return ok ? 0 : -1;
}

int micsa_read_data_record(FILE *f, micsa_data *d) {
  int32_t ints[6];
  uint64_t s2[2];
  int ok = fread(&d->maxtime, 8, 1, f) == 1 && fread(&d->now, 8, 1, f) == 1 &&
           fread(ints, 4, 6, f) == 6 && fread(s2, 8, 2, f) == 2;
  if (!ok) return -1;
  d->ntimes = ints[0]; d->nterm = ints[1]; d->nc = ints[2];
  d->nr = ints[3]; d->l = ints[4]; d->flag = ints[5];
  d->seed_J = s2[0];
  d->seed_u = s2[1];
  if (d->nr <= 0 || d->nr > 4096) return -1;
  d->seed_MC = (uint64_t *)calloc((size_t)d->nr, 8);
  if (!d->seed_MC) return -1;
  return fread(d->seed_MC, 8, (size_t)d->nr, f) == (size_t)d->nr ? 0 : -1;
}

void micsa_pack_bits(const uint8_t *u, int64_t n, uint8_t *out) {
  for (int64_t i = 0; i < n / 8; i++) {
    uint8_t b = 0;
    for (int j = 0; j < 8; j++) b |= (uint8_t)((u[8 * i + j] & 1) << j);
    out[i] = b;
  }
}

void micsa_unpack_bits(const uint8_t *in, int64_t n, uint8_t *u) {
  for (int64_t i = 0; i < n; i++) u[i] = (uint8_t)((in[i >> 3] >> (i & 7)) & 1);
}

int micsa_write_conf_record(FILE *f, const micsa_data *d, double beta,
                            const micsa_prc_t *prc, const micsa_xoshiro_t *xo,
                            const uint8_t *u, int L, int32_t energy) {
  const int64_t V = (int64_t)L * L * L;
  uint8_t *bits = (uint8_t *)malloc((size_t)(V / 8));
  if (!bits) return -1;
  micsa_pack_bits(u, V, bits);
  const uint8_t perm = 0;
  int ok = micsa_write_data_record(f, d) == 0 && fwrite(&beta, 8, 1, f) == 1 &&
           fwrite(prc, sizeof *prc, 1, f) == 1 && fwrite(xo, sizeof *xo, 1, f) == 1 &&
           fwrite(&perm, 1, 1, f) == 1 && fwrite(bits, 1, (size_t)(V / 8), f) == (size_t)(V / 8) &&
           fwrite(&energy, 4, 1, f) == 1;
  free(bits);
  return ok ? 0 : -1;
}

void micsa_measure_time(int L, int nr, int nbits, int nc, unsigned long long t) {
  static struct timespec ini = {0, 0}, cpu_ini;
  struct timespec fin, cpu_fin;
  clock_gettime(CLOCK_MONOTONIC, &fin);
  clock_gettime(CLOCK_PROCESS_CPUTIME_ID, &cpu_fin);
  if (ini.tv_sec > 0) {
    double elapsed = (fin.tv_sec - ini.tv_sec) * 1.e9 + (fin.tv_nsec - ini.tv_nsec);
    double consumed = (cpu_fin.tv_sec - cpu_ini.tv_sec) * 1.e9 + (cpu_fin.tv_nsec - cpu_ini.tv_nsec);
    double spins = (double)((int64_t)L * L * L * nr * nbits) * (double)nc * (double)t;
    printf("%4.0fs (%.3f ps/s, %.0f%%): ", elapsed * 1e-9, elapsed / spins * 1e3,
           consumed / elapsed * 100);
  }
  ini = fin;
  cpu_ini = cpu_fin;
}

int micsa_check_time(unsigned long long max_time, unsigned long long dt0,
                     unsigned long long dt1) {
  static struct timespec ini = {0, 0};
  static unsigned int total = 0;
  struct timespec fin;
  clock_gettime(CLOCK_MONOTONIC, &fin);
  if (ini.tv_sec > 0 && max_time != 0) {
    unsigned int elapsed = (unsigned int)(fin.tv_sec - ini.tv_sec);
    total += elapsed;
    unsigned int next = (unsigned int)(elapsed * (dt0 ? dt1 / dt0 : 0) * 1.1);
    if (((double)max_time) - total - next <= 0) return 1;
  }
  ini = fin;
  return 0;
}
