/*
 * micsa_run -- command-line drop-in for the reference program
 * bin/EA_CUBE_L<L>_NB1_NBPRE10 of IsidoroGlez/micSA-EA-MC
 * (PROGRAM/src/main.cu:10-195).
 *
 *   micsa_run isample nbits beta.dat input.in LUT list_times device
 *             [max_time [list_samples]]
 *
 * Same inputs, same output tree ({dir}I<isample>/BIT<s>/R<r>/), same
 * measurement, seed, checkpoint, lock and error files.  L and the replica
 * count come from input.in (the reference fixes them at compile time and
 * checks that input.in agrees).  The sweeps run on the GPU through libmicsa;
 * the demon refresh runs on host threads while the GPU sweeps, as in the
 * reference.  Differences from the reference are limited to: the output
 * directory is "{dir}I%03d/" as io.c:661 intends (the reference formats it
 * with overlapping sprintf buffers); changentimes.in is parsed as "count
 * then times" (io.c:930-968 reads through an uninitialised pointer).
 * Environment: MICSA_OBSERVABLES=1 also writes evol_q.txt, evol_C4.txt and
 * evol_xi.txt (correlation lengths xi12, xi23 from C4); MICSA_REFRESH=host
 * draws the demon refreshes on host threads (the reference's InitWalkers)
 * instead of the GPU; MICSA_HOST_THREADS=n sets the host threads used for
 * initialisation and host refreshes (default: all cores).  The library's own
 * variables are listed in micsa.h.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <math.h>
#include <pthread.h>
#include <signal.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include "micsa.h"
#include "micsa_host.h"
#include "micsa_io.h"

#define MAXNSAMPLES 2 /* header.h:20: fixes the spin and seed streams */
#define JANUS_SEED 9164166177945067407ULL /* io.c:797-799 */

/* ------------------------------------------------------------ run state */
static char dir[MICSA_MAXSTR], dirsample[MAXNSAMPLES][MICSA_MAXSTR];
static char my_host[100];
static int my_pid;
static micsa_data data;
static volatile sig_atomic_t got_signal = 0;
static int signals_deferred = 0;

static void delete_running(void) {
  char name[MICSA_MAXSTR + 16];
  snprintf(name, sizeof name, "%s/running", dir);
  remove(name);
}

/* create_error (io.c:996-1014) */
static void create_error(const char *fmt, ...) {
  char name[MICSA_MAXSTR + 16];
  snprintf(name, sizeof name, "%s/error", dir);
  FILE *f = fopen(name, "w");
  va_list ap;
  if (f) {
    va_start(ap, fmt);
    vfprintf(f, fmt, ap);
    va_end(ap);
    micsa_print_data(f, &data);
    fclose(f);
  }
  micsa_print_data(stderr, &data);
  delete_running();
}

static void die(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  exit(1);
}

/* handle_sigterm / ignore_sigterm / stop_run (io.c:970-994): the handler
 * only records the signal; it is acted on between iterations, and while
 * files are being written (the reference ignores signals then). */
static void on_signal(int s) { got_signal = s; }
static void handle_sigterm(void) {
  signals_deferred = 0;
  signal(SIGTERM, on_signal);
  signal(SIGINT, on_signal);
  signal(SIGUSR1, on_signal);
}
static void ignore_sigterm(void) { signals_deferred = 1; }
static void act_on_signal(void) {
  if (!got_signal || signals_deferred) return;
  const char *nm = got_signal == SIGTERM ? "SIGTERM" : got_signal == SIGINT ? "SIGINT" : "SIGUSR1";
  create_error("Received %s\n", nm);
  die("Aborting programma (SIGNAL=%d)\n", (int)got_signal);
}

static void writelog(FILE *f, time_t t) { fprintf(f, "%s %5d %10ld %s", my_host, my_pid, (long)t, ctime(&t)); }

/* create_running (io.c:1016-1047): hard-link lock */
static void create_running(void) {
  char name[MICSA_MAXSTR + 160], link_name[MICSA_MAXSTR + 16];
  gethostname(my_host, 99);
  my_pid = getpid();
  snprintf(name, sizeof name, "%srunning.%s.%d", dir, my_host, my_pid);
  snprintf(link_name, sizeof link_name, "%srunning", dir);
  FILE *f = fopen(name, "w");
  if (!f) die("Unable to open %s\n", name);
  writelog(f, time(NULL));
  fclose(f);
  if (link(name, link_name) == -1) {
    remove(name);
    die("%s exists\n", link_name);
  }
  remove(name);
  snprintf(name, sizeof name, "%srun.log", dir);
  if (!(f = fopen(name, "a"))) die("Unable to open %s\n", name);
  writelog(f, time(NULL));
  fclose(f);
}

/* ------------------------------------------------------- model state */
typedef struct {
  int L, nr, nc, nbits;
  int64_t V, H;
  int list_samples[MAXNSAMPLES];
  uint64_t seeds_J[MAXNSAMPLES];
  uint64_t *seeds_C;                 /* MAXNSAMPLES * nr */
  int countJ0[MAXNSAMPLES];
  micsa_prc_t random_u;
  micsa_prc_t *random_PRC;           /* nr Metropolis streams */
  micsa_xoshiro_t *random_xo;
  uint32_t *seed_keys;
  micsa_prc_t *random_PRC_C[MAXNSAMPLES];   /* demon streams */
  micsa_xoshiro_t *random_xo_C[MAXNSAMPLES];
  micsa_prc_t *write_PRC_C[MAXNSAMPLES];    /* snapshot at upload */
  micsa_xoshiro_t *write_xo_C[MAXNSAMPLES];
  uint8_t *uu;                       /* [nbits][nr][V] */
  uint8_t *Jx[MAXNSAMPLES], *Jy[MAXNSAMPLES], *Jz[MAXNSAMPLES];
  uint64_t *even[MAXNSAMPLES], *odd[MAXNSAMPLES], *J[MAXNSAMPLES];
  uint64_t *w0[MAXNSAMPLES], *w1[MAXNSAMPLES];         /* CPUwalker */
  uint64_t *ww0[MAXNSAMPLES], *ww1[MAXNSAMPLES];       /* write_CPUwalker */
  micsa_icds icds[MAXNSAMPLES];
  uint64_t thr[3];
  double beta;
  int32_t *e_spin;
  uint64_t *e_demon;
  int nthreads;
  int gpu_refresh; /* demon refresh on the GPU (default) or on host threads */
} model_t;

static model_t M;

static void *xmalloc(size_t n) {
  void *p = calloc(1, n ? n : 1);
  if (!p) die("Out of host memory (%zu bytes)\n", n);
  return p;
}

/* create_sample_path (io.c:657-677) */
static void create_sample_path(int sample) {
  char tmp[MICSA_MAXSTR];
  snprintf(tmp, sizeof tmp, "%sI%03d/", dir, sample);
  snprintf(dir, sizeof dir, "%s", tmp);
  mkdir(dir, 0775);
  for (int b = 0; b < M.nbits; b++) {
    snprintf(dirsample[b], MICSA_MAXSTR, "%sBIT%03d/", dir, M.list_samples[b]);
    mkdir(dirsample[b], 0775);
    for (int r = 0; r < M.nr; r++) {
      char rd[MICSA_MAXSTR + 8];
      snprintf(rd, sizeof rd, "%sR%02d/", dirsample[b], r);
      mkdir(rd, 0775);
    }
  }
  printf("Dirsample = %s\n", dir);
  fflush(stdout);
}

/* get_seeds (io.c:754-870); returns 1 when the seed files must be written */
static int get_seeds(void) {
  char name[MICSA_MAXSTR + 32];
  int no_seeds = 0;
  unsigned long long sJ = 0, su = 0;
  snprintf(name, sizeof name, "%s/master_seedJ.in", dir);
  FILE *f = fopen(name, "r");
  if (!f) {
    if (data.flag == 1) no_seeds++;
    else {
      sleep(1);
      if (!(f = fopen(name, "r"))) {
        create_error("There is not file %s, and it must exist\n", name);
        die("Problems reading seeds\n");
      }
    }
  }
  if (f) {
    if (fscanf(f, "%llu", &sJ) == EOF) die("Nothing in file %s\n", name);
    fclose(f);
    if (data.seed_J > 0 && data.seed_J != sJ) {
      create_error("Master seedJ in input file and %s differ\n", name);
      die("Problems reading master seedJ\n");
    }
    data.seed_J = sJ;
  }
  uint64_t tmp[MAXNSAMPLES];
  micsa_seeds_from_one(&data.seed_J, tmp, MAXNSAMPLES);
  for (int b = 0; b < M.nbits; b++) M.seeds_J[b] = JANUS_SEED; /* -DJANUS */
  memset(M.countJ0, 0, sizeof M.countJ0);
  unsigned long long *sMC = (unsigned long long *)xmalloc(sizeof(unsigned long long) * M.nr);
  for (int b = 0; b < M.nbits; b++) {
    snprintf(name, sizeof name, "%s/seeds.in", dirsample[b]);
    if (!(f = fopen(name, "r"))) {
      if (data.flag == 1) { no_seeds++; continue; }
      sleep(1);
      if (!(f = fopen(name, "r"))) {
        create_error("There is not file %s, and it must exist\n", name);
        die("Problems reading seeds\n");
      }
    }
    int nf = fscanf(f, "%llu %llu", &sJ, &su);
    for (int r = 0; r < M.nr; r++) nf += fscanf(f, " %llu", &sMC[r]);
    nf += fscanf(f, " %d", &M.countJ0[b]);
    fclose(f);
    if (nf != M.nr + 3) {
      create_error("File %s must have 7 fields\n", name);
      die("Problems reading seeds from %s\n", name);
    }
    if (M.seeds_J[b] != sJ) {
      create_error("Seed J generated and %s differ (bit=%d)\n", name, M.list_samples[b]);
      die("Problems reading seeds\n");
    }
    if (data.seed_u > 0 && data.seed_u != su) {
      create_error("Seed u in input and %s differ\n", name);
      die("Problems reading seeds\n");
    }
    data.seed_u = su;
    for (int r = 0; r < M.nr; r++) {
      if (data.seed_MC[r] > 0 && data.seed_MC[r] != sMC[r]) {
        create_error("Seed MC in input and %s differ\n", name);
        die("Problems reading seeds\n");
      }
      data.seed_MC[r] = sMC[r];
    }
  }
  free(sMC);
  if (no_seeds == M.nbits + 1) return 1;
  if (no_seeds > 0) die("Some samples have file seeds.in, others not have\n");
  return 0;
}

/* check_and_prepare_simulation_backup (io.c:689-752) */
static int check_and_prepare(void) {
  int there_is_conf = 0;
  for (int b = 0; b < M.nbits; b++) {
    there_is_conf = 0;
    for (int r = 0; r < M.nr; r++) {
      char name[MICSA_MAXSTR + 16];
      snprintf(name, sizeof name, "%sR%02d//conf", dirsample[b], r);
      FILE *f = fopen(name, "r");
      if (f) {
        there_is_conf++;
        fclose(f);
      }
    }
    if (there_is_conf > 0 && there_is_conf != M.nr) {
      create_error("There are less conf files than it must be in %s (%d/%d)\n", dirsample[b],
                   there_is_conf, M.nr);
      die("Problems with conf files\n");
    }
  }
  if (data.flag == 2) data.flag = there_is_conf ? 0 : 1;
  if (data.flag == 1) {
    if (there_is_conf) {
      create_error("There are some confs in %s.\nIf you want to make a new run, please delete the configuration manually\n", dir);
      die("There are confs\n");
    }
  } else if (data.flag == 0) {
    if (!there_is_conf) {
      create_error("There is no conf, it is impossible to do a backup\n");
      die("Impossible to do a backup\n");
    }
  } else {
    die("data.flag is not recognize\n");
  }
  return get_seeds();
}

/* write_seeds_in_file (io.c:872-911) */
static void write_seeds_in_file(void) {
  char name[MICSA_MAXSTR + 32];
  ignore_sigterm();
  snprintf(name, sizeof name, "%s/master_seedJ.in", dir);
  FILE *f = fopen(name, "w");
  if (!f) {
    create_error("Impossible to open seed file to write\n");
    die("Problems writing seeds\n");
  }
  fprintf(f, "%llu\n", (unsigned long long)data.seed_J);
  fclose(f);
  for (int b = 0; b < M.nbits; b++) {
    snprintf(name, sizeof name, "%s/seeds.in", dirsample[b]);
    if (!(f = fopen(name, "w"))) {
      create_error("Impossible to open seed file to write\n");
      die("Problems writing seeds\n");
    }
    fprintf(f, "%llu %llu", (unsigned long long)M.seeds_J[b], (unsigned long long)data.seed_u);
    for (int r = 0; r < M.nr; r++) fprintf(f, " %llu", (unsigned long long)data.seed_MC[r]);
    fprintf(f, " %d\n", M.countJ0[b]);
    fclose(f);
  }
  handle_sigterm();
}

/* Init (ini.c:8-32) minus the GPU tables */
static void init_model(void) {
  const int nr = M.nr, L = M.L;
  M.V = (int64_t)L * L * L;
  M.H = micsa_half_words(L);
  data.seed_u = micsa_check_seed(data.seed_u);
  for (int r = 0; r < nr; r++) data.seed_MC[r] = micsa_check_seed(data.seed_MC[r]);
  micsa_init_rand_hq(&M.random_u, data.seed_u);
  M.random_PRC = (micsa_prc_t *)xmalloc(sizeof(micsa_prc_t) * nr);
  M.random_xo = (micsa_xoshiro_t *)xmalloc(sizeof(micsa_xoshiro_t) * nr);
  M.seed_keys = (uint32_t *)xmalloc(4 * (size_t)nr);
  for (int r = 0; r < nr; r++)
    micsa_init_cpu_generators(&M.random_PRC[r], &M.random_xo[r], &M.seed_keys[r], data.seed_MC[r]);
  M.seeds_C = (uint64_t *)xmalloc(8 * (size_t)MAXNSAMPLES * nr);
  micsa_seeds_from_one(&data.seed_u, M.seeds_C, MAXNSAMPLES * nr);
  /* the samples' demon streams contiguous ([nbits][nr]): one GPU refresh
   * call covers all samples */
  micsa_prc_t *prc_all = (micsa_prc_t *)xmalloc(sizeof(micsa_prc_t) * nr * (M.nbits ? M.nbits : 1));
  micsa_xoshiro_t *xo_all =
      (micsa_xoshiro_t *)xmalloc(sizeof(micsa_xoshiro_t) * nr * (M.nbits ? M.nbits : 1));
  for (int b = 0; b < M.nbits; b++) {
    M.random_PRC_C[b] = prc_all + (int64_t)b * nr;
    M.random_xo_C[b] = xo_all + (int64_t)b * nr;
    M.write_PRC_C[b] = (micsa_prc_t *)xmalloc(sizeof(micsa_prc_t) * nr);
    M.write_xo_C[b] = (micsa_xoshiro_t *)xmalloc(sizeof(micsa_xoshiro_t) * nr);
    for (int r = 0; r < nr; r++) {
      uint32_t k;
      micsa_init_cpu_generators(&M.random_PRC_C[b][r], &M.random_xo_C[b][r], &k,
                                M.seeds_C[b * nr + r]);
    }
  }
  M.uu = (uint8_t *)xmalloc((size_t)M.nbits * nr * M.V);
  if (micsa_init_spins(&M.random_u, L, nr, MAXNSAMPLES, M.list_samples, M.nbits, M.uu))
    die("Problems generating spins\n");
  for (int b = 0; b < M.nbits; b++) {
    M.even[b] = (uint64_t *)xmalloc(8 * (size_t)(M.H * nr));
    M.odd[b] = (uint64_t *)xmalloc(8 * (size_t)(M.H * nr));
    micsa_pack_spins(L, nr, M.uu + (int64_t)b * nr * M.V, M.even[b], M.odd[b]);
  }
  printf("Packing spins well done.\n");
  printf("J random\n");
  for (int b = 0; b < M.nbits; b++) {
    M.Jx[b] = (uint8_t *)xmalloc((size_t)M.V);
    M.Jy[b] = (uint8_t *)xmalloc((size_t)M.V);
    M.Jz[b] = (uint8_t *)xmalloc((size_t)M.V);
    int count = micsa_init_couplings_janus(M.seeds_J[b], L, M.Jx[b], M.Jy[b], M.Jz[b]);
    if ((data.flag == 0 && count != M.countJ0[b]) || (M.countJ0[b] != 0 && M.countJ0[b] != count)) {
      create_error("countJ and countJ0 differ (%d != %d --- ibit=%d)\n", count, M.countJ0[b],
                   M.list_samples[b]);
      die("Problems generating J's\n");
    }
    M.countJ0[b] = count;
    M.J[b] = (uint64_t *)xmalloc(8 * (size_t)(12 * M.H));
    micsa_pack_couplings(L, M.Jx[b], M.Jy[b], M.Jz[b], M.J[b]);
    /* write_conf_Js (io.c:1147-1164) */
    char name[MICSA_MAXSTR + 16];
    snprintf(name, sizeof name, "%s/conf_Js", dirsample[b]);
    FILE *f = fopen(name, "w");
    if (!f) die("No pude abrir el fichero de configs. de Js.\n");
    uint8_t *bits = (uint8_t *)xmalloc((size_t)(M.V / 8));
    uint8_t *js[3] = {M.Jx[b], M.Jy[b], M.Jz[b]};
    for (int d = 0; d < 3; d++) {
      micsa_pack_bits(js[d], M.V, bits);
      fwrite(bits, 1, (size_t)(M.V / 8), f);
    }
    free(bits);
    fclose(f);
  }
  /* Init_threads_for_walkers (ini.c:624-676) */
  micsa_thresholds(M.beta, M.thr);
  for (int b = 0; b < M.nbits; b++) {
    M.icds[b] = (micsa_icds){1, (unsigned)b, (unsigned)nr, (unsigned)M.nc, (unsigned)L, 0,
                             M.seeds_C[M.list_samples[b]], M.beta};
    const size_t nw = (size_t)(2 * M.H * M.nc * nr);
    M.w0[b] = (uint64_t *)xmalloc(8 * nw);
    M.w1[b] = (uint64_t *)xmalloc(8 * nw);
    M.ww0[b] = (uint64_t *)xmalloc(8 * nw);
    M.ww1[b] = (uint64_t *)xmalloc(8 * nw);
  }
  M.e_spin = (int32_t *)xmalloc(4 * (size_t)M.nbits * nr);
  M.e_demon = (uint64_t *)xmalloc(8 * (size_t)M.nbits * nr);
}

/* ---------------------------------------------- checkpoint read/write */
static void read_conf(void) {
  const int64_t expect = micsa_conf_bytes(M.L, M.nr);
  uint8_t *bits = (uint8_t *)xmalloc((size_t)(M.V / 8));
  for (int b = 0; b < M.nbits; b++) {
    for (int r = 0; r < M.nr; r++) {
      char name[MICSA_MAXSTR + 16];
      snprintf(name, sizeof name, "%sR%02d//conf", dirsample[b], r);
      struct stat st;
      if (stat(name, &st) || st.st_size != expect) {
        create_error("There are only %lld bytes in %s (must be %lld)\n", (long long)st.st_size, name,
                     (long long)expect);
        die("Problems reading confs\n");
      }
      FILE *f = fopen(name, "rb");
      micsa_data dc;
      memset(&dc, 0, sizeof dc);
      double bc;
      uint8_t perm;
      int32_t ener;
      if (!f || micsa_read_data_record(f, &dc) || dc.nr != M.nr || (dc.l != data.l) ||
          dc.nc != data.nc || dc.nterm != data.nterm || dc.seed_J != M.seeds_J[b]) {
        create_error("Different data from input and %s\n", name);
        die("Problems reading confs\n");
      }
      data.now = dc.now;
      micsa_free_data(&dc);
      if (fread(&bc, 8, 1, f) != 1 || fabs(bc - M.beta) > 1e-12 ||
          fread(&M.random_PRC[r], sizeof(micsa_prc_t), 1, f) != 1 ||
          fread(&M.random_xo[r], sizeof(micsa_xoshiro_t), 1, f) != 1 || fread(&perm, 1, 1, f) != 1 ||
          perm != 0 || fread(bits, 1, (size_t)(M.V / 8), f) != (size_t)(M.V / 8) ||
          fread(&ener, 4, 1, f) != 1) {
        create_error("Problems reading conf in %s\n", name);
        die("Problems reading confs\n");
      }
      fclose(f);
      uint8_t *u = M.uu + ((int64_t)b * M.nr + r) * M.V;
      micsa_unpack_bits(bits, M.V, u);
      /* calculate_scalar_energy check (io.c:186-196) */
      int64_t e = 0;
      for (int z = 0; z < M.L; z++)
        for (int y = 0; y < M.L; y++)
          for (int x = 0; x < M.L; x++) {
            int64_t s = x + (int64_t)M.L * (y + (int64_t)M.L * z);
            int64_t sx = (x + 1) % M.L + (int64_t)M.L * (y + (int64_t)M.L * z);
            int64_t sy = x + (int64_t)M.L * ((y + 1) % M.L + (int64_t)M.L * z);
            int64_t sz = x + (int64_t)M.L * (y + (int64_t)M.L * ((z + 1) % M.L));
            e += (u[s] ^ M.Jx[b][s] ^ u[sx]) + (u[s] ^ M.Jy[b][s] ^ u[sy]) + (u[s] ^ M.Jz[b][s] ^ u[sz]);
          }
      int32_t es = (int32_t)(3 * M.V - 2 * e);
      if (es != ener) {
        create_error("Energy read and calculate differ in ibit=%d ir=%d ibeta=0:escalar=%d, read=%d\n",
                     b, r, es, ener);
        die("Problems reading confs\n");
      }
    }
    micsa_pack_spins(M.L, M.nr, M.uu + (int64_t)b * M.nr * M.V, M.even[b], M.odd[b]);
  }
  free(bits);
  printf("Packing spins well done.\n");
}

static void read_walkers(void) {
  const int64_t expect = micsa_walkers_bytes(M.L, M.nr, M.nc);
  const size_t nw = (size_t)(2 * M.H * M.nc * M.nr);
  for (int b = 0; b < M.nbits; b++) {
    char name[MICSA_MAXSTR + 16];
    snprintf(name, sizeof name, "%s/walkers", dirsample[b]);
    struct stat st;
    if (stat(name, &st) || st.st_size != expect) {
      create_error("There are only %lld bytes in %s (must be %lld)\n", (long long)st.st_size, name,
                   (long long)expect);
      die("Problems reading walkers\n");
    }
    FILE *f = fopen(name, "rb");
    micsa_icds c;
    if (!f || fread(&c, sizeof c, 1, f) != 1 || c.isample != M.icds[b].isample ||
        c.Nrep != M.icds[b].Nrep || c.NUM_WALKERS_PER_SITE != M.icds[b].NUM_WALKERS_PER_SITE ||
        c.Lv != M.icds[b].Lv || c.seed != M.icds[b].seed || fabs(c.beta - M.icds[b].beta) > 1e-6) {
      create_error("Different icds from simulation and %s\n", name);
      die("Problems reading walkers\n");
    }
    M.icds[b].first = c.first;
    if (fread(M.random_PRC_C[b], sizeof(micsa_prc_t), (size_t)M.nr, f) != (size_t)M.nr ||
        fread(M.random_xo_C[b], sizeof(micsa_xoshiro_t), (size_t)M.nr, f) != (size_t)M.nr ||
        fread(M.w0[b], 8, nw, f) != nw || fread(M.w1[b], 8, nw, f) != nw) {
      create_error("Problems reading walkers in %s\n", name);
      die("Problems reading walkers\n");
    }
    fclose(f);
  }
}

static void link_latest(const char *target, const char *link_name, int64_t expect) {
  remove(link_name);
  if (link(target, link_name)) {
    create_error("Problems in hard-lin to %s\n", target);
    die("Problems writing checkpoint\n");
  }
  struct stat st;
  stat(link_name, &st);
  if (st.st_nlink != 2) {
    create_error("The number of hard-link %s is not 2\n", link_name);
    die("Problems writing checkpoint\n");
  }
  if (st.st_size != expect) {
    create_error("There are only %lld bytes in %s (must be %lld)\n", (long long)st.st_size, link_name,
                 (long long)expect);
    die("Problems writing checkpoint\n");
  }
}

/* write_walkers (io.c:254-323) */
static void write_walkers(unsigned long long ib, unsigned long long prev) {
  const size_t nw = (size_t)(2 * M.H * M.nc * M.nr);
  for (int b = 0; b < M.nbits; b++) {
    char name[MICSA_MAXSTR + 40], ln[MICSA_MAXSTR + 16];
    snprintf(name, sizeof name, "%s/walkers.%016llu", dirsample[b], ib);
    FILE *f = fopen(name, "wb");
    if (!f || fwrite(&M.icds[b], sizeof(micsa_icds), 1, f) != 1 ||
        fwrite(M.write_PRC_C[b], sizeof(micsa_prc_t), (size_t)M.nr, f) != (size_t)M.nr ||
        fwrite(M.write_xo_C[b], sizeof(micsa_xoshiro_t), (size_t)M.nr, f) != (size_t)M.nr ||
        fwrite(M.ww0[b], 8, nw, f) != nw || fwrite(M.ww1[b], 8, nw, f) != nw) {
      create_error("Problems writing walkers in %s\n", name);
      die("Problems writing walkers\n");
    }
    fclose(f);
    snprintf(ln, sizeof ln, "%s/walkers", dirsample[b]);
    link_latest(name, ln, micsa_walkers_bytes(M.L, M.nr, M.nc));
    if (prev) {
      snprintf(name, sizeof name, "%s/walkers.%016llu", dirsample[b], prev);
      remove(name);
    }
  }
}

/* write_conf (io.c:17-96) */
static void write_conf(unsigned long long ib) {
  for (int b = 0; b < M.nbits; b++) {
    uint8_t *uu = M.uu + (int64_t)b * M.nr * M.V;
    micsa_unpack_spins(M.L, M.nr, M.even[b], M.odd[b], uu);
    data.seed_J = M.seeds_J[b];
    for (int r = 0; r < M.nr; r++) {
      char name[MICSA_MAXSTR + 48], ln[MICSA_MAXSTR + 16];
      snprintf(name, sizeof name, "%sR%02d//conf.%016llu", dirsample[b], r, ib);
      FILE *f = fopen(name, "wb");
      if (!f || micsa_write_conf_record(f, &data, M.beta, &M.random_PRC[r], &M.random_xo[r],
                                        uu + (int64_t)r * M.V, M.L, M.e_spin[b * M.nr + r])) {
        create_error("Problems writing conf in %s\n", name);
        die("Problems writing confs\n");
      }
      fclose(f);
      snprintf(ln, sizeof ln, "%sR%02d//conf", dirsample[b], r);
      link_latest(name, ln, micsa_conf_bytes(M.L, M.nr));
    }
  }
}

/* write_measures (io.c:395-462), plus the optional q / C4 files */
static void write_measures(unsigned long long ib, const int64_t *q, const int64_t *c4) {
  printf("Block = %d\n", (int)ib);
  double es[MAXNSAMPLES], ss[MAXNSAMPLES], ec[MAXNSAMPLES], sc[MAXNSAMPLES];
  for (int b = 0; b < M.nbits; b++) {
    micsa_energy_stats(M.e_spin + b * M.nr, M.nr, M.L, &es[b], &ss[b]);
    micsa_demon_stats(M.e_demon + b * M.nr, M.nr, M.L, M.nc, &ec[b], &sc[b]);
    printf("Sample = %d\n", M.list_samples[b]);
    double Bc = 0.25 * log(1. + 1. / ec[b]);
    printf("ibeta=%d: E_s=%10.8g E_c=%10.8g T_cl=%10.8g ", 0, es[b], ec[b], 1. / Bc);
    printf("\n");
  }
  fflush(stdout);
  for (int b = 0; b < M.nbits; b++) {
    char name[MICSA_MAXSTR + 32];
    const char *fn[3] = {"evol_E_spins.txt", "evol_E_walkers.txt", "evol_T_walkers.txt"};
    for (int k = 0; k < 3; k++) {
      snprintf(name, sizeof name, "%s%s", dirsample[b], fn[k]);
      FILE *f = fopen(name, "a");
      if (!f) {
        create_error("Problems opening %s\n", name);
        die("Problems writing measures\n");
      }
      fprintf(f, "%llu ", ib);
      if (k == 0) fprintf(f, "%14.10g %14.10g", es[b], ss[b]);
      if (k == 1) fprintf(f, "%14.10g %14.10g", ec[b], sc[b]);
      if (k == 2) fprintf(f, "%14.10g ", 1. / (0.25 * log(1. + 1. / ec[b])));
      fprintf(f, "\n");
      fclose(f);
    }
    if (q && c4) {
      const int np = M.nr / 2, nd = M.L / 2 + 1;
      snprintf(name, sizeof name, "%sevol_q.txt", dirsample[b]);
      FILE *f = fopen(name, "a");
      if (f) {
        fprintf(f, "%llu", ib);
        for (int k = 0; k < np; k++) fprintf(f, " %lld", (long long)q[b * np + k]);
        fprintf(f, "\n");
        fclose(f);
      }
      snprintf(name, sizeof name, "%sevol_C4.txt", dirsample[b]);
      if ((f = fopen(name, "a"))) {
        for (int d = 0; d < nd; d++) {
          /* pair- and axis-summed C4(d) */
          long long s = 0;
          for (int k = 0; k < np; k++)
            for (int a = 0; a < 3; a++) s += c4[(((int64_t)b * np + k) * 3 + a) * nd + d];
          fprintf(f, "%llu %d %lld\n", ib, d, s);
        }
        fclose(f);
      }
      snprintf(name, sizeof name, "%sevol_xi.txt", dirsample[b]);
      if ((f = fopen(name, "a"))) {
        double x12, x23;
        int rc;
        micsa_correlation_lengths(M.L, np, c4 + (int64_t)b * np * 3 * nd, MICSA_XI_KAPPA, 0, NULL,
                                  NULL, &x12, &x23, &rc);
        if (ftell(f) == 0)
          fprintf(f, "# t xi12 xi23 r_cut: integrals of C4(r) over r < r_cut, the first r >= 1 "
                     "where C4(r) < %g x its standard error over the %d replica pairs\n",
                  MICSA_XI_KAPPA, np);
        fprintf(f, "%llu %14.10g %14.10g %d\n", ib, x12, x23, rc);
        fclose(f);
      }
    }
  }
}

/* ---------------------------------------------------- demon refresh */
typedef struct {
  pthread_t tid;
  int running;
} refresher_t;
static refresher_t R;

static void *refresh_worker(void *arg) {
  (void)arg;
  for (int b = 0; b < M.nbits; b++) {
    M.icds[b].first = 0; /* InitWalkers, ini.c:739-741 */
    micsa_draw_demons_all(M.random_PRC_C[b], M.random_xo_C[b], M.thr, M.L, M.nr, M.nc, M.w0[b],
                          M.w1[b], M.nthreads);
  }
  return NULL;
}

/* refresh_walkers (main.cu:340-377) with the draws on the GPU.  As in the
 * reference, the next walkers are drawn while the GPU runs: there a host
 * thread, here a draw on a side stream (micsa_refresh_demons_ahead).  At a
 * refresh the walkers drawn ahead become current, the snapshot written with
 * the next checkpoint is the streams' state after them, and the next draw
 * starts.  A resumed run first uploads the walkers of its checkpoint. */
static void refresh_walkers_gpu(micsa_ctx *ctx, int *first) {
  int rc = 0;
  if (!(*first && data.flag)) {
    if (*first) {
      for (int b = 0; b < M.nbits && !rc; b++) rc = micsa_upload_demons(ctx, b, M.w0[b], M.w1[b]);
    } else {
      rc = micsa_refresh_commit(ctx);
    }
    if (!rc) rc = micsa_refresh_wait(ctx);
    if (rc) die("demon refresh: %s\n", micsa_last_error(ctx));
    for (int b = 0; b < M.nbits; b++) {
      memcpy(M.write_PRC_C[b], M.random_PRC_C[b], sizeof(micsa_prc_t) * M.nr);
      memcpy(M.write_xo_C[b], M.random_xo_C[b], sizeof(micsa_xoshiro_t) * M.nr);
    }
  }
  for (int b = 0; b < M.nbits; b++) M.icds[b].first = 0; /* InitWalkers, ini.c:739-741 */
  *first = 0;
  /* the next walkers, from the streams as they stand (InitWalkers thread) */
  if ((rc = micsa_refresh_demons_ahead(ctx, 0, M.nbits, M.random_PRC_C[0], M.random_xo_C[0], M.thr)))
    die("demon refresh: %s\n", micsa_last_error(ctx));
}

/* refresh_walkers (main.cu:340-377) */
static void refresh_walkers(micsa_ctx *ctx, int *first) {
  if (M.gpu_refresh) {
    refresh_walkers_gpu(ctx, first);
    return;
  }
  if (!(*first * data.flag)) {
    if (!*first && R.running) {
      pthread_join(R.tid, NULL);
      R.running = 0;
    }
    for (int b = 0; b < M.nbits; b++) {
      int rc = micsa_upload_demons(ctx, b, M.w0[b], M.w1[b]);
      if (rc) die("micsa_upload_demons: %s\n", micsa_last_error(ctx));
      memcpy(M.write_PRC_C[b], M.random_PRC_C[b], sizeof(micsa_prc_t) * M.nr);
      memcpy(M.write_xo_C[b], M.random_xo_C[b], sizeof(micsa_xoshiro_t) * M.nr);
    }
  }
  *first = 0;
  if (pthread_create(&R.tid, NULL, refresh_worker, NULL) != 0) {
    refresh_worker(NULL);
    R.running = 0;
  } else {
    R.running = 1;
  }
}

/* changentimes.in: "n t_1 ... t_n" replaces the measurement list */
static void stop_file(unsigned long long **list_times) {
  char name[MICSA_MAXSTR + 32];
  snprintf(name, sizeof name, "%schangentimes.in", dir);
  FILE *f = fopen(name, "rb");
  if (!f) return;
  int n = 0;
  if (fscanf(f, "%d", &n) != 1 || n <= 0) {
    fclose(f);
    remove(name);
    delete_running();
    printf(" File '%s' exists .\a\n", name);
    return;
  }
  unsigned long long *t = (unsigned long long *)xmalloc(sizeof(unsigned long long) * n);
  for (int i = 0; i < n; i++)
    if (fscanf(f, "%llu ", &t[i]) == EOF) die("File %s only has %d lines (it needs %d)\n", name, i, n);
  fclose(f);
  for (int i = 0; i + 1 < n; i++)
    if (t[i] >= t[i + 1]) {
      create_error("List of times %s is not sorted.\n", name);
      die("List of times must be sorted!\n");
    }
  free(*list_times);
  *list_times = t;
  data.ntimes = n;
}

static void print_help(const char *prog) {
  printf("Usage: %s isample ibit beta.dat input.in LUT list_times", prog);
  printf(" device [max_time [list_samples]]\n");
  printf("\nArguments:\n");
  printf("  isample              Sample index (int)\n");
  printf("  nbits                Number of subsample (int)\n");
  printf("  beta.dat             Path to beta.dat file (string)\n");
  printf("  input.in             Path to input.in file (string)\n");
  printf("  LUT                  Path to LUT file (string)\n");
  printf("  list_times           Path to the list_of_times file (string)\n");
  printf("  device               Device number (int)\n");
  printf("  max_time (opt.)      Maximum time allowed (unsigned long long)\n");
  printf("                       A 0 value disable this option.\n");
  printf("  list_samples (opt.)  Path to the list_of_samples file (string)\n");
  printf("\nUse -h to display this help message.\n");
  exit(EXIT_SUCCESS);
}

int main(int argc, char **argv) {
  if (argc > 1 && (!strcmp(argv[1], "-h") || !strcmp(argv[1], "--help"))) print_help(argv[0]);
  char name_list[MICSA_MAXSTR] = {0};
  int sample = 0, nbits = 0, device = 0;
  unsigned long long max_time = 0;
  if (argc < 8 || argc > 10)
    die("Usage: %s isample nbits beta.dat input.in LUT list_times device [max_time [list_samples]]\n",
        argv[0]);
  if (argc == 10) snprintf(name_list, sizeof name_list, "%s", argv[9]);
  if (argc >= 9) sscanf(argv[8], "%llu", &max_time);
  sscanf(argv[7], "%d", &device);
  sscanf(argv[2], "%d", &nbits);
  sscanf(argv[1], "%d", &sample);
  printf("count device = ?; device = %d\n", device);
  micsa_measure_time(8, 32, 1, 1, 0);
  micsa_check_time(max_time, 1, 0);
  if (nbits < 0 || nbits > MAXNSAMPLES) die("Error: nbits out of range, 0 < bit < %d\n", MAXNSAMPLES);
  if (sample < 0) die("Error: sample out of range, 0 <= sample\n");
  if (sample > (1 << 14) - 1) die("Our Counter-based PRNG  cannot accomodate more than %d samples\n", 1 << 14);
  const uint32_t jobid = (uint32_t)sample;

  char msg[2 * MICSA_MAXSTR];
  unsigned long long *list_times = NULL;
  uint8_t lut[4096];
  if (micsa_read_input(argv[4], dir, &data, msg, sizeof msg)) die("%s", msg);
  M.L = data.l & 0xffff;
  M.nr = data.nr;
  M.nc = data.nc;
  M.nbits = nbits;
  if (M.L < 8 || M.L % 8) die("l=%d must be a multiple of 8\n", M.L);
  if (M.nr % 32) die("d.nr = %d: this build needs a multiple of 32 replicas\n", M.nr);
  if (M.nc < 1 || M.nc > 6) die("nc=%d: the demon walk supports 1..6 demons per site\n", M.nc);
  printf("Path: %s\n", dir);
  micsa_print_data(stdout, &data);
  fflush(stdout);
  if (micsa_read_beta(argv[3], &M.beta, msg, sizeof msg)) die("%s", msg);
  if (micsa_read_lut(argv[5], M.beta, lut, msg, sizeof msg)) die("%s", msg);
  if (micsa_read_times(argv[6], data.ntimes, &list_times, msg, sizeof msg)) die("%s", msg);
  if (micsa_read_samples(name_list, nbits, M.list_samples, msg, sizeof msg)) die("%s", msg);
  {
    const char *nt = getenv("MICSA_HOST_THREADS");
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    M.nthreads = nt ? atoi(nt) : (int)(cores > 1 ? cores : 1);
    const char *where = getenv("MICSA_REFRESH");
    M.gpu_refresh = !(where && !strcmp(where, "host"));
  }
  create_sample_path(sample);
  int write_seeds = check_and_prepare();
  printf("Betas and LUT have been read correctly.\n");
  printf("Initializating J's and Spins ...\n");
  fflush(stdout);
  handle_sigterm();
  create_running();
  init_model();
  if (data.flag == 0) {
    read_conf();
    read_walkers();
    micsa_print_data(stdout, &data);
    if (data.now >= data.maxtime) {
      delete_running();
      create_error("There are %llu iterations in %s\n", data.now, dir);
      die("Problems in backup\n");
    }
  }
  if (write_seeds) write_seeds_in_file();
  stop_file(&list_times);

  micsa_config cfg = {device, M.L, M.nr, M.nbits, M.nc};
  micsa_ctx *ctx = NULL;
  int rc = micsa_create(&cfg, &ctx);
  if (rc) die("micsa_create failed (%d)\n", rc);
#define CHECK(call) do { if ((rc = (call))) die("%s: %s\n", #call, micsa_last_error(ctx)); } while (0)
  CHECK(micsa_set_lut(ctx, lut, sizeof lut));
  for (int b = 0; b < M.nbits; b++) {
    CHECK(micsa_upload_couplings(ctx, b, M.J[b]));
    CHECK(micsa_upload_spins(ctx, b, M.even[b], M.odd[b]));
  }

  /* thermalisation: Monte_Carlo flag = 0 (main.cu:126-128, 206-253) */
  uint32_t *te = (uint32_t *)xmalloc(4 * 8 * (size_t)M.nr);
  for (unsigned long long t = 0; t < (unsigned long long)data.nterm; t++) {
    micsa_fill_bits(M.random_PRC, M.random_xo, M.nr, 2 * t, 0, jobid, te);
    micsa_fill_bits(M.random_PRC, M.random_xo, M.nr, 2 * t + 1, 1, jobid, te + 4 * M.nr);
    CHECK(micsa_monte_carlo(ctx, 0, te, M.seed_keys));
    act_on_signal();
  }
  free(te);

  int first = 1;
  refresh_walkers(ctx, &first);
  unsigned long long iter = data.now;
  int i = 0;
  while (i < data.ntimes && data.now >= list_times[i]) i++;
  const int observables = getenv("MICSA_OBSERVABLES") && atoi(getenv("MICSA_OBSERVABLES"));
  int64_t *q = NULL, *c4 = NULL;
  if (observables) {
    q = (int64_t *)xmalloc(8 * (size_t)M.nbits * (M.nr / 2));
    c4 = (int64_t *)xmalloc(8 * (size_t)M.nbits * (M.nr / 2) * 3 * (M.L / 2 + 1));
  }
  while (iter < data.maxtime && i < data.ntimes) {
    if (!(iter & (iter - 1))) refresh_walkers(ctx, &first);
    /* run up to the next refresh, measurement or end in one graph replay */
    unsigned long long next = list_times[i];
    unsigned long long pow2 = 1;
    while (pow2 <= iter) pow2 <<= 1;
    if (pow2 < next) next = pow2;
    if (data.maxtime < next) next = data.maxtime;
    if (got_signal) next = iter + 1;
    CHECK(micsa_iterate(ctx, (int64_t)(next - iter)));
    CHECK(micsa_synchronize(ctx));
    iter = next;
    data.now = iter;
    act_on_signal();
    if (iter == list_times[i]) {
      micsa_measure_time(M.L, M.nr, M.nbits, M.nc, (i > 0) ? (iter - list_times[i - 1]) : iter);
      ignore_sigterm();
      for (int b = 0; b < M.nbits; b++) {
        CHECK(micsa_download_spins(ctx, b, M.even[b], M.odd[b]));
        CHECK(micsa_download_demons(ctx, b, M.ww0[b], M.ww1[b]));
      }
      CHECK(micsa_measure(ctx, M.e_spin, M.e_demon, q, c4));
      write_measures(iter, q, c4);
      write_walkers(data.now, (i > 0) ? list_times[i - 1] : 0);
      write_conf(data.now);
      stop_file(&list_times);
      handle_sigterm();
      act_on_signal();
      if (micsa_check_time(max_time, (i > 0) ? (iter - list_times[i - 1]) : iter,
                           ((i + 1) < data.ntimes) ? list_times[i + 1] - iter : 0) ||
          (++i) == data.ntimes)
        break;
    }
  }
  ignore_sigterm();
  if (R.running) pthread_join(R.tid, NULL);
  delete_running();
  printf("Simulation I=%d, nbits=%d finished at iteration %llu\n", sample, nbits, iter);
  fflush(stdout);
  micsa_destroy(ctx);
  free(list_times);
  free(q);
  free(c4);
  micsa_free_data(&data);
  return 0;
}
