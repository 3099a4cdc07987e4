/*
 * Batched runs: many independent reference runs of one shape in one
 * context.  A job is what one reference process computes for one sample
 * (nbits = 1, nterm = 0, flag 1): Init (ini.c:8-32) from the job's own seeds,
 * then the main loop (main.cu:130-180) with a demon refresh at t = 0 and at
 * every power of two and energy measurements at every power of two and at
 * the end.  The batch puts job j in sample slot j: one sweep launch, one
 * refresh launch and one measurement launch serve every job, and each job's
 * numbers equal those of the same job run alone.
 */
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "micsa.h"
#include "micsa_host.h"

#define MAXNSAMPLES_REF 2 /* header.h:20, sizes the reference's seed fan-out */

int64_t micsa_job_measurements(int64_t iterations) {
  if (iterations < 1) return 0;
  int64_t n = 0, p = 1;
  for (; p <= iterations; p <<= 1) n++;
  return n + ((iterations & (iterations - 1)) ? 1 : 0);
}

static void errf(char *err, size_t n, const char *fmt, ...) {
  if (!err || !n) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, n, fmt, ap);
  va_end(ap);
}

typedef struct {
  const micsa_job *jobs;
  int j0, j1, H;
  uint64_t *J, *even, *odd; /* [job][12H], [job][H nr] */
  micsa_prc_t *prc;         /* [job][nr] */
  micsa_xoshiro_t *xo;
  int rc;
} init_share;

/* Init (ini.c:8-32) for one sample of one job: spin stream and demon-stream
 * seeds from seed_u (Init_Random ini.c:34-60, generate_seeds_from_one),
 * spins (Init_u ini.c:275-299), couplings from the Janus generator seeded
 * with seed_J (Init_J ini.c:457-471; the reference's -DJANUS build uses one
 * fixed seed for every run, a batch gives each job its own). */
static void *init_jobs(void *arg) {
  init_share *a = (init_share *)arg;
  for (int j = a->j0; j < a->j1; j++) {
    const micsa_job *jb = &a->jobs[j];
    const int L = jb->L, nr = jb->nr;
    const int64_t V = (int64_t)L * L * L, H = a->H;
    uint64_t seed_u = micsa_check_seed(jb->seed_u);
    micsa_prc_t random_u;
    micsa_init_rand_hq(&random_u, seed_u);
    uint64_t *seeds = (uint64_t *)malloc(sizeof(uint64_t) * MAXNSAMPLES_REF * nr);
    uint8_t *uu = (uint8_t *)malloc((size_t)(nr * V));
    uint8_t *jx = (uint8_t *)malloc((size_t)(3 * V));
    if (!seeds || !uu || !jx) {
      a->rc = MICSA_ERR_NOMEM;
      free(seeds), free(uu), free(jx);
      return NULL;
    }
    micsa_seeds_from_one(&seed_u, seeds, MAXNSAMPLES_REF * nr);
    for (int r = 0; r < nr; r++) {
      uint32_t key;
      micsa_init_cpu_generators(&a->prc[(int64_t)j * nr + r], &a->xo[(int64_t)j * nr + r], &key,
                                seeds[r]);
    }
    const int list[MAXNSAMPLES_REF + 1] = {0, 0, 0};
    if (micsa_init_spins(&random_u, L, nr, MAXNSAMPLES_REF, list, 1, uu)) a->rc = MICSA_ERR_ARG;
    micsa_pack_spins(L, nr, uu, a->even + (int64_t)j * H * nr, a->odd + (int64_t)j * H * nr);
    micsa_init_couplings_janus(jb->seed_J, L, jx, jx + V, jx + 2 * V);
    micsa_pack_couplings(L, jx, jx + V, jx + 2 * V, a->J + (int64_t)j * 12 * H);
    free(seeds), free(uu), free(jx);
  }
  return NULL;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int micsa_run_batch(int device, const micsa_job *jobs, int njobs, int32_t *e_spin,
                    uint64_t *e_demon, double *seconds, char *err, size_t errlen) {
  if (!jobs || njobs < 1 || njobs > MICSA_MAX_SAMPLES)
    return errf(err, errlen, "need 1..%d jobs", MICSA_MAX_SAMPLES), MICSA_ERR_ARG;
  const micsa_job *j0 = &jobs[0];
  for (int j = 1; j < njobs; j++)
    if (jobs[j].L != j0->L || jobs[j].nr != j0->nr || jobs[j].nc != j0->nc ||
        jobs[j].iterations != j0->iterations || jobs[j].beta != j0->beta)
      return errf(err, errlen, "job %d: a batch runs one shape (L, nr, nc, iterations, beta)", j),
             MICSA_ERR_ARG;
  if (j0->iterations < 1) return errf(err, errlen, "iterations must be >= 1"), MICSA_ERR_ARG;
  micsa_config cfg = {device, j0->L, j0->nr, njobs, j0->nc};
  if (micsa_footprint_bytes(&cfg) < 0)
    return errf(err, errlen, "invalid shape L=%d nr=%d nc=%d", j0->L, j0->nr, j0->nc),
           MICSA_ERR_ARG;
  const int L = j0->L, nr = j0->nr;
  const int64_t H = micsa_half_words(L);

  /* host initialisation of every job, in parallel */
  uint64_t *J = (uint64_t *)malloc(sizeof(uint64_t) * 12 * H * njobs);
  uint64_t *even = (uint64_t *)malloc(sizeof(uint64_t) * H * nr * njobs);
  uint64_t *odd = (uint64_t *)malloc(sizeof(uint64_t) * H * nr * njobs);
  micsa_prc_t *prc = (micsa_prc_t *)malloc(sizeof(micsa_prc_t) * nr * njobs);
  micsa_xoshiro_t *xo = (micsa_xoshiro_t *)malloc(sizeof(micsa_xoshiro_t) * nr * njobs);
  int rc = MICSA_OK;
  micsa_ctx *ctx = NULL;
  if (!J || !even || !odd || !prc || !xo) {
    rc = MICSA_ERR_NOMEM;
    errf(err, errlen, "host memory for %d jobs", njobs);
    goto done;
  }
  {
    enum { MAXT = 64 };
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    int nt = cores > 1 ? (int)cores : 1;
    if (nt > MAXT) nt = MAXT;
    if (nt > njobs) nt = njobs;
    init_share sh[MAXT];
    pthread_t tid[MAXT];
    int spawned[MAXT];
    for (int t = 0; t < nt; t++) {
      sh[t] = (init_share){jobs, njobs * t / nt, njobs * (t + 1) / nt, (int)H, J, even, odd,
                           prc, xo, MICSA_OK};
      spawned[t] = t < nt - 1 && pthread_create(&tid[t], NULL, init_jobs, &sh[t]) == 0;
      if (!spawned[t]) init_jobs(&sh[t]);
    }
    for (int t = 0; t < nt; t++) {
      if (spawned[t]) pthread_join(tid[t], NULL);
      if (sh[t].rc) rc = sh[t].rc;
    }
    if (rc) {
      errf(err, errlen, "job initialisation failed");
      goto done;
    }
  }

  {
    const double t0 = now_s();
    if ((rc = micsa_create(&cfg, &ctx))) {
      errf(err, errlen, "micsa_create failed (%d)", rc);
      goto done;
    }
#define CK(call)                                                          \
  do {                                                                    \
    if ((rc = (call))) {                                                  \
      errf(err, errlen, "%s: %s", #call, micsa_last_error(ctx));          \
      goto done;                                                          \
    }                                                                     \
  } while (0)
    for (int j = 0; j < njobs; j++) {
      CK(micsa_upload_couplings(ctx, j, J + (int64_t)j * 12 * H));
      CK(micsa_upload_spins(ctx, j, even + (int64_t)j * H * nr, odd + (int64_t)j * H * nr));
    }
    uint64_t thr[3];
    micsa_thresholds(j0->beta, thr);
    const int64_t nm = micsa_job_measurements(j0->iterations);
    int32_t *es = (int32_t *)malloc(sizeof(int32_t) * (size_t)njobs * nr);
    uint64_t *ed = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)njobs * nr);
    if (!es || !ed) {
      free(es), free(ed);
      rc = MICSA_ERR_NOMEM;
      errf(err, errlen, "host memory for measurements");
      goto done;
    }
    int64_t t = 0, m = 0;
    while (t < j0->iterations) {
      /* the host advance of the streams overlaps the iterations that follow */
      if (!(t & (t - 1))) CK(micsa_refresh_demons_async(ctx, 0, njobs, prc, xo, thr));
      int64_t next = 1;
      while (next <= t) next <<= 1;
      if (next > j0->iterations) next = j0->iterations;
      CK(micsa_iterate(ctx, next - t));
      t = next;
      if (!(t & (t - 1)) || t == j0->iterations) {
        CK(micsa_measure(ctx, es, ed, NULL, NULL));
        for (int j = 0; j < njobs; j++) {
          if (e_spin) memcpy(e_spin + ((int64_t)j * nm + m) * nr, es + (int64_t)j * nr, 4 * (size_t)nr);
          if (e_demon) memcpy(e_demon + ((int64_t)j * nm + m) * nr, ed + (int64_t)j * nr, 8 * (size_t)nr);
        }
        m++;
      }
    }
    free(es), free(ed);
    CK(micsa_synchronize(ctx));
    if (seconds) *seconds = now_s() - t0;
#undef CK
  }
done:
  micsa_destroy(ctx);
  free(J), free(even), free(odd), free(prc), free(xo);
  return rc;
}
