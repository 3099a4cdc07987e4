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
#include <stdint.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "micsa.h"
#include "micsa_host.h"

#define MAXNSAMPLES_REF 2 /* header.h:20, sizes the reference's seed fan-out */

double micsa_job_beta(const micsa_job *job, int64_t t) {
  if (job->beta_end == 0 || job->beta_end == job->beta || job->iterations < 1) return job->beta;
  return job->beta + (job->beta_end - job->beta) * (double)t / (double)job->iterations;
}

static int has_schedule(const micsa_job *j) { return j->beta_end != 0 && j->beta_end != j->beta; }

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
  int j0, j1, H, NR; /* per-job buffer strides: H words, NR streams */
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
    const int64_t V = (int64_t)L * L * L, H = a->H, NR = a->NR;
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
      micsa_init_cpu_generators(&a->prc[(int64_t)j * NR + r], &a->xo[(int64_t)j * NR + r], &key,
                                seeds[r]);
    }
    const int list[MAXNSAMPLES_REF + 1] = {0, 0, 0};
    if (micsa_init_spins(&random_u, L, nr, MAXNSAMPLES_REF, list, 1, uu)) a->rc = MICSA_ERR_ARG;
    micsa_pack_spins(L, nr, uu, a->even + (int64_t)j * H * NR, a->odd + (int64_t)j * H * NR);
    micsa_init_couplings_janus(jb->seed_J, L, jx, jx + V, jx + 2 * V);
    micsa_pack_couplings(L, jx, jx + V, jx + 2 * V, a->J + (int64_t)j * 12 * H);
    (void)nr;
    free(seeds), free(uu), free(jx);
  }
  return NULL;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int is_pow2(int64_t t) { return t > 0 && !(t & (t - 1)); }

/* One shape group (same L, nr, nc, beta) in its own context and stream:
 * jobs sorted by iterations, longest first, so the running jobs are always
 * the slots [0, nrun).  The context is created before any group runs (see
 * micsa_run_batch) and destroyed by the group. */
typedef struct {
  micsa_ctx *ctx;
  int device, n;
  const micsa_job *jobs; /* all jobs */
  int *idx;              /* this group's jobs, longest first */
  const int64_t *off;    /* output offsets of every job */
  int64_t SH, SNR;       /* strides of the per-job host buffers (words, streams) */
  uint64_t *J, *even, *odd;
  micsa_prc_t *prc;
  micsa_xoshiro_t *xo;
  int32_t *e_spin;
  uint64_t *e_demon;
  int rc;
  char err[256];
  /* run state */
  micsa_prc_t *gprc;     /* [n][nr] the slots' streams */
  micsa_xoshiro_t *gxo;
  int32_t *es;
  uint64_t *ed;
  uint8_t *on;
  int64_t *m;            /* measurements written per slot */
  int nrun;
  uint64_t thr[3];
} group_run;

#define GCK(gr, call)                                                                  \
  do {                                                                                 \
    int rc_ = (call);                                                                  \
    if (rc_) {                                                                         \
      snprintf((gr)->err, sizeof (gr)->err, "%s: %s", #call, micsa_last_error((gr)->ctx)); \
      return rc_;                                                                      \
    }                                                                                  \
  } while (0)

/* host buffers and the uploads of every slot (couplings, spins, streams) */
static int group_prepare(group_run *gr) {
  const micsa_job *j0 = &gr->jobs[gr->idx[0]];
  const int nr = j0->nr, n = gr->n;
  gr->gprc = (micsa_prc_t *)malloc(sizeof(micsa_prc_t) * nr * n);
  gr->gxo = (micsa_xoshiro_t *)malloc(sizeof(micsa_xoshiro_t) * nr * n);
  gr->es = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * nr);
  gr->ed = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n * nr);
  gr->on = (uint8_t *)malloc((size_t)n);
  gr->m = (int64_t *)calloc((size_t)n, sizeof(int64_t));
  if (!gr->gprc || !gr->gxo || !gr->es || !gr->ed || !gr->on || !gr->m) {
    snprintf(gr->err, sizeof gr->err, "host memory for a group of %d jobs", n);
    return MICSA_ERR_NOMEM;
  }
  for (int k = 0; k < n; k++) {
    const int j = gr->idx[k];
    memcpy(gr->gprc + (int64_t)k * nr, gr->prc + (int64_t)j * gr->SNR, sizeof(micsa_prc_t) * nr);
    memcpy(gr->gxo + (int64_t)k * nr, gr->xo + (int64_t)j * gr->SNR, sizeof(micsa_xoshiro_t) * nr);
    GCK(gr, micsa_upload_couplings(gr->ctx, k, gr->J + (int64_t)j * 12 * gr->SH));
    GCK(gr, micsa_upload_spins(gr->ctx, k, gr->even + (int64_t)j * gr->SH * gr->SNR,
                               gr->odd + (int64_t)j * gr->SH * gr->SNR));
    gr->on[k] = 1;
  }
  micsa_thresholds(j0->beta, gr->thr);
  gr->nrun = n;
  return MICSA_OK;
}

/* the demon refresh of the running slots at t = 0 or a power of two */
static int group_refresh(group_run *gr, int64_t t) {
  if (gr->nrun < 1 || (t & (t - 1))) return MICSA_OK;
  const micsa_job *j0 = &gr->jobs[gr->idx[0]];
  const int nr = j0->nr;
  micsa_ctx *ctx = gr->ctx;
  if (!has_schedule(j0)) {
    /* refresh t was drawn ahead (except at t = 0); draw the next one, for
     * the jobs that run past it, while the iterations up to it run (the
     * host advance of the streams overlaps them as well) */
    if (t == 0)
      GCK(gr, micsa_refresh_demons_async(ctx, 0, gr->nrun, gr->gprc, gr->gxo, gr->thr));
    else
      GCK(gr, micsa_refresh_commit(ctx));
    const int64_t tn = t ? 2 * t : 1;
    int nnext = 0;
    while (nnext < gr->nrun && gr->jobs[gr->idx[nnext]].iterations > tn) nnext++;
    if (nnext) GCK(gr, micsa_refresh_demons_ahead(ctx, 0, nnext, gr->gprc, gr->gxo, gr->thr));
  } else { /* each job at its own point of its beta schedule */
    for (int k = 0; k < gr->nrun; k++) {
      uint64_t tk[3];
      micsa_thresholds(micsa_job_beta(&gr->jobs[gr->idx[k]], t), tk);
      GCK(gr, micsa_refresh_demons_async(ctx, k, 1, gr->gprc + (int64_t)k * nr,
                                         gr->gxo + (int64_t)k * nr, tk));
    }
  }
  return MICSA_OK;
}

/* the group's next event after t: a power of two or its shortest running
 * job's end (INT64_MAX when nothing runs) */
static int64_t group_next(const group_run *gr, int64_t t) {
  if (gr->nrun < 1) return INT64_MAX;
  int64_t next = 1;
  while (next <= t) next <<= 1;
  const int64_t last = gr->jobs[gr->idx[gr->nrun - 1]].iterations; /* shortest running */
  return next > last ? last : next;
}

/* measurements at t of the slots that need one, and the freeze of the
 * slots whose job ended at t */
static int group_measure(group_run *gr, int64_t t) {
  if (gr->nrun < 1) return MICSA_OK;
  const int nr = gr->jobs[gr->idx[0]].nr;
  int any = 0;
  for (int k = 0; k < gr->nrun; k++) any |= is_pow2(t) || t == gr->jobs[gr->idx[k]].iterations;
  if (!any) return MICSA_OK;
  GCK(gr, micsa_measure(gr->ctx, gr->es, gr->ed, NULL, NULL));
  int still = gr->nrun;
  for (int k = 0; k < gr->nrun; k++) {
    const int j = gr->idx[k];
    const int64_t it = gr->jobs[j].iterations;
    if (!(is_pow2(t) || t == it)) continue;
    const int64_t o = gr->off[j] + gr->m[k]++ * nr;
    if (gr->e_spin) memcpy(gr->e_spin + o, gr->es + (int64_t)k * nr, 4 * (size_t)nr);
    if (gr->e_demon) memcpy(gr->e_demon + o, gr->ed + (int64_t)k * nr, 8 * (size_t)nr);
    if (t == it) {
      gr->on[k] = 0;
      still--;
    }
  }
  if (still != gr->nrun) {
    gr->nrun = still; /* finished jobs are the tail (longest first) */
    GCK(gr, micsa_set_active(gr->ctx, gr->on));
  }
  return MICSA_OK;
}

static int group_drain(group_run *gr) {
  GCK(gr, micsa_refresh_wait(gr->ctx));
  GCK(gr, micsa_synchronize(gr->ctx));
  return MICSA_OK;
}

static void group_free(group_run *gr) {
  micsa_destroy(gr->ctx);
  gr->ctx = NULL;
  free(gr->gprc), free(gr->gxo), free(gr->es), free(gr->ed), free(gr->on), free(gr->m);
  gr->gprc = NULL, gr->gxo = NULL, gr->es = NULL, gr->ed = NULL, gr->on = NULL, gr->m = NULL;
}
#undef GCK

/* a group on its own host thread and stream */
static void *run_group(void *arg) {
  group_run *gr = (group_run *)arg;
  int rc = group_prepare(gr);
  for (int64_t t = 0; !rc && gr->nrun > 0;) {
    if ((rc = group_refresh(gr, t))) break;
    const int64_t next = group_next(gr, t);
    if ((rc = micsa_iterate(gr->ctx, next - t))) {
      snprintf(gr->err, sizeof gr->err, "micsa_iterate: %s", micsa_last_error(gr->ctx));
      break;
    }
    t = next;
    rc = group_measure(gr, t);
  }
  if (!rc) rc = group_drain(gr);
  group_free(gr);
  gr->rc = rc;
  return NULL;
}

/* All groups in lockstep on one host thread: every group's refreshes and
 * measurements at the common event times, and the iterations between them
 * as mixed-lattice launches (one per iteration for all groups of one
 * replica count).  Each job's numbers are the same as in run_group. */
static int run_lockstep(group_run *grs, int ng, char *err, size_t errlen) {
  int rc = MICSA_OK;
  micsa_multi *multi[8] = {0};
  int nm = 0;
  /* one mixed launch per replica count, up to 16 groups each; created
   * before any upload, so that its launch shape is timed on empty buffers */
  {
    int used[64] = {0};
    if (ng > 64) {
      rc = MICSA_ERR_UNSUPPORTED;
      errf(err, errlen, "lockstep batches take at most 64 shape groups, got %d", ng);
      goto out;
    }
    for (int a = 0; a < ng; a++) {
      if (used[a]) continue;
      micsa_ctx *cs[16];
      int k = 0;
      for (int b = a; b < ng && k < 16; b++)
        if (!used[b] && grs[b].jobs[grs[b].idx[0]].nr == grs[a].jobs[grs[a].idx[0]].nr) {
          used[b] = 1;
          cs[k++] = grs[b].ctx;
        }
      if (nm == 8) {
        rc = MICSA_ERR_UNSUPPORTED;
        errf(err, errlen, "too many mixed launches");
        goto out;
      }
      if ((rc = micsa_multi_create(cs, k, &multi[nm], err, errlen))) goto out;
      nm++;
    }
  }
  for (int g = 0; g < ng && !rc; g++) rc = group_prepare(&grs[g]);
  if (rc) goto group_err;
  {
    int64_t t = 0;
    for (;;) {
      int64_t next = INT64_MAX;
      for (int g = 0; g < ng; g++) {
        if ((rc = group_refresh(&grs[g], t))) goto group_err;
        const int64_t n = group_next(&grs[g], t);
        if (n < next) next = n;
      }
      if (next == INT64_MAX) break;
      for (int k = 0; k < nm; k++)
        if ((rc = micsa_multi_iterate(multi[k], next - t))) {
          errf(err, errlen, "micsa_multi_iterate: %s", micsa_multi_last_error(multi[k]));
          goto out;
        }
      t = next;
      for (int g = 0; g < ng; g++)
        if ((rc = group_measure(&grs[g], t))) goto group_err;
    }
    for (int k = 0; k < nm; k++)
      if ((rc = micsa_multi_synchronize(multi[k]))) {
        errf(err, errlen, "micsa_multi_synchronize: %s", micsa_multi_last_error(multi[k]));
        goto out;
      }
    for (int g = 0; g < ng; g++)
      if ((rc = group_drain(&grs[g]))) goto group_err;
  }
  goto out;
group_err:
  for (int g = 0; g < ng; g++)
    if (grs[g].err[0]) {
      errf(err, errlen, "%s", grs[g].err);
      break;
    }
out:
  for (int k = 0; k < nm; k++) micsa_multi_destroy(multi[k]);
  for (int g = 0; g < ng; g++) group_free(&grs[g]);
  return rc;
}

/* MICSA_BATCH=multi: every shape group in lockstep through the
 * mixed-lattice launch; groups: each group on its own stream and host
 * thread (the default) */
static int batch_lockstep(void) {
  const char *e = getenv("MICSA_BATCH");
  return e && !strcmp(e, "multi");
}

static int same_group(const micsa_job *a, const micsa_job *b) {
  return a->L == b->L && a->nr == b->nr && a->nc == b->nc && a->beta == b->beta &&
         has_schedule(a) == has_schedule(b) && (!has_schedule(a) || a->beta_end == b->beta_end);
}

int micsa_run_batch(int device, const micsa_job *jobs, int njobs, int32_t *e_spin,
                    uint64_t *e_demon, double *seconds, char *err, size_t errlen) {
  if (!jobs || njobs < 1) return errf(err, errlen, "need at least one job"), MICSA_ERR_ARG;
  for (int j = 0; j < njobs; j++) {
    micsa_config c = {device, jobs[j].L, jobs[j].nr, 1, jobs[j].nc};
    if (micsa_footprint_bytes(&c) < 0 || jobs[j].iterations < 1)
      return errf(err, errlen, "job %d: invalid shape L=%d nr=%d nc=%d iterations=%lld", j,
                  jobs[j].L, jobs[j].nr, jobs[j].nc, (long long)jobs[j].iterations),
             MICSA_ERR_ARG;
  }
  /* output offsets; per-job host buffers are sized for the largest shape */
  int64_t *off = (int64_t *)malloc(sizeof(int64_t) * (size_t)njobs);
  int64_t maxH = 1, maxnr = 32;
  if (!off) return errf(err, errlen, "host memory"), MICSA_ERR_NOMEM;
  for (int j = 0, o = 0; j < njobs; j++) {
    off[j] = o;
    o += (int)(micsa_job_measurements(jobs[j].iterations) * jobs[j].nr);
    const int64_t H = micsa_half_words(jobs[j].L);
    if (H > maxH) maxH = H;
    if (jobs[j].nr > maxnr) maxnr = jobs[j].nr;
  }
  uint64_t *J = (uint64_t *)malloc(sizeof(uint64_t) * 12 * maxH * njobs);
  uint64_t *even = (uint64_t *)malloc(sizeof(uint64_t) * maxH * maxnr * njobs);
  uint64_t *odd = (uint64_t *)malloc(sizeof(uint64_t) * maxH * maxnr * njobs);
  micsa_prc_t *prc = (micsa_prc_t *)malloc(sizeof(micsa_prc_t) * maxnr * njobs);
  micsa_xoshiro_t *xo = (micsa_xoshiro_t *)malloc(sizeof(micsa_xoshiro_t) * maxnr * njobs);
  int *idx = (int *)malloc(sizeof(int) * (size_t)njobs);
  int *gstart = (int *)malloc(sizeof(int) * ((size_t)njobs + 1));
  group_run *grs = (group_run *)calloc((size_t)njobs, sizeof(group_run));
  pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)njobs);
  int *spawned = (int *)calloc((size_t)njobs, sizeof(int));
  int rc = MICSA_OK, ng = 0;
  if (!J || !even || !odd || !prc || !xo || !idx || !gstart || !grs || !tid || !spawned) {
    rc = MICSA_ERR_NOMEM;
    errf(err, errlen, "host memory for %d jobs", njobs);
    goto done;
  }
  /* host initialisation of every job, in parallel (job j's buffers at
   * stride maxH words / maxnr streams) */
  {
    enum { MAXT = 64 };
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    int nt = cores > 1 ? (int)cores : 1;
    if (nt > MAXT) nt = MAXT;
    if (nt > njobs) nt = njobs;
    init_share sh[MAXT];
    pthread_t it[MAXT];
    int sp[MAXT];
    for (int t = 0; t < nt; t++) {
      sh[t] = (init_share){jobs, njobs * t / nt, njobs * (t + 1) / nt, (int)maxH, (int)maxnr,
                           J, even, odd, prc, xo, MICSA_OK};
      sp[t] = t < nt - 1 && pthread_create(&it[t], NULL, init_jobs, &sh[t]) == 0;
      if (!sp[t]) init_jobs(&sh[t]);
    }
    for (int t = 0; t < nt; t++) {
      if (sp[t]) pthread_join(it[t], NULL);
      if (sh[t].rc) rc = sh[t].rc;
    }
    if (rc) {
      errf(err, errlen, "job initialisation failed");
      goto done;
    }
  }
  /* groups: stable grouping by shape, each sorted longest first */
  {
    int n = 0;
    char *used = (char *)calloc((size_t)njobs, 1);
    if (!used) {
      rc = MICSA_ERR_NOMEM;
      goto done;
    }
    for (int a = 0; a < njobs; a++) {
      if (used[a]) continue;
      gstart[ng++] = n;
      for (int b = a; b < njobs; b++)
        if (!used[b] && same_group(&jobs[a], &jobs[b])) {
          used[b] = 1;
          idx[n++] = b;
        }
    }
    gstart[ng] = n;
    free(used);
    for (int g = 0; g < ng; g++) /* insertion sort by iterations, descending */
      for (int i = gstart[g] + 1; i < gstart[g + 1]; i++)
        for (int k = i; k > gstart[g] && jobs[idx[k]].iterations > jobs[idx[k - 1]].iterations; k--) {
          const int tmp = idx[k];
          idx[k] = idx[k - 1];
          idx[k - 1] = tmp;
        }
  }
  {
    const double t0 = now_s();
    /* the contexts first, one after another: a shape's first context times
     * its launch shapes, which needs the GPU to itself (timed beside the
     * other groups' work, the choice would follow the noise) */
    for (int g = 0; g < ng; g++) {
      grs[g] = (group_run){NULL, device, gstart[g + 1] - gstart[g], jobs, idx + gstart[g], off,
                           maxH, maxnr, J, even, odd, prc, xo, e_spin, e_demon, MICSA_OK, {0}};
      const micsa_job *j0 = &jobs[idx[gstart[g]]];
      micsa_config cfg = {device, j0->L, j0->nr, grs[g].n, j0->nc};
      if ((grs[g].rc = micsa_create(&cfg, &grs[g].ctx)))
        snprintf(grs[g].err, sizeof grs[g].err, "micsa_create L=%d nr=%d n=%d failed (%d)", j0->L,
                 j0->nr, grs[g].n, grs[g].rc);
    }
    int created = 1;
    for (int g = 0; g < ng; g++)
      if (!grs[g].ctx) {
        created = 0;
        if (!rc) {
          rc = grs[g].rc;
          errf(err, errlen, "%s", grs[g].err);
        }
      }
    if (created && batch_lockstep()) {
      rc = run_lockstep(grs, ng, err, errlen);
    } else {
      for (int g = 0; g < ng; g++) {
        if (!grs[g].ctx) continue;
        spawned[g] = g < ng - 1 && pthread_create(&tid[g], NULL, run_group, &grs[g]) == 0;
        if (!spawned[g]) run_group(&grs[g]);
      }
      for (int g = 0; g < ng; g++) {
        if (spawned[g]) pthread_join(tid[g], NULL);
        if (grs[g].rc && !rc) {
          rc = grs[g].rc;
          errf(err, errlen, "%s", grs[g].err);
        }
      }
    }
    for (int g = 0; g < ng; g++)
      if (grs[g].ctx) group_free(&grs[g]); /* groups that never ran */
    if (seconds) *seconds = now_s() - t0;
  }
done:
  free(off), free(J), free(even), free(odd), free(prc), free(xo), free(idx), free(gstart);
  free(grs), free(tid), free(spawned);
  return rc;
}
