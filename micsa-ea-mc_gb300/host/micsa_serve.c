/*
 * Serving: anneal requests arriving over time, continuously batched.
 *
 * Each request is a job (one reference run, micsa_job).  Requests of one
 * shape (L, nr, nc) share a pool: one context of S sample slots on its
 * own CUDA stream, driven by its own host thread; S is chosen so that every
 * pool of the trace fits the HBM budget.  A request is initialised on host
 * threads once it has arrived, then waits for a free slot.  A pool thread
 * loops over rounds: it admits waiting requests into free slots (upload of
 * couplings and spins into that slot, its generator streams copied in),
 * refreshes the demons of every slot whose own clock is at 0 or a power of
 * two, runs the iterations up to the nearest slot event (a power of two or a
 * slot's last iteration, at most `chunk`), measures when a slot needs it and
 * frees the slots whose job is done (frozen with micsa_set_active, refilled
 * next round).  Every slot follows its job's own schedule, so each result
 * equals the job run alone; slots of different ages share each launch.
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

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void sleep_until(double t) {
  for (;;) {
    const double d = t - now_s();
    if (d <= 0) return;
    struct timespec ts = {(time_t)d, (long)((d - (double)(time_t)d) * 1e9)};
    nanosleep(&ts, NULL);
  }
}

static int is_pow2(int64_t t) { return t > 0 && !(t & (t - 1)); }

/* host state of one prepared request (Init, ini.c:8-32, as micsa_run_batch) */
typedef struct {
  uint64_t *J, *even, *odd;
  micsa_prc_t *prc;
  micsa_xoshiro_t *xo;
} prepared;

static int prepare(const micsa_job *jb, prepared *p) {
  const int L = jb->L, nr = jb->nr;
  const int64_t V = (int64_t)L * L * L, H = micsa_half_words(L);
  p->J = (uint64_t *)malloc(sizeof(uint64_t) * 12 * H);
  p->even = (uint64_t *)malloc(sizeof(uint64_t) * H * nr);
  p->odd = (uint64_t *)malloc(sizeof(uint64_t) * H * nr);
  p->prc = (micsa_prc_t *)malloc(sizeof(micsa_prc_t) * nr);
  p->xo = (micsa_xoshiro_t *)malloc(sizeof(micsa_xoshiro_t) * nr);
  uint64_t *seeds = (uint64_t *)malloc(sizeof(uint64_t) * MAXNSAMPLES_REF * nr);
  uint8_t *uu = (uint8_t *)malloc((size_t)(nr * V));
  uint8_t *jx = (uint8_t *)malloc((size_t)(3 * V));
  int rc = MICSA_OK;
  if (!p->J || !p->even || !p->odd || !p->prc || !p->xo || !seeds || !uu || !jx) {
    rc = MICSA_ERR_NOMEM;
  } else {
    uint64_t seed_u = micsa_check_seed(jb->seed_u);
    micsa_prc_t random_u;
    micsa_init_rand_hq(&random_u, seed_u);
    micsa_seeds_from_one(&seed_u, seeds, MAXNSAMPLES_REF * nr);
    for (int r = 0; r < nr; r++) {
      uint32_t key;
      micsa_init_cpu_generators(&p->prc[r], &p->xo[r], &key, seeds[r]);
    }
    const int list[MAXNSAMPLES_REF + 1] = {0, 0, 0};
    if (micsa_init_spins(&random_u, L, nr, MAXNSAMPLES_REF, list, 1, uu)) rc = MICSA_ERR_ARG;
    micsa_pack_spins(L, nr, uu, p->even, p->odd);
    micsa_init_couplings_janus(jb->seed_J, L, jx, jx + V, jx + 2 * V);
    micsa_pack_couplings(L, jx, jx + V, jx + 2 * V, p->J);
  }
  free(seeds), free(uu), free(jx);
  return rc;
}

static void release(prepared *p) {
  free(p->J), free(p->even), free(p->odd), free(p->prc), free(p->xo);
  memset(p, 0, sizeof *p);
}

struct server;

typedef struct {
  struct server *sv;
  int L, nr, nc, S;
  micsa_ctx *ctx;
  micsa_prc_t *prc; /* [S][nr] */
  micsa_xoshiro_t *xo;
  int *slot_req;    /* request in the slot, -1 = free */
  int64_t *slot_t;  /* the slot's own iteration count */
  int64_t *slot_m;  /* measurements written */
  uint8_t *on;
  int32_t *es;
  uint64_t *ed;
  int *queue, qhead, qtail; /* prepared requests, FIFO */
  int remaining;            /* requests of this pool not finished */
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int rc;
  char err[256];
} pool;

typedef struct server {
  const micsa_serve_config *cfg;
  const micsa_request *req;
  int n;
  micsa_request_result *res;
  int32_t *e_spin;
  uint64_t *e_demon;
  int64_t *off;
  int *pool_of;
  prepared *prep;
  pool *pools;
  int npools;
  double t0;
  int next_prep; /* next request to prepare (arrival order) */
  int *order;    /* requests sorted by arrival */
  pthread_mutex_t mu;
} server;

static void *prep_thread(void *arg) {
  server *sv = (server *)arg;
  for (;;) {
    pthread_mutex_lock(&sv->mu);
    const int k = sv->next_prep < sv->n ? sv->next_prep++ : -1;
    pthread_mutex_unlock(&sv->mu);
    if (k < 0) return NULL;
    const int j = sv->order[k];
    sleep_until(sv->t0 + sv->req[j].arrival); /* a server cannot start a request early */
    pool *pl = &sv->pools[sv->pool_of[j]];
    const int rc = prepare(&sv->req[j].job, &sv->prep[j]);
    sv->res[j].prepared = now_s() - sv->t0;
    pthread_mutex_lock(&pl->mu);
    if (rc) { /* the pool stops with this error */
      pl->rc = rc;
      snprintf(pl->err, sizeof pl->err, "request %d: host initialisation failed", j);
    } else {
      pl->queue[pl->qtail++] = j;
    }
    pthread_cond_signal(&pl->cv);
    pthread_mutex_unlock(&pl->mu);
  }
}

static void *pool_thread(void *arg) {
  pool *pl = (pool *)arg;
  server *sv = pl->sv;
  const int nr = pl->nr, S = pl->S;
  const int64_t chunk = sv->cfg->chunk > 0 ? sv->cfg->chunk : 1024;
  int rc = MICSA_OK;
#define CK(call)                                                                  \
  do {                                                                            \
    if ((rc = (call))) {                                                          \
      snprintf(pl->err, sizeof pl->err, "%s: %s", #call, micsa_last_error(pl->ctx)); \
      goto out;                                                                   \
    }                                                                             \
  } while (0)
  while (pl->remaining > 0 && !pl->rc) {
    /* admissions into free slots */
    int changed = 0, nact = 0;
    for (int k = 0; k < S; k++) {
      if (pl->slot_req[k] >= 0) continue;
      pthread_mutex_lock(&pl->mu);
      const int j = pl->qhead < pl->qtail ? pl->queue[pl->qhead++] : -1;
      pthread_mutex_unlock(&pl->mu);
      if (j < 0) break;
      prepared *p = &sv->prep[j];
      CK(micsa_refresh_wait(pl->ctx)); /* the slot's structs are rewritten below */
      CK(micsa_upload_couplings(pl->ctx, k, p->J));
      CK(micsa_upload_spins(pl->ctx, k, p->even, p->odd));
      memcpy(pl->prc + (int64_t)k * nr, p->prc, sizeof(micsa_prc_t) * nr);
      memcpy(pl->xo + (int64_t)k * nr, p->xo, sizeof(micsa_xoshiro_t) * nr);
      release(p);
      pl->slot_req[k] = j;
      pl->slot_t[k] = 0;
      pl->slot_m[k] = 0;
      pl->on[k] = 1;
      sv->res[j].admitted = now_s() - sv->t0;
      changed = 1;
    }
    for (int k = 0; k < S; k++) nact += pl->slot_req[k] >= 0;
    if (changed) CK(micsa_set_active(pl->ctx, pl->on));
    if (!nact) {
      pthread_mutex_lock(&pl->mu);
      if (pl->qhead == pl->qtail && pl->remaining > 0 && !pl->rc) pthread_cond_wait(&pl->cv, &pl->mu);
      pthread_mutex_unlock(&pl->mu);
      continue;
    }
    /* refreshes due (refresh_walkers at t = 0 and powers of two) */
    for (int k = 0; k < S; k++)
      if (pl->slot_req[k] >= 0 && (pl->slot_t[k] == 0 || is_pow2(pl->slot_t[k])))
      {
        /* the job's own beta at its own clock (pools mix betas) */
        uint64_t tk[3];
        micsa_thresholds(micsa_job_beta(&sv->req[pl->slot_req[k]].job, pl->slot_t[k]), tk);
        CK(micsa_refresh_demons_async(pl->ctx, k, 1, pl->prc + (int64_t)k * nr,
                                      pl->xo + (int64_t)k * nr, tk));
      }
    /* the round: up to the nearest slot event */
    int64_t R = chunk;
    for (int k = 0; k < S; k++) {
      if (pl->slot_req[k] < 0) continue;
      const int64_t t = pl->slot_t[k], it = sv->req[pl->slot_req[k]].job.iterations;
      int64_t nxt = 1;
      while (nxt <= t) nxt <<= 1;
      if (nxt > it) nxt = it;
      if (nxt - t < R) R = nxt - t;
    }
    CK(micsa_iterate(pl->ctx, R));
    int need = 0;
    for (int k = 0; k < S; k++)
      if (pl->slot_req[k] >= 0) {
        pl->slot_t[k] += R;
        need |= is_pow2(pl->slot_t[k]) || pl->slot_t[k] == sv->req[pl->slot_req[k]].job.iterations;
      }
    if (!need) {
      CK(micsa_synchronize(pl->ctx));
      continue;
    }
    CK(micsa_measure(pl->ctx, pl->es, pl->ed, NULL, NULL));
    const double tm = now_s() - sv->t0;
    changed = 0;
    for (int k = 0; k < S; k++) {
      const int j = pl->slot_req[k];
      if (j < 0) continue;
      const int64_t t = pl->slot_t[k], it = sv->req[j].job.iterations;
      if (!(is_pow2(t) || t == it)) continue;
      const int64_t o = sv->off[j] + pl->slot_m[k]++ * nr;
      if (sv->e_spin) memcpy(sv->e_spin + o, pl->es + (int64_t)k * nr, 4 * (size_t)nr);
      if (sv->e_demon) memcpy(sv->e_demon + o, pl->ed + (int64_t)k * nr, 8 * (size_t)nr);
      if (t == it) {
        sv->res[j].finished = tm;
        pl->slot_req[k] = -1;
        pl->on[k] = 0;
        changed = 1;
        pthread_mutex_lock(&pl->mu);
        pl->remaining--;
        pthread_mutex_unlock(&pl->mu);
      }
    }
    if (changed) CK(micsa_set_active(pl->ctx, pl->on));
  }
  CK(micsa_refresh_wait(pl->ctx));
  CK(micsa_synchronize(pl->ctx));
#undef CK
out:
  if (rc && !pl->rc) pl->rc = rc;
  return NULL;
}

static int same_shape(const micsa_job *a, const micsa_job *b) {
  return a->L == b->L && a->nr == b->nr && a->nc == b->nc;
}

int micsa_serve(const micsa_serve_config *cfg, const micsa_request *req, int n,
                micsa_request_result *res, int32_t *e_spin, uint64_t *e_demon, double *seconds,
                char *err, size_t errlen) {
#define ERR(code, ...) do { if (err && errlen) snprintf(err, errlen, __VA_ARGS__); return (code); } while (0)
  if (!cfg || !req || !res || n < 1) ERR(MICSA_ERR_ARG, "need a configuration and requests");
  for (int j = 0; j < n; j++) {
    micsa_config c = {cfg->device, req[j].job.L, req[j].job.nr, 1, req[j].job.nc};
    if (micsa_footprint_bytes(&c) < 0 || req[j].job.iterations < 1 || req[j].arrival < 0)
      ERR(MICSA_ERR_ARG, "request %d: invalid job or arrival time", j);
  }
  server sv;
  memset(&sv, 0, sizeof sv);
  sv.cfg = cfg, sv.req = req, sv.n = n, sv.res = res, sv.e_spin = e_spin, sv.e_demon = e_demon;
  sv.off = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  sv.pool_of = (int *)malloc(sizeof(int) * (size_t)n);
  sv.prep = (prepared *)calloc((size_t)n, sizeof(prepared));
  sv.pools = (pool *)calloc((size_t)n, sizeof(pool));
  sv.order = (int *)malloc(sizeof(int) * (size_t)n);
  pthread_mutex_init(&sv.mu, NULL);
  int rc = MICSA_OK;
  if (!sv.off || !sv.pool_of || !sv.prep || !sv.pools || !sv.order) {
    rc = MICSA_ERR_NOMEM;
    goto done;
  }
  {
    int64_t o = 0;
    for (int j = 0; j < n; j++) {
      sv.off[j] = o;
      o += micsa_job_measurements(req[j].job.iterations) * req[j].job.nr;
      memset(&res[j], 0, sizeof res[j]);
      sv.order[j] = j;
    }
    for (int i = 1; i < n; i++) /* arrival order (stable) */
      for (int k = i; k > 0 && req[sv.order[k]].arrival < req[sv.order[k - 1]].arrival; k--) {
        const int t = sv.order[k];
        sv.order[k] = sv.order[k - 1];
        sv.order[k - 1] = t;
      }
  }
  /* pools, one per shape; slots from the HBM budget */
  for (int j = 0; j < n; j++) {
    int p = 0;
    for (; p < sv.npools; p++) {
      const pool *pp = &sv.pools[p];
      const micsa_job shape = {pp->L, pp->nr, pp->nc, 0, 0, 0, 0, 0};
      if (same_shape(&req[j].job, &shape)) break;
    }
    if (p == sv.npools) {
      pool *pl = &sv.pools[sv.npools++];
      pl->sv = &sv;
      pl->L = req[j].job.L, pl->nr = req[j].job.nr, pl->nc = req[j].job.nc;
      pthread_mutex_init(&pl->mu, NULL);
      pthread_cond_init(&pl->cv, NULL);
    }
    sv.pool_of[j] = p;
    sv.pools[p].remaining++;
  }
  {
    const int64_t budget = cfg->hbm_budget > 0 ? cfg->hbm_budget : ((int64_t)48 << 30);
    const int smax = cfg->slots_max > 0 ? cfg->slots_max : 64;
    for (int p = 0; p < sv.npools && !rc; p++) {
      pool *pl = &sv.pools[p];
      int S = 1;
      for (;;) {
        if (S >= smax || S >= pl->remaining) break;
        micsa_config c = {cfg->device, pl->L, pl->nr, S + 1, pl->nc};
        if (micsa_footprint_bytes(&c) * sv.npools > budget) break;
        S++;
      }
      pl->S = S;
      micsa_config c = {cfg->device, pl->L, pl->nr, S, pl->nc};
      pl->prc = (micsa_prc_t *)calloc((size_t)S * pl->nr, sizeof(micsa_prc_t));
      pl->xo = (micsa_xoshiro_t *)calloc((size_t)S * pl->nr, sizeof(micsa_xoshiro_t));
      pl->slot_req = (int *)malloc(sizeof(int) * (size_t)S);
      pl->slot_t = (int64_t *)calloc((size_t)S, sizeof(int64_t));
      pl->slot_m = (int64_t *)calloc((size_t)S, sizeof(int64_t));
      pl->on = (uint8_t *)calloc((size_t)S, 1);
      pl->es = (int32_t *)malloc(sizeof(int32_t) * (size_t)S * pl->nr);
      pl->ed = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)S * pl->nr);
      pl->queue = (int *)malloc(sizeof(int) * (size_t)pl->remaining);
      if (!pl->prc || !pl->xo || !pl->slot_req || !pl->slot_t || !pl->slot_m || !pl->on ||
          !pl->es || !pl->ed || !pl->queue) {
        rc = MICSA_ERR_NOMEM;
        break;
      }
      for (int k = 0; k < S; k++) pl->slot_req[k] = -1;
      /* contexts are created (and tuned) before the clock starts: a warm server */
      if ((rc = micsa_create(&c, &pl->ctx))) {
        if (err && errlen) snprintf(err, errlen, "micsa_create L=%d nr=%d S=%d failed", pl->L, pl->nr, S);
        break;
      }
      if ((rc = micsa_set_active(pl->ctx, pl->on))) break;
    }
  }
  if (!rc) {
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    int nprep = cfg->prep_threads > 0 ? cfg->prep_threads : (int)(cores > 2 ? cores - 1 : 1);
    if (nprep > n) nprep = n;
    pthread_t *pt = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)(nprep + sv.npools));
    int *ok = (int *)calloc((size_t)(nprep + sv.npools), sizeof(int));
    if (!pt || !ok) {
      free(pt), free(ok);
      rc = MICSA_ERR_NOMEM;
      goto done;
    }
    sv.t0 = now_s();
    for (int p = 0; p < sv.npools; p++)
      ok[p] = pthread_create(&pt[p], NULL, pool_thread, &sv.pools[p]) == 0;
    for (int t = 0; t < nprep; t++)
      ok[sv.npools + t] = pthread_create(&pt[sv.npools + t], NULL, prep_thread, &sv) == 0;
    int started = 0;
    for (int t = 0; t < nprep; t++) started |= ok[sv.npools + t];
    if (!started) prep_thread(&sv);
    for (int t = 0; t < nprep; t++)
      if (ok[sv.npools + t]) pthread_join(pt[sv.npools + t], NULL);
    for (int p = 0; p < sv.npools; p++) {
      if (ok[p]) {
        pthread_join(pt[p], NULL);
      } else {
        pool_thread(&sv.pools[p]);
      }
    }
    double last = 0;
    for (int j = 0; j < n; j++)
      if (res[j].finished > last) last = res[j].finished;
    if (seconds) *seconds = last;
    free(pt), free(ok);
    for (int p = 0; p < sv.npools; p++)
      if (sv.pools[p].rc && !rc) {
        rc = sv.pools[p].rc;
        if (err && errlen) snprintf(err, errlen, "%s", sv.pools[p].err);
      }
  }
done:
  if (sv.pools)
    for (int p = 0; p < sv.npools; p++) {
      pool *pl = &sv.pools[p];
      micsa_destroy(pl->ctx);
      free(pl->prc), free(pl->xo), free(pl->slot_req), free(pl->slot_t), free(pl->slot_m);
      free(pl->on), free(pl->es), free(pl->ed), free(pl->queue);
      pthread_mutex_destroy(&pl->mu);
      pthread_cond_destroy(&pl->cv);
    }
  if (sv.prep)
    for (int j = 0; j < n; j++) release(&sv.prep[j]);
  free(sv.off), free(sv.pool_of), free(sv.prep), free(sv.pools), free(sv.order);
  pthread_mutex_destroy(&sv.mu);
  if (rc == MICSA_ERR_NOMEM && err && errlen && !err[0]) snprintf(err, errlen, "host memory");
  return rc;
#undef ERR
}
