/*
 * Serving: anneal requests arriving over time, continuously batched.
 *
 * Each request is a job (one reference run, micsa_job).  Requests of one
 * shape (L, nr, nc) share a pool: one context of S sample slots on its own
 * CUDA stream, driven by its own host thread; S is chosen so that every pool
 * fits the HBM budget.  A request is initialised on host threads once it is
 * submitted, then waits for a free slot.  A pool thread loops over rounds:
 * it admits waiting requests into free slots (upload of couplings and spins
 * into that slot, its generator streams copied in), refreshes the demons of
 * every slot whose own clock is at 0 or a power of two, runs the iterations
 * up to the nearest slot event (a power of two or a slot's last iteration,
 * at most `chunk`), measures when a slot needs it and frees the slots whose
 * job is done (frozen with micsa_set_active, refilled next round).  Every
 * slot follows its job's own schedule, so each result equals the job run
 * alone; slots of different ages share each launch.
 *
 * micsa_server_* / micsa_submit / micsa_poll expose this as a long-lived
 * server; micsa_serve replays a trace of timed requests through one.
 */
#include <errno.h>
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

/* ------------------------------------------------------------ records */

enum { REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED };

typedef struct {
  micsa_job job;
  int pool;
  int state, rc;
  prepared prep;
  int32_t *es;  /* [measurements][nr] */
  uint64_t *ed;
  int64_t nm;   /* measurements written */
  double t_submit, t_prepared, t_admitted, t_finished; /* absolute (monotonic) */
} request;

typedef struct fifo {
  int64_t *v;
  int64_t head, tail, cap;
} fifo;

static int fifo_push(fifo *q, int64_t x) {
  if (q->tail == q->cap) {
    if (q->head > 0) { /* compact */
      memmove(q->v, q->v + q->head, sizeof(int64_t) * (size_t)(q->tail - q->head));
      q->tail -= q->head;
      q->head = 0;
    } else {
      const int64_t nc = q->cap ? 2 * q->cap : 64;
      int64_t *nv = (int64_t *)realloc(q->v, sizeof(int64_t) * (size_t)nc);
      if (!nv) return MICSA_ERR_NOMEM;
      q->v = nv;
      q->cap = nc;
    }
  }
  q->v[q->tail++] = x;
  return MICSA_OK;
}

static int fifo_pop(fifo *q, int64_t *x) {
  if (q->head == q->tail) return 0;
  *x = q->v[q->head++];
  return 1;
}

struct micsa_server;

typedef struct {
  struct micsa_server *sv;
  int L, nr, nc, S;
  micsa_ctx *ctx;
  micsa_prc_t *prc; /* [S][nr] */
  micsa_xoshiro_t *xo;
  request **slot;    /* request in the slot, NULL = free (records stay put until polled) */
  int64_t *slot_t;   /* the slot's own iteration count */
  uint8_t *on;
  int32_t *es;
  uint64_t *ed;
  fifo queue; /* prepared requests, FIFO */
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int rc;
  char err[256];
  pthread_t thread;
  int started;
} pool;

struct micsa_server {
  micsa_server_config cfg;
  pool *pools;
  int npools;
  request **req; /* by id; NULL once released */
  int64_t nreq, capreq;
  fifo prepq;     /* submitted, to initialise */
  int64_t outstanding;
  int stop;
  pthread_mutex_t mu;
  pthread_cond_t cv;      /* prepq changed or stop */
  pthread_cond_t done_cv; /* a request finished or failed */
  pthread_t *prep;
  int nprep;
};

static void cond_init_monotonic(pthread_cond_t *c) {
  pthread_condattr_t a;
  pthread_condattr_init(&a);
  pthread_condattr_setclock(&a, CLOCK_MONOTONIC);
  pthread_cond_init(c, &a);
  pthread_condattr_destroy(&a);
}

/* under sv->mu: the request leaves the server's work (done or failed) */
static void finish_locked(micsa_server *sv, request *r, int rc) {
  r->state = rc ? REQ_FAILED : REQ_DONE;
  r->rc = rc;
  r->t_finished = now_s();
  release(&r->prep);
  sv->outstanding--;
  pthread_cond_broadcast(&sv->done_cv);
}

static void *prep_thread(void *arg) {
  micsa_server *sv = (micsa_server *)arg;
  for (;;) {
    pthread_mutex_lock(&sv->mu);
    int64_t id = -1;
    while (!fifo_pop(&sv->prepq, &id)) {
      if (sv->stop) break;
      pthread_cond_wait(&sv->cv, &sv->mu);
    }
    if (id < 0) { /* stopped with nothing left to initialise */
      pthread_mutex_unlock(&sv->mu);
      return NULL;
    }
    request *r = sv->req[id];
    pthread_mutex_unlock(&sv->mu);
    const int rc = prepare(&r->job, &r->prep);
    r->t_prepared = now_s();
    pool *pl = &sv->pools[r->pool];
    int prc = rc;
    pthread_mutex_lock(&pl->mu);
    if (!prc && !pl->rc) prc = fifo_push(&pl->queue, id);
    else if (!prc) prc = pl->rc;
    pthread_cond_signal(&pl->cv);
    pthread_mutex_unlock(&pl->mu);
    if (prc) {
      pthread_mutex_lock(&sv->mu);
      finish_locked(sv, r, prc);
      pthread_mutex_unlock(&sv->mu);
    }
  }
}

/* a pool that failed: its queued and running requests fail with it */
static void pool_fail(pool *pl, int rc) {
  micsa_server *sv = pl->sv;
  pthread_mutex_lock(&pl->mu);
  if (!pl->rc) pl->rc = rc;
  int64_t id;
  fifo drop = {0, 0, 0, 0};
  while (fifo_pop(&pl->queue, &id)) fifo_push(&drop, id);
  pthread_mutex_unlock(&pl->mu);
  pthread_mutex_lock(&sv->mu);
  while (fifo_pop(&drop, &id)) finish_locked(sv, sv->req[id], rc);
  for (int k = 0; k < pl->S; k++)
    if (pl->slot[k]) {
      finish_locked(sv, pl->slot[k], rc);
      pl->slot[k] = NULL;
    }
  pthread_mutex_unlock(&sv->mu);
  free(drop.v);
}

static void *pool_thread(void *arg) {
  pool *pl = (pool *)arg;
  micsa_server *sv = pl->sv;
  const int nr = pl->nr, S = pl->S;
  const int64_t chunk = sv->cfg.chunk > 0 ? sv->cfg.chunk : 1024;
  int rc = MICSA_OK;
#define CK(call)                                                                  \
  do {                                                                            \
    if ((rc = (call))) {                                                          \
      snprintf(pl->err, sizeof pl->err, "%s: %s", #call, micsa_last_error(pl->ctx)); \
      goto out;                                                                   \
    }                                                                             \
  } while (0)
  for (;;) {
    /* admissions into free slots */
    int changed = 0, nact = 0;
    for (int k = 0; k < S; k++) {
      if (pl->slot[k]) continue;
      int64_t id;
      pthread_mutex_lock(&pl->mu);
      const int got = fifo_pop(&pl->queue, &id);
      pthread_mutex_unlock(&pl->mu);
      if (!got) break;
      pthread_mutex_lock(&sv->mu);
      request *r = sv->req[id];
      r->state = REQ_RUNNING;
      pthread_mutex_unlock(&sv->mu);
      pl->slot[k] = r; /* from here a failure fails this request too */
      CK(micsa_refresh_wait(pl->ctx)); /* the slot's structs are rewritten below */
      CK(micsa_upload_couplings(pl->ctx, k, r->prep.J));
      CK(micsa_upload_spins(pl->ctx, k, r->prep.even, r->prep.odd));
      memcpy(pl->prc + (int64_t)k * nr, r->prep.prc, sizeof(micsa_prc_t) * nr);
      memcpy(pl->xo + (int64_t)k * nr, r->prep.xo, sizeof(micsa_xoshiro_t) * nr);
      release(&r->prep);
      pl->slot_t[k] = 0;
      pl->on[k] = 1;
      r->t_admitted = now_s();
      changed = 1;
    }
    for (int k = 0; k < S; k++) nact += pl->slot[k] != NULL;
    if (changed) CK(micsa_set_active(pl->ctx, pl->on));
    if (!nact) {
      pthread_mutex_lock(&pl->mu);
      while (pl->queue.head == pl->queue.tail && !sv->stop) pthread_cond_wait(&pl->cv, &pl->mu);
      const int quit = pl->queue.head == pl->queue.tail && sv->stop;
      pthread_mutex_unlock(&pl->mu);
      if (quit) break;
      continue;
    }
    /* refreshes due (refresh_walkers at t = 0 and powers of two), each slot
     * at its own job's beta at its own clock (pools mix betas) */
    for (int k = 0; k < S; k++)
      if (pl->slot[k] && (pl->slot_t[k] == 0 || is_pow2(pl->slot_t[k]))) {
        uint64_t tk[3];
        micsa_thresholds(micsa_job_beta(&pl->slot[k]->job, pl->slot_t[k]), tk);
        CK(micsa_refresh_demons_async(pl->ctx, k, 1, pl->prc + (int64_t)k * nr,
                                      pl->xo + (int64_t)k * nr, tk));
      }
    /* the round: up to the nearest slot event */
    int64_t R = chunk;
    for (int k = 0; k < S; k++) {
      if (!pl->slot[k]) continue;
      const int64_t t = pl->slot_t[k], it = pl->slot[k]->job.iterations;
      int64_t nxt = 1;
      while (nxt <= t) nxt <<= 1;
      if (nxt > it) nxt = it;
      if (nxt - t < R) R = nxt - t;
    }
    CK(micsa_iterate(pl->ctx, R));
    int need = 0;
    for (int k = 0; k < S; k++)
      if (pl->slot[k]) {
        pl->slot_t[k] += R;
        need |= is_pow2(pl->slot_t[k]) || pl->slot_t[k] == pl->slot[k]->job.iterations;
      }
    if (!need) {
      CK(micsa_synchronize(pl->ctx));
      continue;
    }
    CK(micsa_measure(pl->ctx, pl->es, pl->ed, NULL, NULL));
    changed = 0;
    for (int k = 0; k < S; k++) {
      request *r = pl->slot[k];
      if (!r) continue;
      const int64_t t = pl->slot_t[k], it = r->job.iterations;
      if (!(is_pow2(t) || t == it)) continue;
      memcpy(r->es + r->nm * nr, pl->es + (int64_t)k * nr, 4 * (size_t)nr);
      memcpy(r->ed + r->nm * nr, pl->ed + (int64_t)k * nr, 8 * (size_t)nr);
      r->nm++;
      if (t == it) {
        pl->slot[k] = NULL;
        pl->on[k] = 0;
        changed = 1;
        pthread_mutex_lock(&sv->mu);
        finish_locked(sv, r, MICSA_OK);
        pthread_mutex_unlock(&sv->mu);
      }
    }
    if (changed) CK(micsa_set_active(pl->ctx, pl->on));
  }
  CK(micsa_refresh_wait(pl->ctx));
  CK(micsa_synchronize(pl->ctx));
#undef CK
out:
  if (rc) pool_fail(pl, rc);
  return NULL;
}

static int find_pool(const micsa_server *sv, const micsa_job *jb) {
  for (int p = 0; p < sv->npools; p++)
    if (sv->pools[p].L == jb->L && sv->pools[p].nr == jb->nr && sv->pools[p].nc == jb->nc)
      return p;
  return -1;
}

int micsa_server_destroy(micsa_server *sv) {
  if (!sv) return MICSA_OK;
  pthread_mutex_lock(&sv->mu);
  while (sv->outstanding > 0) pthread_cond_wait(&sv->done_cv, &sv->mu);
  sv->stop = 1;
  pthread_cond_broadcast(&sv->cv);
  pthread_mutex_unlock(&sv->mu);
  for (int p = 0; p < sv->npools; p++) {
    pool *pl = &sv->pools[p];
    pthread_mutex_lock(&pl->mu);
    pthread_cond_broadcast(&pl->cv);
    pthread_mutex_unlock(&pl->mu);
  }
  for (int t = 0; t < sv->nprep; t++) pthread_join(sv->prep[t], NULL);
  for (int p = 0; p < sv->npools; p++) {
    pool *pl = &sv->pools[p];
    if (pl->started) pthread_join(pl->thread, NULL);
    micsa_destroy(pl->ctx);
    free(pl->prc), free(pl->xo), free(pl->slot), free(pl->slot_t);
    free(pl->on), free(pl->es), free(pl->ed), free(pl->queue.v);
    pthread_mutex_destroy(&pl->mu);
    pthread_cond_destroy(&pl->cv);
  }
  for (int64_t i = 0; i < sv->nreq; i++)
    if (sv->req[i]) {
      release(&sv->req[i]->prep);
      free(sv->req[i]->es), free(sv->req[i]->ed), free(sv->req[i]);
    }
  free(sv->req), free(sv->prepq.v), free(sv->pools), free(sv->prep);
  pthread_mutex_destroy(&sv->mu);
  pthread_cond_destroy(&sv->cv);
  pthread_cond_destroy(&sv->done_cv);
  free(sv);
  return MICSA_OK;
}

int micsa_server_create(const micsa_server_config *cfg, micsa_server **out, char *err,
                        size_t errlen) {
#define ERR(code, ...) do { if (err && errlen) snprintf(err, errlen, __VA_ARGS__); return (code); } while (0)
  if (!cfg || !out || !cfg->shapes || cfg->nshapes < 1)
    ERR(MICSA_ERR_ARG, "need a configuration with at least one shape");
  *out = NULL;
  for (int i = 0; i < cfg->nshapes; i++) {
    const micsa_pool_shape *sh = &cfg->shapes[i];
    micsa_config c = {cfg->device, sh->L, sh->nr, 1, sh->nc};
    if (micsa_footprint_bytes(&c) < 0 || sh->slots < 0)
      ERR(MICSA_ERR_ARG, "shape %d (L=%d nr=%d nc=%d): invalid", i, sh->L, sh->nr, sh->nc);
    for (int k = 0; k < i; k++)
      if (cfg->shapes[k].L == sh->L && cfg->shapes[k].nr == sh->nr && cfg->shapes[k].nc == sh->nc)
        ERR(MICSA_ERR_ARG, "shape %d repeats shape %d", i, k);
  }
  micsa_server *sv = (micsa_server *)calloc(1, sizeof(micsa_server));
  if (!sv) ERR(MICSA_ERR_NOMEM, "host memory");
  sv->cfg = *cfg;
  sv->cfg.shapes = NULL;
  pthread_mutex_init(&sv->mu, NULL);
  pthread_cond_init(&sv->cv, NULL);
  cond_init_monotonic(&sv->done_cv);
  sv->pools = (pool *)calloc((size_t)cfg->nshapes, sizeof(pool));
  long cores = sysconf(_SC_NPROCESSORS_ONLN);
  const int nprep = cfg->prep_threads > 0 ? cfg->prep_threads : (int)(cores > 2 ? cores - 1 : 1);
  sv->prep = (pthread_t *)calloc((size_t)nprep, sizeof(pthread_t));
  int rc = MICSA_OK;
  if (!sv->pools || !sv->prep) {
    micsa_server_destroy(sv);
    ERR(MICSA_ERR_NOMEM, "host memory");
  }
  const int64_t budget = cfg->hbm_budget > 0 ? cfg->hbm_budget : ((int64_t)48 << 30);
  const int smax = cfg->slots_max > 0 ? cfg->slots_max : 64;
  for (int p = 0; p < cfg->nshapes; p++) {
    pool *pl = &sv->pools[p];
    const micsa_pool_shape *sh = &cfg->shapes[p];
    pl->sv = sv;
    pl->L = sh->L, pl->nr = sh->nr, pl->nc = sh->nc;
    pthread_mutex_init(&pl->mu, NULL);
    pthread_cond_init(&pl->cv, NULL);
    sv->npools++;
    const int cap = sh->slots > 0 && sh->slots < smax ? sh->slots : smax;
    int S = 1;
    for (;;) {
      if (S >= cap) break;
      micsa_config c = {cfg->device, pl->L, pl->nr, S + 1, pl->nc};
      if (micsa_footprint_bytes(&c) * cfg->nshapes > budget) break;
      S++;
    }
    pl->S = S;
    pl->prc = (micsa_prc_t *)calloc((size_t)S * pl->nr, sizeof(micsa_prc_t));
    pl->xo = (micsa_xoshiro_t *)calloc((size_t)S * pl->nr, sizeof(micsa_xoshiro_t));
    pl->slot = (request **)calloc((size_t)S, sizeof(request *));
    pl->slot_t = (int64_t *)calloc((size_t)S, sizeof(int64_t));
    pl->on = (uint8_t *)calloc((size_t)S, 1);
    pl->es = (int32_t *)malloc(sizeof(int32_t) * (size_t)S * pl->nr);
    pl->ed = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)S * pl->nr);
    if (!pl->prc || !pl->xo || !pl->slot || !pl->slot_t || !pl->on || !pl->es || !pl->ed) {
      rc = MICSA_ERR_NOMEM;
      if (err && errlen) snprintf(err, errlen, "host memory");
      break;
    }
    /* contexts are created (and tuned) here, before any request: a warm server */
    micsa_config c = {cfg->device, pl->L, pl->nr, S, pl->nc};
    if ((rc = micsa_create(&c, &pl->ctx))) {
      if (err && errlen) snprintf(err, errlen, "micsa_create L=%d nr=%d S=%d failed", pl->L, pl->nr, S);
      break;
    }
    if ((rc = micsa_set_active(pl->ctx, pl->on))) {
      if (err && errlen) snprintf(err, errlen, "%s", micsa_last_error(pl->ctx));
      break;
    }
  }
  if (!rc) {
    for (int p = 0; p < sv->npools && !rc; p++) {
      if (pthread_create(&sv->pools[p].thread, NULL, pool_thread, &sv->pools[p])) {
        rc = MICSA_ERR_NOMEM;
        if (err && errlen) snprintf(err, errlen, "cannot start a pool thread");
      } else {
        sv->pools[p].started = 1;
      }
    }
    for (int t = 0; t < nprep && !rc; t++) {
      if (pthread_create(&sv->prep[t], NULL, prep_thread, sv)) {
        if (t == 0) {
          rc = MICSA_ERR_NOMEM;
          if (err && errlen) snprintf(err, errlen, "cannot start a host thread");
        }
        break;
      }
      sv->nprep++;
    }
  }
  if (rc) {
    micsa_server_destroy(sv);
    return rc;
  }
  *out = sv;
  return MICSA_OK;
#undef ERR
}

int micsa_submit(micsa_server *sv, const micsa_job *job, int64_t *id) {
  if (!sv || !job || !id) return MICSA_ERR_ARG;
  micsa_config c = {sv->cfg.device, job->L, job->nr, 1, job->nc};
  if (micsa_footprint_bytes(&c) < 0 || job->iterations < 1) return MICSA_ERR_ARG;
  const int p = find_pool(sv, job);
  if (p < 0) return MICSA_ERR_UNSUPPORTED;
  pthread_mutex_lock(&sv->pools[p].mu);
  const int prc = sv->pools[p].rc;
  pthread_mutex_unlock(&sv->pools[p].mu);
  if (prc) return prc;
  request *r = (request *)calloc(1, sizeof(request));
  const int64_t nm = micsa_job_measurements(job->iterations);
  if (!r) return MICSA_ERR_NOMEM;
  r->es = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nm * job->nr));
  r->ed = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nm * job->nr));
  if (!r->es || !r->ed) {
    free(r->es), free(r->ed), free(r);
    return MICSA_ERR_NOMEM;
  }
  r->job = *job;
  r->pool = p;
  r->state = REQ_QUEUED;
  r->t_submit = now_s();
  pthread_mutex_lock(&sv->mu);
  int rc = MICSA_OK;
  if (sv->stop) {
    rc = MICSA_ERR_STATE;
  } else if (sv->nreq == sv->capreq) {
    const int64_t nc = sv->capreq ? 2 * sv->capreq : 256;
    request **nv = (request **)realloc(sv->req, sizeof(request *) * (size_t)nc);
    if (!nv) rc = MICSA_ERR_NOMEM;
    else sv->req = nv, sv->capreq = nc;
  }
  if (!rc) rc = fifo_push(&sv->prepq, sv->nreq);
  if (rc) {
    pthread_mutex_unlock(&sv->mu);
    free(r->es), free(r->ed), free(r);
    return rc;
  }
  *id = sv->nreq;
  sv->req[sv->nreq++] = r;
  sv->outstanding++;
  pthread_cond_signal(&sv->cv);
  pthread_mutex_unlock(&sv->mu);
  return MICSA_OK;
}

int micsa_poll(micsa_server *sv, int64_t id, double timeout_s, int *done, int32_t *e_spin,
               uint64_t *e_demon, micsa_request_result *times) {
  if (!sv || !done) return MICSA_ERR_ARG;
  *done = 0;
  pthread_mutex_lock(&sv->mu);
  if (id < 0 || id >= sv->nreq || !sv->req[id]) {
    pthread_mutex_unlock(&sv->mu);
    return MICSA_ERR_ARG;
  }
  request *r = sv->req[id];
  if (timeout_s > 0 && r->state != REQ_DONE && r->state != REQ_FAILED) {
    struct timespec dl;
    clock_gettime(CLOCK_MONOTONIC, &dl);
    const double end = (double)dl.tv_sec + 1e-9 * (double)dl.tv_nsec + timeout_s;
    dl.tv_sec = (time_t)end;
    dl.tv_nsec = (long)((end - (double)(time_t)end) * 1e9);
    while (r->state != REQ_DONE && r->state != REQ_FAILED)
      if (pthread_cond_timedwait(&sv->done_cv, &sv->mu, &dl) == ETIMEDOUT) break;
  }
  int rc = MICSA_OK;
  if (r->state == REQ_DONE || r->state == REQ_FAILED) {
    sv->req[id] = NULL;
    pthread_mutex_unlock(&sv->mu);
    *done = 1;
    rc = r->state == REQ_FAILED ? r->rc : MICSA_OK;
    if (!rc) {
      const int64_t n = r->nm * r->job.nr;
      if (e_spin) memcpy(e_spin, r->es, sizeof(int32_t) * (size_t)n);
      if (e_demon) memcpy(e_demon, r->ed, sizeof(uint64_t) * (size_t)n);
    }
    if (times) {
      times->prepared = r->t_prepared > 0 ? r->t_prepared - r->t_submit : 0;
      times->admitted = r->t_admitted > 0 ? r->t_admitted - r->t_submit : 0;
      times->finished = r->t_finished - r->t_submit;
    }
    release(&r->prep);
    free(r->es), free(r->ed), free(r);
    return rc;
  }
  pthread_mutex_unlock(&sv->mu);
  return rc;
}

/* ------------------------------------------------------- trace replay */

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
  /* one pool per shape, with at most as many slots as the trace has requests of it */
  micsa_pool_shape *shapes = (micsa_pool_shape *)calloc((size_t)n, sizeof(micsa_pool_shape));
  int *order = (int *)malloc(sizeof(int) * (size_t)n);
  int64_t *ids = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  double *t_sub = (double *)malloc(sizeof(double) * (size_t)n);
  if (!shapes || !order || !ids || !t_sub) {
    free(shapes), free(order), free(ids), free(t_sub);
    ERR(MICSA_ERR_NOMEM, "host memory");
  }
  int nsh = 0;
  for (int j = 0; j < n; j++) {
    int p = 0;
    for (; p < nsh; p++)
      if (shapes[p].L == req[j].job.L && shapes[p].nr == req[j].job.nr && shapes[p].nc == req[j].job.nc)
        break;
    if (p == nsh) {
      shapes[nsh].L = req[j].job.L, shapes[nsh].nr = req[j].job.nr, shapes[nsh].nc = req[j].job.nc;
      nsh++;
    }
    shapes[p].slots++;
    order[j] = j;
    memset(&res[j], 0, sizeof res[j]);
  }
  for (int i = 1; i < n; i++) /* arrival order (stable) */
    for (int k = i; k > 0 && req[order[k]].arrival < req[order[k - 1]].arrival; k--) {
      const int t = order[k];
      order[k] = order[k - 1];
      order[k - 1] = t;
    }
  micsa_server_config sc = {cfg->device, cfg->hbm_budget, cfg->slots_max, cfg->chunk,
                            cfg->prep_threads, shapes, nsh};
  micsa_server *sv = NULL;
  int rc = micsa_server_create(&sc, &sv, err, errlen);
  if (!rc) {
    /* the clock starts with every context created and tuned */
    const double t0 = now_s();
    for (int k = 0; k < n && !rc; k++) {
      const int j = order[k];
      sleep_until(t0 + req[j].arrival); /* a server cannot start a request early */
      t_sub[j] = now_s() - t0;
      if ((rc = micsa_submit(sv, &req[j].job, &ids[j])) && err && errlen)
        snprintf(err, errlen, "request %d: submit failed (%d)", j, rc);
    }
    double last = 0;
    int64_t off = 0;
    for (int j = 0; j < n && !rc; j++) {
      int done = 0;
      micsa_request_result tm;
      while (!rc && !done)
        rc = micsa_poll(sv, ids[j], 60.0, &done, e_spin ? e_spin + off : NULL,
                        e_demon ? e_demon + off : NULL, &tm);
      if (rc) {
        if (err && errlen) snprintf(err, errlen, "request %d: %d", j, rc);
        break;
      }
      res[j].prepared = t_sub[j] + tm.prepared;
      res[j].admitted = t_sub[j] + tm.admitted;
      res[j].finished = t_sub[j] + tm.finished;
      if (res[j].finished > last) last = res[j].finished;
      off += micsa_job_measurements(req[j].job.iterations) * req[j].job.nr;
    }
    if (seconds) *seconds = last;
  }
  micsa_server_destroy(sv);
  free(shapes), free(order), free(ids), free(t_sub);
  return rc;
#undef ERR
}
