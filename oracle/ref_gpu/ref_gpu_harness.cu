/*
 * ref_gpu_harness.cu -- TEST INFRASTRUCTURE ONLY (oracle).
 *
 * Runs the reference's own CUDA kernels on the GPU host.  The kernels come
 * from a cubin compiled from the unmodified PROGRAM/src/main.cu
 * (build_ref_gpu.sh); this file is only the host side that the reference's
 * main.cu would otherwise provide: it rebuilds the device data structures of
 * CopyDataOnDevice (main.cu:404-471) -- per sample two spin rows, twelve
 * coupling rows, twelve neighbour rows, two walker rows of each demon bit,
 * the colour rotate tables, all reached through pointer tables as mmcuda
 * (main.cu:1219-1289) lays them out -- and launches
 * d_oneMCstepBN_multisample and d_Walk exactly as Monte_Carlo with flag = 1
 * does (main.cu:254-305), with calculate_blocks' launch geometry
 * (ini.c:580-602).  Nothing in the product links or calls it.
 *
 * Host layouts (the reference's): spins even/odd[h*nr + r], couplings
 * J[(p*6 + d)*H + h], demons w[((p*nc + ic)*H + h)*nr + r], neighbour table
 * neig[(p*6 + d)*H + h] (other-colour word of the d-neighbour) and rotate
 * bytes rot[p*H + h] as oracle_tables gives them.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

namespace {

struct rg_ctx {
  CUmodule mod = nullptr;
  CUfunction sweep = nullptr, walk = nullptr;
  int L = 0, nr = 0, ns = 0, nc = 0;
  int64_t H = 0;
  int tpb = 0, nblocks = 0;
  std::vector<void *> allocs;
  /* rows */
  std::vector<uint64_t *> spin, J, w0, w1; /* [s][2], [s][12], [s][2], [s][2] */
  std::vector<int *> neig;                 /* [12], shared by the samples */
  unsigned char *rot[2] = {nullptr, nullptr};
  /* pointer tables as the kernels take them */
  void *spinAll = nullptr, *JAll = nullptr, *neigAll = nullptr, *w0All = nullptr,
       *w1All = nullptr, *whichAll = nullptr;
  cudaStream_t stream = nullptr;
  char err[512] = {0};
};

int fail(rg_ctx *c, const char *what, const char *msg) {
  if (c) snprintf(c->err, sizeof c->err, "%s: %s", what, msg);
  return 1;
}
#define RT(call)                                                         \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) return fail(c, #call, cudaGetErrorString(e_)); \
  } while (0)
#define DRV(call)                                       \
  do {                                                  \
    CUresult r_ = (call);                               \
    if (r_ != CUDA_SUCCESS) {                           \
      const char *s_ = "?";                             \
      cuGetErrorString(r_, &s_);                        \
      return fail(c, #call, s_);                        \
    }                                                   \
  } while (0)

template <class T>
int dev_alloc(rg_ctx *c, T **p, size_t n) {
  void *v = nullptr;
  RT(cudaMalloc(&v, n * sizeof(T)));
  RT(cudaMemset(v, 0, n * sizeof(T)));
  c->allocs.push_back(v);
  *p = (T *)v;
  return 0;
}

/* a device copy of a host array of device pointers */
template <class T>
int dev_table(rg_ctx *c, void **out, const std::vector<T> &host) {
  T *d = nullptr;
  if (dev_alloc(c, &d, host.size())) return 1;
  RT(cudaMemcpy(d, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = d;
  return 0;
}

}  // namespace

extern "C" {

const char *rg_error(void *h) { return h ? ((rg_ctx *)h)->err : "null handle"; }

/* Load the cubin and lay out the reference's device structures for ns
 * samples of an L^3 lattice, nr replicas, nc demons per site.  neig and rot
 * are the tables above (shared by every sample, as the geometry is). */
int rg_create(const char *cubin, int L, int nr, int ns, int nc, const int32_t *neig,
              const uint8_t *rot, void **out, char *err, size_t errlen) {
  *out = nullptr;
  rg_ctx *c = new rg_ctx;
  auto bail = [&](int rc) {
    if (err && errlen) snprintf(err, errlen, "%s", c->err);
    for (void *p : c->allocs) cudaFree(p);
    if (c->mod) cuModuleUnload(c->mod);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return rc;
  };
  c->L = L, c->nr = nr, c->ns = ns, c->nc = nc;
  const int64_t m = L / 4;
  c->H = m * m * m / 2;
  if (cudaSetDevice(0) != cudaSuccess || cudaFree(0) != cudaSuccess)
    return fail(c, "cudaSetDevice", "no device"), bail(1);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(c, "cudaStreamCreate", "failed"), bail(1);
  {
    CUresult r = cuModuleLoad(&c->mod, cubin);
    if (r != CUDA_SUCCESS) {
      const char *s = "?";
      cuGetErrorString(r, &s);
      return fail(c, "cuModuleLoad", s), bail(1);
    }
    unsigned nf = 0;
    if (cuModuleGetFunctionCount(&nf, c->mod) != CUDA_SUCCESS || !nf)
      return fail(c, "cuModuleGetFunctionCount", "no kernels"), bail(1);
    std::vector<CUfunction> fs(nf);
    if (cuModuleEnumerateFunctions(fs.data(), nf, c->mod) != CUDA_SUCCESS)
      return fail(c, "cuModuleEnumerateFunctions", "failed"), bail(1);
    for (CUfunction f : fs) {
      const char *name = nullptr;
      if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
      if (strstr(name, "d_oneMCstepBN_multisample")) c->sweep = f;
      if (strstr(name, "d_Walk")) c->walk = f;
    }
    if (!c->sweep || !c->walk) return fail(c, "cubin", "sweep or walk kernel not found"), bail(1);
  }
  /* calculate_blocks (ini.c:580-602), NBETAS = 1 */
  const int64_t hvnr = c->H * nr;
  int64_t t = hvnr;
  while (t > 512 || t % 32) t /= 2;
  if (t == 0) t = 32;
  c->tpb = (int)t;
  c->nblocks = (int)((hvnr + t - 1) / t);

  const int64_t H = c->H, wrow = H * nr * nc;
  std::vector<void *> spin_tabs, J_tabs, w0_tabs, w1_tabs, which_tabs, neig_tabs;
  c->neig.resize(12);
  for (int k = 0; k < 12; k++) {
    if (dev_alloc(c, &c->neig[k], (size_t)H)) return bail(1);
    if (cudaMemcpy(c->neig[k], neig + k * H, H * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(c, "neig", "copy"), bail(1);
  }
  for (int p = 0; p < 2; p++) {
    if (dev_alloc(c, &c->rot[p], (size_t)H)) return bail(1);
    if (cudaMemcpy(c->rot[p], rot + p * H, H, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(c, "rotate", "copy"), bail(1);
  }
  void *neig_rows = nullptr;
  if (dev_table(c, &neig_rows, std::vector<int *>(c->neig))) return bail(1);
  for (int s = 0; s < ns; s++) {
    std::vector<uint64_t *> sp(2), jr(12), a(2), b(2);
    for (int p = 0; p < 2; p++) {
      if (dev_alloc(c, &sp[p], (size_t)(H * nr)) || dev_alloc(c, &a[p], (size_t)wrow) ||
          dev_alloc(c, &b[p], (size_t)wrow))
        return bail(1);
    }
    for (int k = 0; k < 12; k++)
      if (dev_alloc(c, &jr[k], (size_t)H)) return bail(1);
    unsigned *wc = nullptr;
    if (dev_alloc(c, &wc, (size_t)nr)) return bail(1);
    c->spin.insert(c->spin.end(), sp.begin(), sp.end());
    c->J.insert(c->J.end(), jr.begin(), jr.end());
    c->w0.insert(c->w0.end(), a.begin(), a.end());
    c->w1.insert(c->w1.end(), b.begin(), b.end());
    void *ts = nullptr, *tj = nullptr, *ta = nullptr, *tb = nullptr;
    if (dev_table(c, &ts, sp) || dev_table(c, &tj, jr) || dev_table(c, &ta, a) ||
        dev_table(c, &tb, b))
      return bail(1);
    spin_tabs.push_back(ts);
    J_tabs.push_back(tj);
    w0_tabs.push_back(ta);
    w1_tabs.push_back(tb);
    which_tabs.push_back(wc);
    neig_tabs.push_back(neig_rows);
  }
  if (dev_table(c, &c->spinAll, spin_tabs) || dev_table(c, &c->JAll, J_tabs) ||
      dev_table(c, &c->w0All, w0_tabs) || dev_table(c, &c->w1All, w1_tabs) ||
      dev_table(c, &c->whichAll, which_tabs) || dev_table(c, &c->neigAll, neig_tabs))
    return bail(1);
  *out = c;
  return 0;
}

int rg_destroy(void *h) {
  rg_ctx *c = (rg_ctx *)h;
  if (!c) return 0;
  cudaStreamSynchronize(c->stream);
  for (void *p : c->allocs) cudaFree(p);
  if (c->mod) cuModuleUnload(c->mod);
  cudaStreamDestroy(c->stream);
  delete c;
  return 0;
}

/* state of one sample in (J may be NULL to keep the couplings) */
int rg_upload(void *h, int s, const uint64_t *J, const uint64_t *even, const uint64_t *odd,
              const uint64_t *w0, const uint64_t *w1) {
  rg_ctx *c = (rg_ctx *)h;
  const int64_t H = c->H, n = H * c->nr, wrow = n * c->nc;
  if (J)
    for (int k = 0; k < 12; k++) RT(cudaMemcpy(c->J[s * 12 + k], J + k * H, 8 * H, cudaMemcpyHostToDevice));
  RT(cudaMemcpy(c->spin[s * 2], even, 8 * n, cudaMemcpyHostToDevice));
  RT(cudaMemcpy(c->spin[s * 2 + 1], odd, 8 * n, cudaMemcpyHostToDevice));
  for (int p = 0; p < 2; p++) {
    RT(cudaMemcpy(c->w0[s * 2 + p], w0 + p * wrow, 8 * wrow, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(c->w1[s * 2 + p], w1 + p * wrow, 8 * wrow, cudaMemcpyHostToDevice));
  }
  return 0;
}

int rg_download(void *h, int s, uint64_t *even, uint64_t *odd, uint64_t *w0, uint64_t *w1) {
  rg_ctx *c = (rg_ctx *)h;
  const int64_t n = c->H * c->nr, wrow = n * c->nc;
  RT(cudaStreamSynchronize(c->stream));
  RT(cudaMemcpy(even, c->spin[s * 2], 8 * n, cudaMemcpyDeviceToHost));
  RT(cudaMemcpy(odd, c->spin[s * 2 + 1], 8 * n, cudaMemcpyDeviceToHost));
  for (int p = 0; p < 2; p++) {
    RT(cudaMemcpy(w0 + p * wrow, c->w0[s * 2 + p], 8 * wrow, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(w1 + p * wrow, c->w1[s * 2 + p], 8 * wrow, cudaMemcpyDeviceToHost));
  }
  return 0;
}

/* n iterations of Monte_Carlo with flag = 1 (main.cu:254-305) on every
 * sample, queued on the harness's stream */
int rg_iterate(void *h, int64_t n) {
  rg_ctx *c = (rg_ctx *)h;
  int H = (int)c->H, nrep = c->nr, nclone = 1, nc = c->nc;
  void *rand0 = nullptr;
  for (int64_t it = 0; it < n; it++) {
    for (int ic = 0; ic < c->nc; ic++)
      for (int dir = 0; dir < 2; dir++) {
        void *rot = c->rot[dir];
        void *args[] = {&c->spinAll, &dir, &c->JAll, &c->neigAll, &H, &nrep, &nclone,
                        &c->whichAll, &rot, &rand0, &c->w0All, &c->w1All, &ic};
        DRV(cuLaunchKernel(c->sweep, c->nblocks, c->ns, 1, c->tpb, 1, 1, 0,
                           (CUstream)c->stream, args, nullptr));
      }
    for (int dir = 0; dir < 2; dir++) {
      void *rot = c->rot[dir];
      void *args[] = {&dir, &c->neigAll, &H, &nrep, &nclone, &nc, &rot, &c->w0All, &c->w1All};
      DRV(cuLaunchKernel(c->walk, c->nblocks, c->ns, 1, c->tpb, 1, 1, 0, (CUstream)c->stream,
                         args, nullptr));
    }
  }
  return 0;
}

/* mean milliseconds of one iteration over n iterations (CUDA events on the
 * harness's stream, after `warm` untimed ones) */
int rg_time(void *h, int64_t warm, int64_t n, double *ms) {
  rg_ctx *c = (rg_ctx *)h;
  if (rg_iterate(h, warm)) return 1;
  cudaEvent_t a, b;
  RT(cudaEventCreate(&a));
  RT(cudaEventCreate(&b));
  RT(cudaEventRecord(a, c->stream));
  if (rg_iterate(h, n)) return 1;
  RT(cudaEventRecord(b, c->stream));
  RT(cudaEventSynchronize(b));
  float t = 0;
  RT(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = (double)t / (double)n;
  return 0;
}

int rg_launch_shape(void *h, int *tpb, int *nblocks) {
  rg_ctx *c = (rg_ctx *)h;
  *tpb = c->tpb;
  *nblocks = c->nblocks;
  return 0;
}

}  // extern "C"
