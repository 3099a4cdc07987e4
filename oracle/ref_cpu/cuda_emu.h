/*
 * cuda_emu.h -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * A minimal CUDA-runtime emulation that lets the reference program
 * (IsidoroGlez/micSA-EA-MC, PROGRAM/src/main.cu) be compiled by g++ and run
 * entirely on the host.  It is force-included (`-include`) into main.cu only.
 *
 * Why this is a faithful execution of the reference kernels:
 *   - d_oneMCstepBN_multisample (main.cu:847-1080) writes only the thread's own
 *     spin and demon words and reads the other checkerboard colour: every
 *     thread order gives the same result.
 *   - d_Walk (main.cu:1084-1193) swaps each demon word with the word of its
 *     ic-direction neighbour; the neighbour map is a bijection between the two
 *     colours, so every pair is touched by exactly one thread.
 *   - d_gen_rndbits_cuda (main.cu:647-702) is a pure function of the thread id.
 *   - d_computeEne (main.cu:745-815) only accumulates with atomicAdd (integer,
 *     order independent).
 * None of the kernels uses shared memory or barriers, so running the threads
 * one after another in a loop reproduces the GPU result bit for bit.
 *
 * Device memory is host memory; cudaMemcpy is memcpy.  Kernel launches are
 * rewritten (by the build recipe, in a pipe) from `k<<<g,b[,s,st]>>>(args)` to
 * `EMU_LAUNCH(k, g, b[, s, st])(args)`.
 */
#ifndef MICSA_CUDA_EMU_H
#define MICSA_CUDA_EMU_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

struct uint4 { uint32_t x, y, z, w; };
struct uint2 { uint32_t x, y; };
struct uint3 { unsigned int x, y, z; };
struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

static uint3 threadIdx, blockIdx;
static dim3 blockDim, gridDim;

#define __global__
#define __device__
#define __host__
#define __constant__
#define __managed__
#define __launch_bounds__(...)

typedef int cudaError;
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3
};
typedef void *cudaStream_t;

static inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }
static inline cudaError_t cudaGetLastError(void) { return cudaSuccess; }
static inline cudaError_t cudaGetDeviceCount(int *n) { *n = 1; return cudaSuccess; }
static inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
static inline cudaError_t cudaStreamCreate(cudaStream_t *s) { *s = 0; return cudaSuccess; }

static inline cudaError_t cudaMalloc(void **p, size_t n) {
  *p = calloc(1, n ? n : 1);
  return *p ? cudaSuccess : 2;
}
template <class T> static inline cudaError_t cudaMalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, n);
}
static inline cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
  memmove(d, s, n);
  return cudaSuccess;
}
static inline cudaError_t cudaMemset(void *d, int v, size_t n) {
  memset(d, v, n);
  return cudaSuccess;
}
template <class T>
static inline cudaError_t cudaMemcpyToSymbol(T &sym, const void *src, size_t n,
                                             size_t off = 0,
                                             cudaMemcpyKind = cudaMemcpyHostToDevice) {
  memcpy((char *)&sym + off, src, n);
  return cudaSuccess;
}

static inline uint32_t __umulhi(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}
template <class T> static inline T __ldg(const T *p) { return *p; }
static inline int atomicAdd(int *a, int v) { int o = *a; *a = o + v; return o; }

static inline dim3 emu_dim(dim3 d) { return d; }
static inline dim3 emu_dim(unsigned int n) { return dim3(n); }
static inline dim3 emu_dim(int n) { return dim3((unsigned int)n); }

/* Serial grid execution of a kernel: block by block, thread by thread. */
template <class K, class G, class B, class... Rest>
static auto emu_make_launch(K kernel, G g, B b, Rest...) {
  dim3 grid = emu_dim(g), block = emu_dim(b);
  return [=](auto... args) {
    gridDim = grid;
    blockDim = block;
    for (unsigned bz = 0; bz < grid.z; bz++)
      for (unsigned by = 0; by < grid.y; by++)
        for (unsigned bx = 0; bx < grid.x; bx++)
          for (unsigned tz = 0; tz < block.z; tz++)
            for (unsigned ty = 0; ty < block.y; ty++)
              for (unsigned tx = 0; tx < block.x; tx++) {
                blockIdx.x = bx; blockIdx.y = by; blockIdx.z = bz;
                threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = tz;
                kernel(args...);
              }
  };
}
#define EMU_LAUNCH(k, ...) emu_make_launch(k, __VA_ARGS__)

#endif
