/*
 * cuda_runtime.h -- host-only CUDA emulation prelude used by oracle/build.py (build_ref) to compile the
 * reference's CUDA sources (src/cuda_*.cu) as ordinary C++ for the CPU.
 *
 * TEST INFRASTRUCTURE ONLY: it lets the reference's own kernels run sequentially on the host so
 * the oracle's GPU flavour can be checked against them bit-for-bit.  Device memory is host
 * memory, "atomics" are plain read-modify-writes (kernels run one thread at a time), kernel
 * launches loop over the grid and the block, and the one kernel that uses __syncthreads runs its
 * threads as ucontext fibers (vh_emu_launch_sync).
 */
#pragma once
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cstddef>

struct uint3 {
  unsigned int x, y, z;
};
struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

enum cudaError_t { cudaSuccess = 0, cudaErrorUnknown = 999 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
inline const char* cudaGetErrorString(cudaError_t) { return "cuda emulation"; }
inline cudaError_t cudaMalloc(void** p, size_t n) {
  *p = calloc(n ? n : 1, 1);
  return *p ? cudaSuccess : cudaErrorUnknown;
}
inline cudaError_t cudaFree(void* p) {
  free(p);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  memmove(d, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemset(void* d, int v, size_t n) {
  memset(d, v, n);
  return cudaSuccess;
}
template <class T>
cudaError_t cudaMemcpyToSymbol(T& sym, const void* s, size_t n) {
  memcpy((void*)&sym, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int* c) {
  *c = 1;
  return cudaSuccess;
}

inline unsigned long long atomicCAS(unsigned long long* a, unsigned long long c, unsigned long long v) {
  const unsigned long long o = *a;
  if (o == c) *a = v;
  return o;
}
inline unsigned int atomicAdd(unsigned int* a, unsigned int v) {
  const unsigned int o = *a;
  *a = o + v;
  return o;
}
inline unsigned long long atomicAdd(unsigned long long* a, unsigned long long v) {
  const unsigned long long o = *a;
  *a = o + v;
  return o;
}
inline unsigned int atomicExch(unsigned int* a, unsigned int v) {
  const unsigned int o = *a;
  *a = v;
  return o;
}
inline int min(int a, int b) { return a < b ? a : b; }

#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__ static

void vh_emu_syncthreads();
#define __syncthreads() vh_emu_syncthreads()

/* runs body(arg, t) for t in [0, n) as fibers that switch at every __syncthreads */
void vh_emu_run_fibers(unsigned n, void (*body)(void*, unsigned), void* arg);

template <class K, class... A>
void vh_emu_launch(K kernel, dim3 g, dim3 b, A... args) {
  gridDim = g;
  blockDim = b;
  for (unsigned bz = 0; bz < g.z; ++bz)
    for (unsigned by = 0; by < g.y; ++by)
      for (unsigned bx = 0; bx < g.x; ++bx) {
        blockIdx = uint3{bx, by, bz};
        for (unsigned tz = 0; tz < b.z; ++tz)
          for (unsigned ty = 0; ty < b.y; ++ty)
            for (unsigned tx = 0; tx < b.x; ++tx) {
              threadIdx = uint3{tx, ty, tz};
              kernel(args...);
            }
      }
}

template <class K, class... A>
void vh_emu_launch_sync(K kernel, dim3 g, dim3 b, A... args) {
  gridDim = g;
  blockDim = b;
  auto body = [&](unsigned t) {
    threadIdx = uint3{t % b.x, (t / b.x) % b.y, t / (b.x * b.y)};
    kernel(args...);
  };
  using Body = decltype(body);
  for (unsigned bz = 0; bz < g.z; ++bz)
    for (unsigned by = 0; by < g.y; ++by)
      for (unsigned bx = 0; bx < g.x; ++bx) {
        blockIdx = uint3{bx, by, bz};
        vh_emu_run_fibers(b.x * b.y * b.z, [](void* p, unsigned t) { (*static_cast<Body*>(p))(t); }, &body);
      }
}
