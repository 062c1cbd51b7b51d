// emu_runtime.cpp -- thread-index state and the fiber scheduler behind the CUDA emulation prelude
// (oracle/ref_emu/cuda_runtime.h).  TEST INFRASTRUCTURE ONLY.
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cuda_runtime.h"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace {
struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  uint3 idx;
  bool done = false;
};
thread_local ucontext_t t_sched;
thread_local std::vector<Fiber>* t_fibers = nullptr;
thread_local unsigned t_current = 0;
thread_local void (*t_body)(void*, unsigned) = nullptr;
thread_local void* t_arg = nullptr;

void trampoline(int t) {
  t_body(t_arg, static_cast<unsigned>(t));
  (*t_fibers)[static_cast<unsigned>(t)].done = true;
}
}  // namespace

void vh_emu_syncthreads() {
  if (t_fibers == nullptr) {
    std::fprintf(stderr, "cuda emulation: __syncthreads outside a fiber launch\n");
    std::abort();
  }
  Fiber& f = (*t_fibers)[t_current];
  f.idx = threadIdx;
  swapcontext(&f.ctx, &t_sched);
}

void vh_emu_run_fibers(unsigned n, void (*body)(void*, unsigned), void* arg) {
  std::vector<Fiber> fibers(n);
  t_fibers = &fibers;
  t_body = body;
  t_arg = arg;
  for (unsigned t = 0; t < n; ++t) {
    Fiber& f = fibers[t];
    f.stack.resize(256 * 1024);
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = f.stack.data();
    f.ctx.uc_stack.ss_size = f.stack.size();
    f.ctx.uc_link = &t_sched;
    makecontext(&f.ctx, reinterpret_cast<void (*)()>(trampoline), 1, static_cast<int>(t));
  }
  bool started = false;
  for (;;) {
    bool any = false;
    for (unsigned t = 0; t < n; ++t) {
      Fiber& f = fibers[t];
      if (f.done) continue;
      any = true;
      t_current = t;
      if (started) threadIdx = f.idx;
      swapcontext(&t_sched, &f.ctx);
    }
    started = true;
    if (!any) break;
  }
  t_fibers = nullptr;
}
