// Grid-wide barrier with a bounded wait, for the persistent kernels that run
// every iteration of a solve in one cooperative launch (the band-only solver
// and the batched solver).  A Jacobi step reads its neighbours' psi of the
// iteration before, so the blocks must all finish an iteration before any
// starts the next; a kernel boundary gave that barrier before, at the cost of
// a launch per iteration.
//
// The launch is cooperative (cudaLaunchCooperativeKernel), so every block of
// the grid is resident and the barrier cannot deadlock on a block that never
// started.  Each wait is still bounded: a block that has waited longer than
// the limit (kf_set_wait_limit, one second by default) marks the barrier as
// failed and returns, and every other block returns at its next wait or
// right after its current one, so the kernel always ends.  The host then
// reports KF_ERR_TIMEOUT.  A limit of zero makes every wait give up at once.
//
// The count only grows: barrier b (0, 1, ...) is passed once it reaches
// nblocks * (b + 1), so no block has to reset it and release the others.
// Arrival is a release reduction (this block's writes become visible before
// its count), the wait an acquire load (the other blocks' writes are visible
// after it): every thread of the block reaches them through __syncthreads,
// as in a cooperative-groups grid sync.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

struct GridSync {
  unsigned count;  // arrivals at all barriers so far
  unsigned pad_;
  int timed_out;   // set by the first block whose wait gave up
  int where;       // the barrier (iteration) at which it gave up
};

__device__ __forceinline__ unsigned long long kf_globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void kf_red_release_add(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned kf_ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Barrier number `where` (0, 1, ... in the order the kernel reaches them).
// Every thread of every block calls it.  Returns true when all blocks have
// arrived; false when this block's wait gave up or another block's had (the
// kernel must then return).
__device__ __forceinline__ bool grid_sync(GridSync *g, unsigned nblocks, unsigned long long limit_ns,
                                          int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile int *timed_out = &g->timed_out;
    kf_red_release_add(&g->count, 1u);
    const unsigned target = nblocks * (unsigned)(where + 1);
    int ok = 1;
    if (limit_ns == 0) {
      ok = 0;
      if (atomicExch(&g->timed_out, 1) == 0) g->where = where;
    } else {
      unsigned long long t0 = 0;
      for (int spin = 0;; ++spin) {
        if ((int)(kf_ld_acquire(&g->count) - target) >= 0) break;
        if (*timed_out) {
          ok = 0;
          break;
        }
        // the first polls run back to back (a barrier normally completes
        // within a few microseconds); then sleep between polls and watch
        // the clock
        if (spin == 64) t0 = kf_globaltimer_ns();
        if (spin > 64) {
          if (kf_globaltimer_ns() - t0 > limit_ns) {
            if (atomicExch(&g->timed_out, 1) == 0) g->where = where;
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    if (ok && *timed_out) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}
