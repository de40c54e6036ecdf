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
// reports KF_ERR_TIMEOUT.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

struct GridSync {
  unsigned count;  // blocks arrived at the current barrier
  unsigned gen;    // barriers completed
  int timed_out;   // set by the first block whose wait gave up
  int where;       // the barrier (iteration) at which it gave up
};

__device__ __forceinline__ unsigned long long kf_globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Every thread of every block calls it.  Returns true when all blocks have
// arrived; false when this block's wait gave up or another block's had
// (the kernel must then return).  Memory written before the barrier by any
// block is visible after it to every block: each block fences before it
// arrives and after it leaves (the pattern of a cooperative-groups grid sync).
__device__ __forceinline__ bool grid_sync(GridSync *g, unsigned nblocks, unsigned long long limit_ns,
                                          int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile GridSync *vg = g;
    const unsigned gen = vg->gen;  // read before arriving: it cannot advance until we have
    __threadfence();
    int ok = 1;
    if (atomicAdd(&g->count, 1u) == nblocks - 1) {
      // the last to arrive: reset the count for the next barrier, then release
      atomicExch(&g->count, 0u);
      __threadfence();
      atomicAdd(&g->gen, 1u);
    } else {
      const unsigned long long t0 = kf_globaltimer_ns();
      while (vg->gen == gen) {
        if (vg->timed_out) {
          ok = 0;
          break;
        }
        if (kf_globaltimer_ns() - t0 > limit_ns) {
          if (atomicExch(&g->timed_out, 1) == 0) g->where = where;
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (vg->timed_out) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}
