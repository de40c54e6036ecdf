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
  unsigned long long word[2];  // grid_sync_verdict's arrivals, by barrier parity
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

__device__ __forceinline__ void kf_red_release_add64(unsigned long long *p, unsigned long long v) {
  asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long kf_ld_acquire64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Thread 0's wait after an arrival: polls until `done(value)` holds, the
// limit passes or another block gives up; false in the last two cases.
template <typename Load, typename Done>
__device__ __forceinline__ bool kf_bounded_poll(GridSync *g, unsigned long long limit_ns, int where, Load load,
                                                Done done) {
  volatile int *timed_out = &g->timed_out;
  if (limit_ns == 0) {
    if (atomicExch(&g->timed_out, 1) == 0) g->where = where;
    return false;
  }
  unsigned long long t0 = 0;
  for (int spin = 0;; ++spin) {
    if (done(load())) return !*timed_out;
    if (*timed_out) return false;
    // the first polls run back to back (a barrier normally completes
    // within a few microseconds); then sleep between polls and watch
    // the clock
    if (spin == 64) t0 = kf_globaltimer_ns();
    if (spin > 64) {
      if (kf_globaltimer_ns() - t0 > limit_ns) {
        if (atomicExch(&g->timed_out, 1) == 0) g->where = where;
        return false;
      }
      __nanosleep(64);
    }
  }
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
    kf_red_release_add(&g->count, 1u);
    const unsigned target = nblocks * (unsigned)(where + 1);
    s_ok = kf_bounded_poll(
        g, limit_ns, where, [&] { return kf_ld_acquire(&g->count); },
        [&](unsigned v) { return (int)(v - target) >= 0; });
  }
  __syncthreads();
  return s_ok != 0;
}

// The same barrier, whose arrival also carries two facts about the block's
// iteration: they come back with the barrier, in the round trip of its last
// poll, where reading them from memory after the barrier would take one
// more.  Barrier b uses word[b % 2]; a block adds
//   1 + (kVerdictOpen if `open`) + (kVerdictFail if `fail`)
// (bits 0-31 count arrivals, 32-47 and 48-63 the blocks with each fact),
// and thread 0 keeps in `seen` the word's value when its previous barrier
// completed.  The increase since then is barrier b's alone: no block
// arrives at barrier b + 2 before every block has arrived at b + 1, and a
// block reads the word of barrier b only before its own arrival at b + 1.
// The barrier is complete when the increase counts nblocks arrivals
// (nblocks < 2^16); *any_open and *any_fail then tell whether some block
// had each fact.  `after_arrive` runs on thread 0 between its arrival and
// its wait (writes that no block reads before the kernel ends).
constexpr unsigned long long kVerdictOpen = 1ull << 32;
constexpr unsigned long long kVerdictFail = 1ull << 48;

template <typename AfterArrive>
__device__ __forceinline__ bool grid_sync_verdict(GridSync *g, unsigned nblocks, unsigned long long limit_ns,
                                                  int where, bool open, bool fail, unsigned long long &seen,
                                                  bool &any_open, bool &any_fail, AfterArrive after_arrive) {
  __shared__ int s_ok, s_open, s_fail;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long *w = &g->word[where & 1];
    kf_red_release_add64(w, 1ull + (open ? kVerdictOpen : 0ull) + (fail ? kVerdictFail : 0ull));
    after_arrive();
    unsigned long long inc = 0;
    const bool ok = kf_bounded_poll(
        g, limit_ns, where, [&] { return kf_ld_acquire64(w); },
        [&](unsigned long long v) {
          inc = v - seen;
          return (unsigned)inc == nblocks;
        });
    seen += inc;
    s_ok = ok;
    s_open = (inc >> 32 & 0xffffu) != 0;
    s_fail = (inc >> 48) != 0;
  }
  __syncthreads();
  any_open = s_open != 0;
  any_fail = s_fail != 0;
  return s_ok != 0;
}
