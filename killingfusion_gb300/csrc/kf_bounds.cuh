// Bounds-check build mode (the library compiled with -DKF_BOUNDS_CHECK,
// killingfusion_gb300/_lib/libkillingfusion_bc.so).
//
// compute-sanitizer is not available where this library is tested, so the
// kernels of the hot path check, in this build, every index they take from
// data rather than from their own loop bounds: band-list entries and the
// positions they are appended at, the dense passes' shared-memory queues and
// run tables, the in-place write-back, the side lists of warp + fuse and of
// integration, and the marching-cubes block list and triangle slots.  An index outside its bound is not used (the access is
// skipped) and the first one is recorded -- its site, index and bound -- in
// a device record that the host reads with kf_bounds_status.  In the normal
// build every check compiles to nothing.
//
// kf_bounds_set_limit lowers every bound to a given value, in this build
// only, so that a test can make the checks fire on a small grid without any
// access leaving its buffer: the flagged accesses are then skipped.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kf_internal.h"

// Sites of the checks (kf_bounds_status reports the first one hit).
enum KfBoundsSite {
  KF_SITE_BAND_LIST = 1,    // a voxel read from a band list
  KF_SITE_BAND_APPEND = 2,  // a position appended to in a band list
  KF_SITE_STREAM_QUEUE = 3, // a dense pass's shared-memory queue
  KF_SITE_STREAM_LIST = 4,  // a position the dense pass lists a voxel at
  KF_SITE_WRITE_BACK = 5,   // a voxel or slot of the in-place write-back
  KF_SITE_SIDE_LIST = 7,    // warp + fuse's moved-voxel list
  KF_SITE_INTEGRATE_LIST = 8, // integration's float64 list
  KF_SITE_MC_BLOCK = 9,     // a marching-cubes block or triangle slot
  KF_SITE_RUNS = 10         // the split schedule's run lists
};


#ifdef KF_BOUNDS_CHECK
namespace {
// one record and one limit per translation unit (read and reset through
// kf_bounds_tu_* of that unit)
__device__ KfBoundsRecord g_kf_bounds;
__device__ long long g_kf_bounds_limit = 0x7fffffffffffffffLL;

__device__ __noinline__ bool kf_bounds_fail(long long idx, long long bound, int site) {
  if (atomicAdd(&g_kf_bounds.count, 1u) == 0u) {
    g_kf_bounds.site = site;
    g_kf_bounds.index = idx;
    g_kf_bounds.bound = bound;
  }
  return false;
}

__device__ __forceinline__ bool kf_in_bounds(long long idx, long long bound, int site) {
  const long long b = bound < g_kf_bounds_limit ? bound : g_kf_bounds_limit;
  return (idx >= 0 && idx < b) ? true : kf_bounds_fail(idx, b, site);
}
}  // namespace
#define KF_IN_BOUNDS(idx, bound, site) kf_in_bounds((long long)(idx), (long long)(bound), (site))

// Host side of one translation unit's record and limit.
#define KF_BOUNDS_TU_API(tu)                                                         \
  int kf_bounds_tu_read_##tu(KfBoundsRecord *r) {                                    \
    return (int)cudaMemcpyFromSymbol(r, g_kf_bounds, sizeof(*r));                    \
  }                                                                                  \
  int kf_bounds_tu_reset_##tu(long long limit) {                                     \
    KfBoundsRecord z = {0u, 0, 0, 0};                                                \
    cudaError_t e = cudaMemcpyToSymbol(g_kf_bounds, &z, sizeof(z));                  \
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_kf_bounds_limit, &limit, sizeof(limit)); \
    return (int)e;                                                                   \
  }
#else
#define KF_IN_BOUNDS(idx, bound, site) true
#define KF_BOUNDS_TU_API(tu)                                                          \
  int kf_bounds_tu_read_##tu(KfBoundsRecord *r) {                                     \
    r->count = 0;                                                                     \
    r->site = 0;                                                                      \
    r->index = r->bound = 0;                                                          \
    return 0;                                                                         \
  }                                                                                   \
  int kf_bounds_tu_reset_##tu(long long) { return 0; }
#endif
