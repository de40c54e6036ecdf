// Fused float32 psi update (KillingFusion::computeDisplacementField,
// KillingFusion.cpp:248-352, with the gradient of
// KillingFusion::computeEnergyGradient, :399-476) and the CUDA-graph capture
// of the fixed-iteration loop.
//
// An iteration (KF_SOLVER_FUSED) is two passes over psi held in place:
//   k_fused_stream (dense)  reads psi and phi_live and applies the band test
//     of KillingFusion.cpp:272-274.  The warped value phi_live(i + psi(i)) is
//     phi_live(i) itself when psi(i) == 0 (zero interpolation weights), so only
//     voxels that have moved gather their 8 corners.  A voxel outside the
//     band keeps its psi, which therefore need not be written; the voxels
//     inside are compacted into a list.  16 bytes per voxel.
//   k_fused_band  evaluates the full gradient of every listed voxel, one
//     thread per voxel: the thread loads the 20 psi neighbours
//     of the stencil per component, takes the 25 warped-SDF samples of the
//     gradient and Hessian at compile-time offsets plus the warped value (26
//     independent trilinear gathers), and applies the reference's difference
//     stencils.  The new psi goes to a side buffer indexed by list position,
//     so every voxel still reads its neighbours' old values (Jacobi).
//   The next iteration's dense pass writes the band voxels' new psi back,
//     each run of voxels its own (k_fused_scatter after the last iteration).
// The band-only solver (KF_SOLVER_BAND) runs the dense pass once.  A voxel
// outside the band keeps psi, so its band test keeps failing and the band can
// only shrink: each band pass hands the voxels it updated to the next
// iteration, which re-tests them with the warped value it samples anyway and
// copies the ones that left the band into its output buffer (ping-pong
// buffers).  Both solvers produce the same psi.
//
// In the interior the psi samples that the reference takes at sub-voxel offsets
// are closed-form linear combinations of the 3x3x3 neighbourhood:
//   Killing (at i + h*o):  second differences 2h*(psi(+1) - 2psi(0) + psi(-1))
//     on the axes and h^2*(psi(++) - psi(+-) - psi(-+) + psi(--)) on the
//     diagonals;
//   cell centre (at i + 0.5 + h*o):  m0 + h*(o.m1) + h^2*(pairwise o o.m2)
//     from eight moments of the cell [i, i+1]^3.
// Voxels on the grid's outer shell take the generic reference-order path
// (truncating casts, linear-index wrap, outside values).
#include <algorithm>

#include "kf_fused_body.cuh"
#include "kf_grid_sync.cuh"

namespace {

// Dense pass: stream the slab, list the band voxels (st[iter].list counts
// them); kPassThrough copies psi of the other voxels to the output buffer.
// In place (runs != NULL): the run first writes back the new psi that the
// previous iteration's band pass left for its own band voxels -- the entries
// runs[run] of prev_list and of the second planes (a.ox..a.oz) -- and then
// streams; it records where its band voxels land in `list`.
template <bool kPassThrough>
__global__ void __launch_bounds__(kThreads) k_fused_stream(FusedArgs a, int *__restrict__ list,
                                                          const int *__restrict__ prev_list,
                                                          int2 *__restrict__ runs) {
  if (runs && a.iter > 0 && !a.st[a.iter - 1].skipped) {
    const int2 r = runs[blockIdx.x];
    float *px = const_cast<float *>(a.ix), *py = const_cast<float *>(a.iy), *pz = const_cast<float *>(a.iz);
    for (int j = threadIdx.x; j < r.y; j += kThreads) {
      const int slot = r.x + j;
      if (!KF_IN_BOUNDS(slot, a.dp.count, KF_SITE_WRITE_BACK)) continue;
      const int v = prev_list[slot];
      if (!KF_IN_BOUNDS(v, a.dp.count, KF_SITE_WRITE_BACK)) continue;
      px[v] = a.ox[slot];
      py[v] = a.oy[slot];
      pz[v] = a.oz[slot];
    }
    __syncthreads();
  }
  if (iteration_gated(a.st, a.iter, a.dp)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st[a.iter].skipped = 1;
    return;
  }
  stream_flat<kPassThrough>(a, blockIdx.x, list, &a.st[a.iter].list, runs ? runs + blockIdx.x : nullptr);
}

// The band-only solver's first band test when both psi buffers are zero at
// every voxel: psi(i) = 0 samples voxel i's own cell with zero weights, so
// the test reads phi_live alone (4 B a voxel, against 16 B read and 12 B
// copied by k_fused_stream<true>), and the second buffer already holds
// every voxel's psi.  The same list as k_fused_stream<true> gives.
__global__ void __launch_bounds__(kThreads) k_band_first_zero(FusedArgs a, int *__restrict__ list) {
  stream_flat<false, false, true>(a, blockIdx.x, list, &a.st[a.iter].list, nullptr);
}

// Split dense schedule (grids of at least kSplitMinRuns runs).  After the
// first iteration's dense pass, k_split_runs sorts the runs into those that
// listed band voxels ("hot") and the others ("cold"), each in run order.  A
// voxel outside the band keeps its psi and phi_live does not change, so the
// band tests of a cold run give the first iteration's result again: a cold
// run has no psi to write back and no band voxel, and no band pass reads
// anything a cold pass writes.  Every later iteration streams its hot runs
// (write-back, test, list) on the solve's stream, before its band pass, and
// its cold runs (test only) on a second stream, beside the band pass of the
// iteration before.  A band voxel found in a cold run is counted in
// IterStats::cold and fails the solve.
constexpr int kSplitMinRuns = 512;
constexpr int kSplitThreads = 1024;
constexpr int kHotBlocksPerSM = 5;  // resident CTAs of k_fused_stream (48 registers)

__global__ void __launch_bounds__(kSplitThreads) k_split_runs(const int2 *__restrict__ runs, int nruns,
                                                             int *__restrict__ hot, int *__restrict__ cold,
                                                             unsigned *__restrict__ counts) {
  __shared__ int s_warp[kSplitThreads / 32];
  __shared__ int s_total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // thread t takes the runs [r0, r1)
  const int per = (nruns + kSplitThreads - 1) / kSplitThreads;
  const int r0 = min(tid * per, nruns), r1 = min(r0 + per, nruns);
  int mine = 0;
  for (int r = r0; r < r1; ++r) mine += runs[r].y > 0;
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int w = s_warp[lane];
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += v;
    }
    s_warp[lane] = wi - w;
    if (lane == 31) s_total = wi;
  }
  __syncthreads();
  int h = s_warp[warp] + incl - mine;  // hot runs before r0
  int c = r0 - h;                       // cold runs before r0
  for (int r = r0; r < r1; ++r) {
    if (runs[r].y > 0) {
      if (KF_IN_BOUNDS(h, nruns, KF_SITE_RUNS)) hot[h] = r;
      ++h;
    } else {
      if (KF_IN_BOUNDS(c, nruns, KF_SITE_RUNS)) cold[c] = r;
      ++c;
    }
  }
  if (tid == 0) {
    counts[0] = (unsigned)s_total;
    counts[1] = (unsigned)(nruns - s_total);
  }
}

// Dense pass of iteration a.iter >= 1 over the listed runs (counts[0] hot
// runs, counts[1] cold runs), a run per loop step.  Hot: each run writes
// back its band voxels' new psi from the iteration before (as
// k_fused_stream), then streams and lists.  Cold (kCold): the runs are
// tested only; their band voxels, never expected, are counted in
// st[iter].cold.  A cold pass stops once the iteration before it was
// skipped (the statistics of that iteration's band pass may still be in
// flight when it runs, so it may run once after convergence, to no effect).
template <bool kCold>
__global__ void __launch_bounds__(kThreads) k_fused_stream_runs(FusedArgs a, const int *__restrict__ run_list,
                                                               const unsigned *__restrict__ counts,
                                                               int *__restrict__ list,
                                                               const int *__restrict__ prev_list,
                                                               int2 *__restrict__ runs) {
  const unsigned n = counts[kCold ? 1 : 0];
  if (kCold) {
    if (a.st[a.iter - 1].skipped) return;
    for (unsigned idx = blockIdx.x; idx < n; idx += gridDim.x) {
      const int r = run_list[idx];
      if (KF_IN_BOUNDS(r, max((a.dp.count / 4 + kThreads * kFlatGroups - 1) / (kThreads * kFlatGroups), (int64_t)1),
                       KF_SITE_RUNS))
        stream_flat<false, true>(a, r, nullptr, &a.st[a.iter].cold);
      __syncthreads();
    }
    return;
  }
  const bool write_back = !a.st[a.iter - 1].skipped;
  const bool gated = iteration_gated(a.st, a.iter, a.dp);
  if (gated && blockIdx.x == 0 && threadIdx.x == 0) a.st[a.iter].skipped = 1;
  float *px = const_cast<float *>(a.ix), *py = const_cast<float *>(a.iy), *pz = const_cast<float *>(a.iz);
  for (unsigned idx = blockIdx.x; idx < n; idx += gridDim.x) {
    const int r = run_list[idx];
    if (!KF_IN_BOUNDS(r, max((a.dp.count / 4 + kThreads * kFlatGroups - 1) / (kThreads * kFlatGroups), (int64_t)1),
                      KF_SITE_RUNS))
      continue;
    if (write_back) {
      const int2 rr = runs[r];
      for (int j = threadIdx.x; j < rr.y; j += kThreads) {
        const int slot = rr.x + j;
        if (!KF_IN_BOUNDS(slot, a.dp.count, KF_SITE_WRITE_BACK)) continue;
        const int v = prev_list[slot];
        if (!KF_IN_BOUNDS(v, a.dp.count, KF_SITE_WRITE_BACK)) continue;
        px[v] = a.ox[slot];
        py[v] = a.oy[slot];
        pz[v] = a.oz[slot];
      }
      __syncthreads();
    }
    if (!gated) stream_flat<false>(a, r, list, &a.st[a.iter].list, runs + r);
    __syncthreads();
  }
}

// Band pass: one thread per listed voxel, launched as one resident
// wave that loops over the list.  kCarry (band-only solver): the voxels
// updated here form the next iteration's list (list_out, counted in
// st[iter+1].list).  kInPlace: the new psi of list entry k goes to entry k
// of the output planes, for k_fused_scatter to write back.  kTrust: the
// trust-region step (dp.trust), followed by k_trust_fix.
template <bool kCarry, bool kInPlace, bool kTrust = false>
__global__ void __launch_bounds__(kLaneThreads, kLaneBlocksPerSM) k_fused_band(FusedArgs a, const int *__restrict__ list_in,
                                                             int *__restrict__ list_out) {
  if (iteration_gated(a.st, a.iter, a.dp)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st[a.iter].skipped = 1;
    return;
  }
  const int nq = (int)a.st[a.iter].list;
  const int total_threads = gridDim.x * kLaneThreads;
  const int rounds = (nq + total_threads - 1) / total_threads;
  float maxd = 0.f;
  double energy = 0.0;  // this thread's voxels, summed in float64 as the block and grid sums
  unsigned active = 0;
  bool diverged = false;
  for (int r = 0; r < rounds; ++r) {
    const int k = (r * gridDim.x + blockIdx.x) * kLaneThreads + threadIdx.x;
    int next = -1;  // voxel this thread hands to the next iteration
    if (k < nq) {
      const int v = list_in[k];
      next = update_band_voxel<kTrust>(a, v, kInPlace ? k : v, maxd, energy, active, diverged);
    }
    if (kCarry) block_append<kLaneWarps>(next, &a.st[a.iter + 1].list, list_out, a.dp.count);
  }
  reduce_iter_stats<kLaneThreads>(a.st + a.iter, active, maxd, energy, diverged);
}

// Band-only solver, every iteration in one cooperative launch.  One band pass
// per iteration as k_fused_band<kCarry> (ping-pong buffers, the updated
// voxels carried to the next iteration's list), then a grid-wide barrier
// (kf_grid_sync.cuh) instead of a kernel boundary.
// - Each block takes an equal contiguous slice of the first band list and
//   keeps its own voxels from then on: the band can only shrink, so a
//   block's carried voxels are compacted into its own slice of the other
//   list, with no global atomic on the iteration's critical path.
// - A block's voxels alternate between its warps, so that a small band (a
//   few dozen voxels per block at 256^3) keeps every scheduler of the SM
//   busy; neighbouring band voxels (which share psi neighbours) stay in one
//   SM's L1.
// - psi is read through L1 and L2 (kPsiL1: the blocks write it between
//   iterations, ordered by the barrier's fences), the SDFs through the
//   read-only path.  A gated iteration (converged, diverged) ends the kernel
//   in every block alike: the barrier brings each block the same verdict
//   (grid_sync_verdict), so no block reads the statistics after it, and a
//   block's first round of voxels comes from shared memory: the psi loads
//   of the next iteration start as soon as the barrier lets a block go.
// 96-thread blocks, 1 per SM: a 255-register budget (the band update does
// not spill), three warps a block, most of each SM's registers left to the
// frame's other kernels, which run beside the solve.  The grid barrier's
// cost grows with the number of blocks (alone, with no work between
// barriers: 2.3 us for 608 blocks, 1.5 us for 304, 1.3 us for 152); of
// 64-256 threads a block, 96 gave the bench's band (about 95 voxels a block)
// its shortest iterations.
constexpr int kPersistThreads = 96;
constexpr int kPersistWarps = kPersistThreads / 32;
constexpr int kPersistBlocksPerSM = 1;

// Compacts the voxels `next` (>= 0 on the threads that carry one) of the
// block into out[base...] (capacity entries), with no atomic; returns how
// many there were.  The first kPersistThreads entries of out (the next
// iteration's first round) also go to first[].  Every thread of the block
// calls it.
__device__ __forceinline__ unsigned block_compact(int next, int *__restrict__ out, unsigned base,
                                                  unsigned capacity, int *first) {
  __shared__ unsigned s_w[kPersistWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool has = next >= 0;
  const unsigned ball = __ballot_sync(0xffffffffu, has);
  if (lane == 0) s_w[warp] = (unsigned)__popc(ball);
  __syncthreads();
  unsigned before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kPersistWarps; ++w) {
    const unsigned c = s_w[w];
    before += w < warp ? c : 0u;
    total += c;
  }
  if (has) {
    const unsigned pos = base + before + (unsigned)__popc(ball & ((1u << lane) - 1u));
    if (KF_IN_BOUNDS(pos, capacity, KF_SITE_BAND_APPEND)) out[pos] = next;
    if (pos < (unsigned)kPersistThreads) first[pos] = next;
  }
  __syncthreads();  // s_w is written again by the next call
  return total;
}

// Iteration `it` of the block's n voxels in[0..n) (carried ones to out,
// n updated); false when the kernel must end (the iteration was the last,
// a barrier wait gave up, or the next iteration is gated).  The entries
// in[0..kPersistThreads) are read from first[] (from `in` at it == 0), so
// that a thread's first voxel is known as soon as the barrier lets it go.
// seen: grid_sync_verdict's record of this iteration's barrier word.
__device__ __forceinline__ bool persistent_band_iteration(const FusedArgs &a, int it, bool last,
                                                          const int *__restrict__ in, int *__restrict__ out,
                                                          unsigned &n, unsigned capacity, GridSync *sync,
                                                          unsigned long long limit_ns, int *first,
                                                          unsigned long long &seen) {
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned k0 = lane * kPersistWarps + warp;  // this thread's voxel of round 0
  const int v0 = k0 < n ? (it == 0 ? __ldcg(in + k0) : first[k0]) : -1;
  const unsigned rounds = (n + kPersistThreads - 1) / kPersistThreads;
  float maxd = 0.f;
  double energy = 0.0;
  unsigned active = 0, carried = 0;
  bool diverged = false;
  for (unsigned r = 0; r < rounds; ++r) {
    const unsigned k = r * kPersistThreads + k0;
    int next = -1;
    if (k < n) {
      const int v = r == 0 ? v0 : __ldcg(in + k);
      next = update_band_voxel<false, kPsiL1>(a, v, v, maxd, energy, active, diverged);
    }
    carried += block_compact(next, out, carried, capacity, first);
  }
  n = carried;
  BlockStats b{};  // the block's totals, on thread 0
  reduce_iter_stats<kPersistThreads>(a.st + it, active, maxd, energy, diverged, &b);
  if (last) {
    if (threadIdx.x == 0) commit_iter_stats(a.st + it, b);
    return false;
  }
  // the gate of iteration it + 1 (iteration_gated): no block diverged, and
  // with early_exit some block moved psi by more than the threshold; the
  // statistics are committed while the barrier completes
  bool any_open = false, any_fail = false;
  if (!grid_sync_verdict(sync, gridDim.x, limit_ns, it, b.max_delta > (float)a.dp.threshold, b.diverged, seen,
                         any_open, any_fail, [&] { commit_iter_stats(a.st + it, b); })) {
    if (threadIdx.x == 0) a.st[0].timeout = 1;
    return false;
  }
  if (any_fail || (a.dp.early_exit && !any_open)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st[it + 1].skipped = 1;
    return false;
  }
  return true;
}

// even: psi in the primary planes, out to the second; odd: the reverse.
// The band list of the dense first pass is lst0[0, st[0].list).  touched
// (or NULL): a copy of that list and its length, the only voxels whose psi
// the solve can change (the iterations overwrite lst0).
__global__ void __launch_bounds__(kPersistThreads, kPersistBlocksPerSM)
    k_band_persistent(FusedArgs even, FusedArgs odd, int *lst0, int *lst1, int iterations, GridSync *sync,
                      unsigned long long limit_ns, int *touched, unsigned *touched_n) {
  const unsigned nq = __ldcg(&even.st[0].list);
  const unsigned per = (nq + gridDim.x - 1) / gridDim.x;  // this block's slice [k0, k0 + per)
  const unsigned k0 = min(blockIdx.x * per, nq);
  unsigned n = min(k0 + per, nq) - k0;
  if (touched) {
    for (unsigned j = threadIdx.x; j < n; j += kPersistThreads) touched[k0 + j] = __ldcg(lst0 + k0 + j);
    if (blockIdx.x == 0 && threadIdx.x == 0) *touched_n = nq;
  }
  __shared__ int s_first[kPersistThreads];
  unsigned long long seen_even = 0, seen_odd = 0;
  for (int it = 0; it < iterations; it += 2) {
    if (!persistent_band_iteration(even, it, it + 1 == iterations, lst0 + k0, lst1 + k0, n, per, sync, limit_ns,
                                   s_first, seen_even))
      return;
    if (it + 1 < iterations && !persistent_band_iteration(odd, it + 1, it + 2 == iterations, lst1 + k0, lst0 + k0,
                                                          n, per, sync, limit_ns, s_first, seen_odd))
      return;
  }
}

// In-place update after the last iteration: psi(list[k]) = entry k of the
// band pass's output planes (the dense passes write back the others).
__global__ void __launch_bounds__(kThreads) k_fused_scatter(FusedArgs a, const int *__restrict__ list,
                                                           float *__restrict__ px, float *__restrict__ py,
                                                           float *__restrict__ pz) {
  if (iteration_gated(a.st, a.iter, a.dp)) return;
  const int nq = (int)a.st[a.iter].list;
  for (int k = blockIdx.x * kThreads + threadIdx.x; k < nq; k += gridDim.x * kThreads) {
    const int v = list[k];
    if (!KF_IN_BOUNDS(k, a.dp.count, KF_SITE_WRITE_BACK) || !KF_IN_BOUNDS(v, a.dp.count, KF_SITE_WRITE_BACK))
      continue;
    px[v] = a.ox[k];
    py[v] = a.oy[k];
    pz[v] = a.oz[k];
  }
}

// Trust-region step, after the band pass of iteration a.iter: the reference
// breaks out of a row's x loop at the first voxel whose step failed
// (KillingFusion.cpp:312-313), so listed voxels at or after that x (a.rows)
// get their old psi back in the output planes (entry k in place, voxel v
// ping-pong).  Also clears next_rows, the table of the next band pass.
__global__ void __launch_bounds__(kThreads) k_trust_fix(FusedArgs a, const int *__restrict__ list, bool in_place,
                                                       int *__restrict__ next_rows) {
  const int nrows = a.dp.ny * a.dp.nz;
  const int stride = gridDim.x * kThreads;
  const int t0 = blockIdx.x * kThreads + threadIdx.x;
  for (int r = t0; r < nrows; r += stride) next_rows[r] = kRowClear;
  if (a.st[a.iter].skipped) return;
  const int nq = (int)a.st[a.iter].list;
  for (int k = t0; k < nq; k += stride) {
    const int v = list[k];
    if (!KF_IN_BOUNDS(v, a.dp.count, KF_SITE_BAND_LIST)) continue;
    int x, y, z;
    voxel_xyz(a.dp, v, x, y, z);
    if (x >= a.rows[z * a.dp.ny + y]) {
      const int slot = in_place ? k : v;
      a.ox[slot] = a.ix[v];
      a.oy[slot] = a.iy[v];
      a.oz[slot] = a.iz[v];
    }
  }
}

// KillingFusion::computeDisplacementField, default per-voxel schedule
// (KillingFusion.cpp:353-396), for the listed voxels (inside the symmetric
// band) of one colour (x&1) | (y&1)<<1 | (z&1)<<2: each is taken by one
// thread, which steps its psi in place -- a.ix and a.ox are the same planes --
// until the step or the gradient is at most the threshold or max_iters steps
// were taken.  A voxel's gradient reads psi only in its 3x3x3 neighbourhood,
// where no other voxel has its colour, so its neighbours stay fixed while it
// iterates, as in the reference's sequential loop, and the result does not
// depend on scheduling.  Statistics: record 0 voxels (list, from the band
// pass), last step, last monitored energy, divergence; record 1 voxels that
// hit the cap (active) and the most steps of one voxel (list).
__global__ void __launch_bounds__(kLaneThreads, kLaneBlocksPerSM) k_pervoxel(FusedArgs a, const int *__restrict__ list,
                                                            int max_iters, int color) {
  const DevParams &dp = a.dp;
  const int nq = (int)a.st[0].list;
  const float thr = (float)dp.threshold;
  float maxd = 0.f;
  double energy = 0.0;  // float64 from the per-voxel terms up
  unsigned capped = 0, most = 0;
  bool diverged = false;
  for (int k = blockIdx.x * kLaneThreads + threadIdx.x; k < nq; k += gridDim.x * kLaneThreads) {
    const int i = list[k];
    if (!KF_IN_BOUNDS(i, dp.count, KF_SITE_BAND_LIST)) continue;
    int x, y, z;
    voxel_xyz(dp, i, x, y, z);
    if (((x & 1) | (y & 1) << 1 | (z & 1) << 2) != color) continue;
    const bool interior = x >= 1 && y >= 1 && z >= 1 && x <= dp.nx - 2 && y <= dp.ny - 2 && z <= dp.nz - 2;
    int iter = 0;
    unsigned steps = 0;
    float dn = 0.f, en = 0.f;
    bool div = false;
    while (true) {
      float d[3] = {0.f, 0.f, 0.f}, sv = 0.f, e = 0.f, c0[3] = {0.f, 0.f, 0.f};
      if (interior) {
        gradient_lane<kPsiL2>(a, x, y, z, i, d, sv, e, c0);
      } else {
        gradient_generic<kPsiL2>(a, x, y, z, d, sv, e);
        c0[0] = __ldcg(a.ix + i);
        c0[1] = __ldcg(a.iy + i);
        c0[2] = __ldcg(a.iz + i);
      }
      const float n0 = c0[0] + d[0], n1 = c0[1] + d[1], n2 = c0[2] + d[2];
      // DisplacementField::update (DisplacementField.cpp:65-71)
      a.ox[i] = n0;
      a.oy[i] = n1;
      a.oz[i] = n2;
      ++steps;
      dn = sqrtf(ff(d[2], d[2], ff(d[1], d[1], fm(d[0], d[0]))));
      en = e;
      if (dn <= thr) break;
      if (!isfinite(n0) || !isfinite(n1) || !isfinite(n2)) {
        div = true;
        break;
      }
      ++iter;
      // |gradient| = |step| / alpha
      if (!(dn / a.alpha > thr) || iter >= max_iters) break;
    }
    maxd = fmaxf(maxd, dn);
    energy += en;
    capped += iter >= max_iters;
    most = max(most, steps);
    diverged |= div;
  }
  // voxels processed are counted by the band pass (record 0's list)
  reduce_iter_stats<kLaneThreads>(a.st, 0u, maxd, energy, diverged);
  if (capped) atomicAdd(&a.st[1].active, capped);
  if (most) atomicMax(&a.st[1].list, most);
}

}  // namespace

// A captured iteration loop, valid for one set of buffers and parameters.
struct FusedGraph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
  cudaStream_t cold = nullptr;                     // cold passes of the split schedule
  cudaEvent_t fork = nullptr, join = nullptr;
  const void *key_ptr[12] = {};
  int iterations = 0;
  bool band_only = false;
  DevParams dp;
};

void kf_fused_graph_destroy(FusedGraph *g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->capture) cudaStreamDestroy(g->capture);
  if (g->cold) cudaStreamDestroy(g->cold);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->join) cudaEventDestroy(g->join);
  delete g;
}

static int64_t num_runs(const DevParams &dp) {
  return std::max<int64_t>((dp.count / 4 + kThreads * kFlatGroups - 1) / (kThreads * kFlatGroups), 1);
}

static bool split_schedule(const DevParams &dp, bool band_only) {
  return !band_only && !dp.trust && num_runs(dp) >= kSplitMinRuns;
}

// A launch whose graph node carries a priority: the hot chain of the split
// schedule (hot pass, band pass) goes ahead of the cold passes' CTAs.
template <typename... KArgs, typename... Args>
static void launch_prio(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, int prio,
                        Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = prio;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

// The split schedule's lists after the run table: hot runs, cold runs (one
// int per run each) and their two counts.
static size_t runs_table_bytes(int64_t nruns) {
  return (size_t)nruns * sizeof(int2) + ((size_t)2 * nruns + 4) * sizeof(int);
}

// The dense fused iterations on the split schedule (see k_split_runs).
static void launch_split_iterations(FusedArgs a, kf_field psi, const DevParams &dp, int iterations,
                                    int *lists, int2 *runs, cudaStream_t s, cudaStream_t cold_s,
                                    cudaEvent_t fork, cudaEvent_t join) {
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  // the cold passes rank between the hot chain and default-priority work
  // that a caller runs beside the solve (the next frame's integration,
  // meshes), where the device has more than two priority levels
  const int mid = hi < lo - 1 ? (lo + hi) / 2 : lo;
  const unsigned band_blocks = (unsigned)kf_num_sms() * kLaneBlocksPerSM;
  const int64_t nruns = num_runs(dp);
  const unsigned grid = (unsigned)nruns;
  const unsigned hot_grid = (unsigned)std::min<int64_t>(nruns, (int64_t)kf_num_sms() * kHotBlocksPerSM);
  int *hot = reinterpret_cast<int *>(runs + nruns), *cold = hot + nruns;
  unsigned *counts = reinterpret_cast<unsigned *>(cold + nruns);
  int *lst[2] = {lists, lists + dp.count};
  a.ix = (const float *)psi->p[0];
  a.iy = (const float *)psi->p[1];
  a.iz = (const float *)psi->p[2];
  a.ox = (float *)psi->q[0];
  a.oy = (float *)psi->q[1];
  a.oz = (float *)psi->q[2];
  for (int it = 0; it < iterations; ++it) {
    a.iter = it;
    if (it == 0) {
      launch_prio(k_fused_stream<false>, grid, kThreads, s, hi, a, lst[0], lst[1], runs);
      launch_prio(k_split_runs, 1, kSplitThreads, s, hi, (const int2 *)runs, (int)nruns, hot, cold, counts);
    } else {
      // cold runs beside the band pass of the iteration before
      cudaStreamWaitEvent(cold_s, fork, 0);
      launch_prio(k_fused_stream_runs<true>, grid, kThreads, cold_s, mid, a, (const int *)cold,
                  (const unsigned *)counts, (int *)nullptr, (const int *)nullptr, (int2 *)nullptr);
      launch_prio(k_fused_stream_runs<false>, hot_grid, kThreads, s, hi, a, (const int *)hot,
                  (const unsigned *)counts, lst[it & 1], (const int *)lst[(it + 1) & 1], runs);
    }
    if (it + 1 < iterations) cudaEventRecord(fork, s);
    launch_prio(k_fused_band<false, true>, band_blocks, kLaneThreads, s, hi, a, (const int *)lst[it & 1],
                (int *)nullptr);
    if (it == iterations - 1)
      launch_prio(k_fused_scatter, band_blocks, kThreads, s, hi, a, (const int *)lst[it & 1],
                  (float *)psi->p[0], (float *)psi->p[1], (float *)psi->p[2]);
  }
  if (iterations > 1) {
    cudaEventRecord(join, cold_s);
    cudaStreamWaitEvent(s, join, 0);
  }
}

static void launch_iterations(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                              int iterations, IterStats *st, int *lists, int2 *runs, int *rows,
                              bool band_only, cudaStream_t s) {
  const unsigned band_blocks = (unsigned)kf_num_sms() * kLaneBlocksPerSM;  // one resident wave
  const unsigned grid = (unsigned)std::max<int64_t>((dp.count / 4 + kThreads * kFlatGroups - 1) /
                                                        (kThreads * kFlatGroups), 1);
  const unsigned block = kThreads;
  FusedArgs a = make_args(live, can, dp, st);
  void *buf[2][3] = {{psi->p[0], psi->p[1], psi->p[2]}, {psi->q[0], psi->q[1], psi->q[2]}};
  int *lst[2] = {lists, lists + dp.count};
  const int nrows = dp.ny * dp.nz;
  if (dp.trust) cudaMemsetAsync(rows, 0x7f, (size_t)nrows * sizeof(int), s);
  for (int it = 0; it < iterations; ++it) {
    // dense: psi stays in the primary planes, the second planes hold the
    // band voxels' new values by list position; band-only: ping-pong
    void **in = band_only ? buf[it & 1] : buf[0], **out = band_only ? buf[(it + 1) & 1] : buf[1];
    a.ix = (const float *)in[0];
    a.iy = (const float *)in[1];
    a.iz = (const float *)in[2];
    a.ox = (float *)out[0];
    a.oy = (float *)out[1];
    a.oz = (float *)out[2];
    a.iter = it;
    a.rows = dp.trust ? rows + (it & 1) * nrows : nullptr;
    int *next_rows = dp.trust ? rows + ((it + 1) & 1) * nrows : nullptr;
    if (!band_only) {
      // lists alternate so that a run can still read the previous iteration's
      k_fused_stream<false><<<grid, block, 0, s>>>(a, lst[it & 1], lst[(it + 1) & 1], runs);
      if (dp.trust) {
        k_fused_band<false, true, true><<<band_blocks, kLaneThreads, 0, s>>>(a, lst[it & 1], nullptr);
        k_trust_fix<<<band_blocks, kThreads, 0, s>>>(a, lst[it & 1], true, next_rows);
      } else {
        k_fused_band<false, true><<<band_blocks, kLaneThreads, 0, s>>>(a, lst[it & 1], nullptr);
      }
      if (it == iterations - 1)
        k_fused_scatter<<<band_blocks, kThreads, 0, s>>>(a, lst[it & 1], (float *)in[0], (float *)in[1],
                                                        (float *)in[2]);
    } else {
      if (it == 0) k_fused_stream<true><<<grid, block, 0, s>>>(a, lst[0], nullptr, nullptr);
      if (dp.trust) {
        k_fused_band<true, false, true><<<band_blocks, kLaneThreads, 0, s>>>(a, lst[it & 1], lst[(it + 1) & 1]);
        k_trust_fix<<<band_blocks, kThreads, 0, s>>>(a, lst[it & 1], false, next_rows);
      } else {
        k_fused_band<true, false><<<band_blocks, kLaneThreads, 0, s>>>(a, lst[it & 1], lst[(it + 1) & 1]);
      }
    }
  }
}

// Resident blocks per SM of k_band_persistent on the current device (at most
// kPersistBlocksPerSM): the cooperative launch must fit on the GPU at once.
// Its shared-memory carveout is kBesideSolveCarveout (kf_internal.h), the
// one of the kernels that run beside it.
static int persistent_blocks_per_sm() {
  static int cached[64] = {};
  static bool carveout[64] = {};
  kf_prefer_carveout((const void *)k_band_persistent, kBesideSolveCarveout, carveout);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (!cached[dev]) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_band_persistent, kPersistThreads, 0) !=
        cudaSuccess)
      return 0;
    cached[dev] = std::min(n, kPersistBlocksPerSM);
  }
  return cached[dev];
}

// KF_SOLVER_BAND without the trust-region step: the dense first pass (on
// phi_live alone when both buffers are zero), then every band pass in one
// cooperative launch (k_band_persistent).  Iteration k reads buffer k % 2
// and writes (k + 1) % 2, as the per-iteration form.  From a zero p the
// first pass leaves both buffers zero outside its list (it copies p to q),
// and the solve records the list: the field's buffers are then zero outside
// its records (kf_field_zero clears just those).
static int launch_band_persistent(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                                  int iterations, IterStats *st, bool p_zero, bool q_zero, cudaStream_t s) {
  void *sync = nullptr;
  int rc = kf_field_sync(psi, &sync);
  if (rc) return rc;
  const int bps = persistent_blocks_per_sm();
  if (bps < 1) return kf_fail(KF_ERR_CUDA, "the persistent band pass does not fit on an SM");
  KF_CHECK_CUDA(cudaMemsetAsync(sync, 0, sizeof(GridSync), s));
  FusedArgs even = make_args(live, can, dp, st);
  even.ix = (const float *)psi->p[0];
  even.iy = (const float *)psi->p[1];
  even.iz = (const float *)psi->p[2];
  even.ox = (float *)psi->q[0];
  even.oy = (float *)psi->q[1];
  even.oz = (float *)psi->q[2];
  FusedArgs odd = even;
  odd.ix = (const float *)psi->q[0];
  odd.iy = (const float *)psi->q[1];
  odd.iz = (const float *)psi->q[2];
  odd.ox = (float *)psi->p[0];
  odd.oy = (float *)psi->p[1];
  odd.oz = (float *)psi->p[2];
  int *lst0 = psi->band, *lst1 = psi->band + dp.count;
  int *touched = nullptr;
  unsigned *touched_n = nullptr;
  if (p_zero) {
    KfRecords r;
    rc = kf_field_records(psi, s, &r);
    if (rc) return rc;
    KF_CHECK_CUDA(cudaMemsetAsync(r.side_n, 0, sizeof(unsigned), s));
    touched = r.touched;
    touched_n = r.touched_n;
  }
  if (p_zero && q_zero)
    k_band_first_zero<<<(unsigned)num_runs(dp), kThreads, 0, s>>>(even, lst0);
  else
    k_fused_stream<true><<<(unsigned)num_runs(dp), kThreads, 0, s>>>(even, lst0, nullptr, nullptr);
  KF_CHECK_LAUNCH("dense first pass of the band-only solver");
  GridSync *gs = static_cast<GridSync *>(sync);
  unsigned long long limit = kf_wait_limit_ns();
  int iters = iterations;
  void *args[] = {&even, &odd, &lst0, &lst1, &iters, &gs, &limit, &touched, &touched_n};
  KF_CHECK_CUDA(cudaLaunchCooperativeKernel((const void *)k_band_persistent,
                                            dim3((unsigned)(kf_num_sms() * bps)), dim3(kPersistThreads), args, 0,
                                            s));
  if (p_zero) {
    psi->p_state = psi->q_state = kPsiRecorded;
    psi->side_recorded = false;
  }
  return KF_OK;
}

int kf_solve_fused(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, int iterations,
                   IterStats *st, bool band_only, bool p_zero, bool q_zero, cudaStream_t s) {
  int rc = kf_field_ensure_pair(psi);
  if (rc) return rc;
  rc = kf_field_band_list(psi, &psi->band);
  if (rc) return rc;
  const int64_t nruns = num_runs(dp);
  if (psi->runs_cap < nruns) {
    cudaFree(psi->runs);
    psi->runs = nullptr;
    psi->runs_cap = 0;
    if (cudaMalloc(&psi->runs, runs_table_bytes(nruns)) != cudaSuccess) {
      cudaGetLastError();
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the dense pass's run table failed");
    }
    psi->runs_cap = nruns;
  }
  if (band_only && !dp.trust) return launch_band_persistent(live, can, psi, dp, iterations, st, p_zero, q_zero, s);
  int *rows = nullptr;
  if (dp.trust) {
    rc = kf_field_trust_rows(psi, &rows);
    if (rc) return rc;
  }
  const void *key[12] = {live->phi, can->phi, psi->p[0], psi->p[1], psi->p[2],
                         psi->q[0], psi->q[1], psi->q[2], st, psi->band, psi->runs, rows};
  FusedGraph *g = psi->graph;
  bool hit = g && g->iterations == iterations && g->band_only == band_only &&
             memcmp(g->key_ptr, key, sizeof(key)) == 0 && memcmp(&g->dp, &dp, sizeof(dp)) == 0;
  if (!hit) {
    kf_fused_graph_destroy(psi->graph);
    psi->graph = g = new FusedGraph();
    KF_CHECK_CUDA(cudaStreamCreateWithFlags(&g->capture, cudaStreamNonBlocking));
    const bool split = split_schedule(dp, band_only);
    if (split) {
      KF_CHECK_CUDA(cudaStreamCreateWithFlags(&g->cold, cudaStreamNonBlocking));
      KF_CHECK_CUDA(cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming));
      KF_CHECK_CUDA(cudaEventCreateWithFlags(&g->join, cudaEventDisableTiming));
    }
    cudaGraph_t graph;
    KF_CHECK_CUDA(cudaStreamBeginCapture(g->capture, cudaStreamCaptureModeThreadLocal));
    if (split)
      launch_split_iterations(make_args(live, can, dp, st), psi, dp, iterations, psi->band, psi->runs,
                              g->capture, g->cold, g->fork, g->join);
    else
      launch_iterations(live, can, psi, dp, iterations, st, psi->band, psi->runs, rows, band_only,
                        g->capture);
    cudaError_t le = cudaGetLastError();
    KF_CHECK_CUDA(cudaStreamEndCapture(g->capture, &graph));
    if (le != cudaSuccess) {
      cudaGraphDestroy(graph);
      return kf_cuda_fail(le, "fused kernel launch during capture");
    }
    cudaError_t ie = cudaGraphInstantiateWithFlags(&g->exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return kf_cuda_fail(ie, "cudaGraphInstantiate");
    g->iterations = iterations;
    g->band_only = band_only;
    memcpy(g->key_ptr, key, sizeof(key));
    g->dp = dp;
  }
  KF_CHECK_CUDA(cudaGraphLaunch(g->exec, s));
  return KF_OK;
}

int kf_solve_pervoxel(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, int max_iters,
                      IterStats *st, cudaStream_t s) {
  int rc = kf_field_band_list(psi, &psi->band);
  if (rc) return rc;
  // the symmetric band of KillingFusion.cpp:369 and psi read and written in
  // place
  DevParams pd = dp;
  pd.early_exit = 0;
  pd.trust = 0;  // the per-voxel schedule has no trust-region step
  FusedArgs a = make_args(live, can, pd, st);
  a.band_lo = dp.pv_lo_f;
  a.ix = (const float *)psi->p[0];
  a.iy = (const float *)psi->p[1];
  a.iz = (const float *)psi->p[2];
  a.ox = (float *)psi->p[0];
  a.oy = (float *)psi->p[1];
  a.oz = (float *)psi->p[2];
  a.iter = 0;
  const unsigned grid = (unsigned)std::max<int64_t>((dp.count / 4 + kThreads * kFlatGroups - 1) /
                                                        (kThreads * kFlatGroups), 1);
  k_fused_stream<false><<<grid, kThreads, 0, s>>>(a, psi->band, nullptr, nullptr);
  for (int color = 0; color < 8; ++color)
    k_pervoxel<<<(unsigned)kf_num_sms() * kLaneBlocksPerSM, kLaneThreads, 0, s>>>(a, psi->band, max_iters, color);
  KF_CHECK_LAUNCH("per-voxel solve");
  return KF_OK;
}


KF_BOUNDS_TU_API(fused)
