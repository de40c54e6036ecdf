// Batched psi solves: many independent registration problems (each a live
// SDF, a canonical SDF and psi, of its own size and parameters) advanced
// together, every iteration of all of them in one persistent launch.
//
// The reference registers one frame at a time (KillingFusion::processNextFrame,
// KillingFusion.cpp:109-175); a batch runs its Jacobi schedule
// (KillingFusion.cpp:248-352) on every problem of the set with the band-only
// fused iteration of kf_fused.cu, so each problem's psi equals what
// kf_psi_solve(KF_SOLVER_BAND) gives it alone, bit for bit:
//   k_batch_stream      the dense first pass over every tile of every problem
//                       (one flat grid; a block finds its problem by binary
//                       search over the tile prefix) building each problem's
//                       band list;
//   k_batch_persistent  every band pass of every iteration, one cooperative
//                       launch: per iteration the band voxels of all problems
//                       are one work list cut into chunks that never cross a
//                       problem; a block scans the per-problem chunk counts
//                       into a prefix, finds each chunk's problem and hands
//                       each thread its voxels; statistics stay in registers
//                       while the block works on one problem, are
//                       warp-reduced into that problem's shared totals when
//                       it moves on, and are flushed once per block and
//                       iteration.  The iterations are separated by a
//                       grid-wide barrier with a bounded wait
//                       (kf_grid_sync.cuh).
// Each problem converges on its own (params.early_exit): once its previous
// iteration moved psi by at most params.threshold it is skipped, and its
// voxels are no longer listed; the launch ends when every problem is.
//
// Launch shapes (kf_batch_autotune): the band pass's CTA size (256 or 512
// threads), chunk size (one or two voxels per thread) and resident CTAs per
// SM (the register budget), and the dense pass's slab depth (4, 8 or 16
// z-planes per tile).
#include <algorithm>
#include <vector>

#include "kf_fused_body.cuh"
#include "kf_grid_sync.cuh"

namespace {

constexpr int kMaxBatch = 256;  // one problem per thread in the count scan (CTAs of >= 256)

// One problem of the batch on the device: the argument blocks of the two
// ping-pong parities, its band lists and its dense-pass tiling.
struct BatchEntry {
  FusedArgs a[2];
  int *band;  // two lists of `count` ints
  int64_t count;
  int gx, gy;  // dense-pass tiles along x and y
};

__device__ __forceinline__ int find_problem(const int64_t *pre, int n, int64_t k) {
  int lo = 0, hi = n;  // pre[lo] <= k < pre[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(pre + mid) <= k)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// tile_pre: the tiles of kSlab z-planes before each problem.
template <int kSlab>
__global__ void __launch_bounds__(kThreads) k_batch_stream(const BatchEntry *__restrict__ tab,
                                                          const int64_t *__restrict__ tile_pre, int nprob) {
  const int64_t b = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
  if (b >= __ldg(tile_pre + nprob)) return;
  const int p = find_problem(tile_pre, nprob, b);
  const BatchEntry &e = tab[p];
  const int64_t local = b - __ldg(tile_pre + p);
  const int bx = (int)(local % e.gx);
  const int by = (int)((local / e.gx) % e.gy);
  const int bz = (int)(local / ((int64_t)e.gx * e.gy));
  stream_tile<true, kSlab>(e.a[0], bx, by, bz, e.band, &e.a[0].st[0].list);
}

// exclusive prefix of cnt[0..n) into pre[0..n], n <= kMaxBatch <= blockDim.x
template <int kT>
__device__ void scan_counts(const unsigned *cnt, unsigned *pre, int n) {
  __shared__ unsigned s_warp[kT / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned v = t < n ? cnt[t] : 0u;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned s = lane < kT / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kT / 32) s_warp[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  const unsigned off = w > 0 ? s_warp[w - 1] : 0u;
  if (t < n) pre[t] = off + x - v;
  if (t == n - 1) pre[n] = off + x;
  __syncthreads();
}

__device__ __forceinline__ int find_work(const unsigned *pre, int n, unsigned k) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (pre[mid] <= k)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Band pass of iteration `it` over all problems, by every block of the grid.
// The work is cut into chunks of kT * kVpt voxels that never cross a
// problem, so a CTA works on one problem at a time: it stages that problem's
// argument block in shared memory (the gradient reads it as often as the
// single-grid kernel reads its constant parameters) and appends each round's
// carried voxels with one atomic.  Returns false when every problem was
// skipped (converged or diverged): nothing is left to run.
template <int kT, int kVpt>
__device__ __forceinline__ bool batch_band_pass(const BatchEntry *__restrict__ tab, int nprob, int it) {
  __shared__ unsigned s_cnt[kMaxBatch];
  __shared__ unsigned s_pre[kMaxBatch + 1];
  __shared__ unsigned s_active[kMaxBatch];
  __shared__ unsigned s_maxd[kMaxBatch];
  __shared__ double s_energy[kMaxBatch];
  __shared__ int s_div[kMaxBatch];
  __shared__ unsigned s_chunks[kMaxBatch];
  __shared__ FusedArgs s_a;
  __shared__ int *s_list_in, *s_list_out;
  __shared__ int s_live;  // problems not skipped this iteration
  constexpr int kChunk = kT * kVpt;
  const int par = it & 1;
  if (threadIdx.x == 0) s_live = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < nprob; q += blockDim.x) {
    const FusedArgs &a = tab[q].a[par];
    const bool gated = iteration_gated(a.st, it, a.dp);
    if (gated && blockIdx.x == 0) a.st[it].skipped = 1;
    if (!gated) atomicAdd(&s_live, 1);
    s_cnt[q] = gated ? 0u : __ldcg(&a.st[it].list);
    s_active[q] = 0u;
    s_maxd[q] = 0u;
    s_energy[q] = 0.0;
    s_div[q] = 0;
  }
  __syncthreads();
  if (s_live == 0) return false;
  // chunks per problem, scanned
  if (threadIdx.x < nprob) s_chunks[threadIdx.x] = (s_cnt[threadIdx.x] + kChunk - 1) / kChunk;
  __syncthreads();
  scan_counts<kT>(s_chunks, s_pre, nprob);
  const unsigned total = s_pre[nprob];
  const int lane = threadIdx.x & 31;
  // statistics of the staged problem, per thread until the problem changes
  float maxd = 0.f;
  double energy = 0.0;  // float64 from the per-voxel terms up
  unsigned active = 0;
  bool diverged = false;
  // warp sums into the problem's shared totals (c, hence p, is the same in
  // every thread of the block, so every warp reaches this together)
  auto flush = [&](int q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      energy += __shfl_xor_sync(0xffffffffu, energy, o);
      maxd = fmaxf(maxd, __shfl_xor_sync(0xffffffffu, maxd, o));
      active += __shfl_xor_sync(0xffffffffu, active, o);
    }
    const bool any_div = __any_sync(0xffffffffu, diverged);
    if (lane == 0) {
      if (active) {
        atomicAdd(&s_active[q], active);
        atomicMax(&s_maxd[q], __float_as_uint(maxd));
        atomicAdd(&s_energy[q], energy);
      }
      if (any_div) s_div[q] = 1;
    }
    maxd = 0.f;
    energy = 0.0;
    active = 0;
    diverged = false;
  };
  int cur = -1;  // problem staged in s_a (the same in every thread)
  for (unsigned c = blockIdx.x; c < total; c += gridDim.x) {
    const int p = find_work(s_pre, nprob, c);
    if (p != cur) {
      if (cur >= 0) flush(cur);
      __syncthreads();  // the previous problem's arguments are no longer read
      const int *src = reinterpret_cast<const int *>(&tab[p].a[par]);
      int *dst = reinterpret_cast<int *>(&s_a);
      for (int w = threadIdx.x; w < (int)(sizeof(FusedArgs) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
      if (threadIdx.x == 0) {
        s_list_in = tab[p].band + (par ? tab[p].count : 0);
        s_list_out = tab[p].band + (par ? 0 : tab[p].count);
      }
      cur = p;
      __syncthreads();
    }
#pragma unroll 1
    for (int v = 0; v < kVpt; ++v) {
      const unsigned k = (c - s_pre[p]) * kChunk + v * kT + threadIdx.x;
      int next = -1;
      if (k < s_cnt[p]) {
        const int i = __ldcg(s_list_in + k);
        next = update_band_voxel<false, kPsiL1>(s_a, i, i, maxd, energy, active, diverged);
      }
      // hand the round's updated voxels to the next iteration
      block_append<kT / 32>(next, &s_a.st[it + 1].list, s_list_out, s_a.dp.count);
    }
  }
  if (cur >= 0) flush(cur);
  __syncthreads();
  for (int q = threadIdx.x; q < nprob; q += blockDim.x) {
    IterStats *st = tab[q].a[par].st + it;
    if (s_active[q]) {
      atomicAdd(&st->active, s_active[q]);
      atomicMax(&st->max_delta, s_maxd[q]);
      atomicAdd(&st->energy, s_energy[q]);
    }
    if (s_div[q]) st->diverged = 1;
  }
  return true;
}

// Every band pass of the batch: `iterations` passes separated by grid-wide
// barriers.  A wait that gives up marks problem 0's first record
// (IterStats::timeout) and ends the kernel.
template <int kT, int kVpt, int kMinBlocks>
__global__ void __launch_bounds__(kT, kMinBlocks)
    k_batch_persistent(const BatchEntry *__restrict__ tab, int nprob, int iterations, GridSync *sync,
                       unsigned long long limit_ns) {
  for (int it = 0; it < iterations; ++it) {
    if (!batch_band_pass<kT, kVpt>(tab, nprob, it) || it + 1 == iterations) return;
    if (!grid_sync(sync, gridDim.x, limit_ns, it)) {
      if (threadIdx.x == 0) tab[0].a[0].st[0].timeout = 1;
      return;
    }
  }
}

// The band-pass shapes the autotuner tries: CTA threads, voxels per thread
// of a chunk, resident CTAs per SM (sets the register budget), registers.
struct BandShape {
  int threads, vpt, min_blocks, regs;
  const void *kernel;
};

const BandShape kBandShapes[] = {
    {256, 1, 2, 128, (const void *)k_batch_persistent<256, 1, 2>},
    {256, 1, 3, 80, (const void *)k_batch_persistent<256, 1, 3>},
    {256, 2, 2, 128, (const void *)k_batch_persistent<256, 2, 2>},
    {256, 2, 3, 80, (const void *)k_batch_persistent<256, 2, 3>},
    {512, 1, 1, 128, (const void *)k_batch_persistent<512, 1, 1>},
    {512, 2, 1, 128, (const void *)k_batch_persistent<512, 2, 1>},
};
constexpr int kNumBandShapes = sizeof(kBandShapes) / sizeof(kBandShapes[0]);
// dense-pass slab depths (z-planes per tile of 32 x 8 columns)
const int kSlabs[] = {4, 8, 16};
constexpr int kNumSlabs = 3;

}  // namespace

struct kf_batch_s {
  std::vector<kf_batch_item> items;
  int iterations = 0;
  int band_shape = 0;                     // index into kBandShapes
  int slab_index = 1;                     // index into kSlabs
  double band_ms = 0.0, stream_ms = 0.0;  // autotuned times of the choice
  int resident[kNumBandShapes] = {};      // CTAs per SM each shape can keep resident
  BatchEntry *tab = nullptr;              // device
  BatchEntry *tab_host = nullptr;         // pinned
  int64_t *tile_pre = nullptr;            // device, kNumSlabs x (nprob + 1)
  int64_t tiles[kNumSlabs] = {};
  IterStats *stats = nullptr;       // device, nprob * (iterations + 1)
  IterStats *stats_host = nullptr;  // pinned
  GridSync *sync = nullptr;         // device
};

static void batch_free(kf_batch b) {
  if (!b) return;
  cudaFree(b->tab);
  cudaFreeHost(b->tab_host);
  cudaFree(b->tile_pre);
  cudaFree(b->stats);
  cudaFreeHost(b->stats_host);
  cudaFree(b->sync);
  delete b;
}

static int stats_stride(kf_batch b) { return b->iterations + 1; }

// Refreshes the argument table from the fields' current buffers.
static int batch_upload_table(kf_batch b, cudaStream_t s) {
  const int n = (int)b->items.size();
  for (int p = 0; p < n; ++p) {
    const kf_batch_item &it = b->items[p];
    kf_field_written(it.psi);  // the batch's passes write both planes
    DevParams dp = kf_make_dev_params(it.live->n, &it.params);
    BatchEntry &e = b->tab_host[p];
    IterStats *st = b->stats + (int64_t)p * stats_stride(b);
    void *buf[2][3] = {{it.psi->p[0], it.psi->p[1], it.psi->p[2]}, {it.psi->q[0], it.psi->q[1], it.psi->q[2]}};
    for (int par = 0; par < 2; ++par) {
      FusedArgs a = make_args(it.live, it.canonical, dp, st);
      a.ix = (const float *)buf[par][0];
      a.iy = (const float *)buf[par][1];
      a.iz = (const float *)buf[par][2];
      a.ox = (float *)buf[par ^ 1][0];
      a.oy = (float *)buf[par ^ 1][1];
      a.oz = (float *)buf[par ^ 1][2];
      e.a[par] = a;
    }
    e.band = it.psi->band;
    e.count = it.psi->count;
    e.gx = (dp.nx + kTX - 1) / kTX;
    e.gy = (dp.ny + kTY - 1) / kTY;
  }
  KF_CHECK_CUDA(cudaMemcpyAsync(b->tab, b->tab_host, sizeof(BatchEntry) * n, cudaMemcpyHostToDevice, s));
  return KF_OK;
}

// The dense first pass with slab depth kSlabs[si].
static int stream_launch(kf_batch b, int si, cudaStream_t s) {
  const int n = (int)b->items.size();
  const int64_t tiles = b->tiles[si];
  const int64_t *pre = b->tile_pre + (int64_t)si * (n + 1);
  const dim3 grid((unsigned)std::min<int64_t>(tiles, 65535), (unsigned)((tiles + 65534) / 65535));
  const dim3 block(kTX, kTY);
  if (kSlabs[si] == 4)
    k_batch_stream<4><<<grid, block, 0, s>>>(b->tab, pre, n);
  else if (kSlabs[si] == 8)
    k_batch_stream<8><<<grid, block, 0, s>>>(b->tab, pre, n);
  else
    k_batch_stream<16><<<grid, block, 0, s>>>(b->tab, pre, n);
  KF_CHECK_LAUNCH("k_batch_stream");
  return KF_OK;
}

// `iterations` band passes in one cooperative launch of shape kBandShapes[sh].
static int band_launch(kf_batch b, int sh, int iterations, cudaStream_t s) {
  const BandShape &bs = kBandShapes[sh];
  const int resident = std::min(b->resident[sh], bs.min_blocks);
  if (resident < 1) return kf_fail(KF_ERR_CUDA, "a batch band-pass shape does not fit on an SM");
  KF_CHECK_CUDA(cudaMemsetAsync(b->sync, 0, sizeof(GridSync), s));
  const BatchEntry *tab = b->tab;
  int nprob = (int)b->items.size();
  GridSync *sync = b->sync;
  unsigned long long limit = kf_wait_limit_ns();
  void *args[] = {&tab, &nprob, &iterations, &sync, &limit};
  KF_CHECK_CUDA(cudaLaunchCooperativeKernel(bs.kernel, dim3((unsigned)(kf_num_sms() * resident)),
                                            dim3((unsigned)bs.threads), args, 0, s));
  return KF_OK;
}

extern "C" int kf_batch_create(const kf_batch_item *items, int count, int iterations, kf_batch *out) {
  KF_REQUIRE(out, "NULL output");
  *out = nullptr;
  KF_REQUIRE(items && count > 0, "empty batch");
  KF_REQUIRE(count <= kMaxBatch, "too many problems in one batch (at most 256)");
  KF_REQUIRE(iterations > 0, "iterations must be positive");
  for (int p = 0; p < count; ++p) {
    const kf_batch_item &it = items[p];
    KF_REQUIRE(it.live && it.canonical && it.psi, "NULL handle in a batch item");
    KF_REQUIRE(it.live != it.canonical, "live and canonical must differ");
    for (int k = 0; k < 3; ++k)
      KF_REQUIRE(it.live->n[k] == it.canonical->n[k] && it.live->n[k] == it.psi->n[k],
                 "grid and field sizes differ within a batch item");
    KF_REQUIRE(it.psi->prec == KF_F32, "batched solves run on KF_F32 fields");
    KF_REQUIRE(it.live->count <= 0x7fffffff, "grid too large for a batch item");
    int rc = kf_check_params(&it.params);
    if (rc) return rc;
    KF_REQUIRE(!kf_make_dev_params(it.live->n, &it.params).trust,
               "batched solves have no trust-region step (use_trust with the data term alone)");
    for (int q = 0; q < p; ++q) KF_REQUIRE(items[q].psi != it.psi, "a field appears twice in a batch");
  }
  kf_batch b = new kf_batch_s();
  b->items.assign(items, items + count);
  b->iterations = iterations;
  std::vector<int64_t> pre((size_t)kNumSlabs * (count + 1), 0);
  for (int si = 0; si < kNumSlabs; ++si) {
    int64_t *pr = pre.data() + (size_t)si * (count + 1);
    for (int p = 0; p < count; ++p) {
      const int *n = items[p].live->n;
      pr[p + 1] = pr[p] + (int64_t)((n[0] + kTX - 1) / kTX) * ((n[1] + kTY - 1) / kTY) *
                              ((n[2] + kSlabs[si] - 1) / kSlabs[si]);
    }
    b->tiles[si] = pr[count];
  }
  const size_t nst = (size_t)count * stats_stride(b);
  cudaError_t e = cudaMalloc(&b->tab, sizeof(BatchEntry) * count);
  if (e == cudaSuccess) e = cudaMallocHost(&b->tab_host, sizeof(BatchEntry) * count);
  if (e == cudaSuccess) e = cudaMalloc(&b->tile_pre, sizeof(int64_t) * pre.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->stats, sizeof(IterStats) * nst);
  if (e == cudaSuccess) e = cudaMallocHost(&b->stats_host, sizeof(IterStats) * nst);
  if (e == cudaSuccess) e = cudaMalloc(&b->sync, sizeof(GridSync));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->tile_pre, pre.data(), sizeof(int64_t) * pre.size(), cudaMemcpyHostToDevice);
  for (int sh = 0; sh < kNumBandShapes && e == cudaSuccess; ++sh)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b->resident[sh], kBandShapes[sh].kernel,
                                                      kBandShapes[sh].threads, 0);
  if (e != cudaSuccess) {
    batch_free(b);
    cudaGetLastError();
    return kf_cuda_fail(e, "kf_batch_create");
  }
  for (int p = 0; p < count; ++p) {
    int rc = kf_field_ensure_pair(items[p].psi);
    if (!rc) rc = kf_field_band_list(items[p].psi, &items[p].psi->band);
    if (rc) {
      batch_free(b);
      return rc;
    }
  }
  *out = b;
  return KF_OK;
}

extern "C" int kf_batch_destroy(kf_batch b) {
  if (b) cudaDeviceSynchronize();
  batch_free(b);
  return KF_OK;
}

// The dense pass and the band passes into the ping-pong buffers and the
// statistics; which buffer holds each field's psi is settled by the caller
// from the statistics.
static int batch_execute(kf_batch b, int iterations, cudaStream_t s) {
  const int n = (int)b->items.size();
  int rc = batch_upload_table(b, s);
  if (rc) return rc;
  KF_CHECK_CUDA(cudaMemsetAsync(b->stats, 0, sizeof(IterStats) * (size_t)n * stats_stride(b), s));
  rc = stream_launch(b, b->slab_index, s);
  if (rc) return rc;
  return band_launch(b, b->band_shape, iterations, s);
}

static bool shape_index(const kf_batch_shape *sh, int *band, int *slab) {
  *band = *slab = -1;
  for (int k = 0; k < kNumBandShapes; ++k)
    if (kBandShapes[k].threads == sh->band_threads &&
        kBandShapes[k].threads * kBandShapes[k].vpt == sh->band_chunk &&
        kBandShapes[k].min_blocks == sh->band_blocks_per_sm && kBandShapes[k].regs == sh->band_registers)
      *band = k;
  for (int k = 0; k < kNumSlabs; ++k)
    if (kSlabs[k] == sh->slab) *slab = k;
  return *band >= 0 && *slab >= 0;
}

static void shape_of(kf_batch b, kf_batch_shape *out) {
  const BandShape &bs = kBandShapes[b->band_shape];
  memset(out, 0, sizeof(*out));
  out->band_threads = bs.threads;
  out->band_chunk = bs.threads * bs.vpt;
  out->band_blocks_per_sm = bs.min_blocks;
  out->band_registers = bs.regs;
  out->slab = kSlabs[b->slab_index];
  out->band_ms = b->band_ms;
  out->stream_ms = b->stream_ms;
}

extern "C" int kf_batch_set_shape(kf_batch b, const kf_batch_shape *shape) {
  KF_REQUIRE(b && shape, "NULL argument");
  int band, slab;
  KF_REQUIRE(shape_index(shape, &band, &slab), "not a batch launch shape (see kf_batch_shape)");
  KF_REQUIRE(b->resident[band] >= kBandShapes[band].min_blocks, "that band-pass shape does not fit on this GPU");
  b->band_shape = band;
  b->slab_index = slab;
  b->band_ms = b->stream_ms = 0.0;
  return KF_OK;
}

// Times the dense first pass at each slab depth, then the band pass of the
// first iteration (the longest band lists) at each band shape, and keeps the
// fastest of each.  Every trial reruns the dense first pass, which reads psi
// and writes only the second ping-pong buffer, and at most one band pass,
// which writes only the second buffer too, so the fields keep their psi.
extern "C" int kf_batch_autotune(kf_batch b, kf_batch_shape *shape, void *stream) {
  KF_REQUIRE(b, "NULL batch");
  cudaStream_t s = kf_stream(stream);
  const int n = (int)b->items.size();
  int rc = batch_upload_table(b, s);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  KF_CHECK_CUDA(cudaEventCreate(&e0));
  KF_CHECK_CUDA(cudaEventCreate(&e1));
  const size_t stats_bytes = sizeof(IterStats) * (size_t)n * stats_stride(b);
  // one trial: the dense pass at slab si, then (sh >= 0) one band pass of
  // shape sh; the time of the dense pass (sh < 0) or of the band pass, the
  // best of repetitions 1..3 (repetition 0 warms up)
  auto trial = [&](int si, int sh, float *best) -> int {
    *best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
      KF_CHECK_CUDA(cudaMemsetAsync(b->stats, 0, stats_bytes, s));
      if (sh < 0) KF_CHECK_CUDA(cudaEventRecord(e0, s));
      int r = stream_launch(b, si, s);
      if (r) return r;
      if (sh >= 0) {
        KF_CHECK_CUDA(cudaEventRecord(e0, s));
        r = band_launch(b, sh, 1, s);
        if (r) return r;
      }
      KF_CHECK_CUDA(cudaEventRecord(e1, s));
      KF_CHECK_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      KF_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep == 1 || (rep > 1 && ms < *best)) *best = ms;
    }
    return KF_OK;
  };
  float best_stream = 0.f, best_band = 0.f;
  int si_best = -1, sh_best = -1;
  for (int si = 0; si < kNumSlabs && rc == KF_OK; ++si) {
    float t = 0.f;
    rc = trial(si, -1, &t);
    if (rc == KF_OK && (si_best < 0 || t < best_stream)) {
      best_stream = t;
      si_best = si;
    }
  }
  for (int sh = 0; sh < kNumBandShapes && rc == KF_OK; ++sh) {
    if (b->resident[sh] < kBandShapes[sh].min_blocks) continue;
    float t = 0.f;
    rc = trial(si_best, sh, &t);
    if (rc == KF_OK && (sh_best < 0 || t < best_band)) {
      best_band = t;
      sh_best = sh;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (sh_best < 0) return kf_fail(KF_ERR_CUDA, "no batch band-pass shape fits on this GPU");
  b->band_shape = sh_best;
  b->slab_index = si_best;
  b->band_ms = best_band;
  b->stream_ms = best_stream;
  if (shape) shape_of(b, shape);
  return KF_OK;
}

extern "C" int kf_batch_run(kf_batch b, kf_solve_stats *stats, void *stream) {
  KF_REQUIRE(b, "NULL batch");
  const int n = (int)b->items.size();
  const int iters = b->iterations;
  cudaStream_t s = kf_stream(stream);
  cudaEvent_t e0, e1;
  KF_CHECK_CUDA(cudaEventCreate(&e0));
  KF_CHECK_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  int rc = batch_execute(b, iters, s);
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  cudaEventRecord(e1, s);
  const size_t nst = (size_t)n * stats_stride(b);
  cudaError_t e = cudaMemcpyAsync(b->stats_host, b->stats, sizeof(IterStats) * nst, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return kf_cuda_fail(e, "kf_batch_run");
  if (b->stats_host[0].timeout)
    return kf_fail(KF_ERR_TIMEOUT, "a grid-wide wait of the batched band pass gave up; psi is undefined");
  int any_diverged = 0;
  for (int p = 0; p < n; ++p) {
    const IterStats *h = b->stats_host + (size_t)p * stats_stride(b);
    int executed = 0, diverged = 0;
    for (int k = 0; k < iters; ++k) {
      if (h[k].skipped) break;
      ++executed;
      if (h[k].diverged) {
        diverged = 1;
        break;
      }
    }
    kf_field f = b->items[p].psi;
    if (executed & 1)
      for (int k = 0; k < 3; ++k) std::swap(f->p[k], f->q[k]);
    any_diverged |= diverged;
    if (stats) {
      kf_solve_stats &o = stats[p];
      memset(&o, 0, sizeof(o));
      o.iterations_run = executed;
      o.converged = (!diverged && executed < iters) ? 1 : 0;
      o.diverged = diverged;
      if (executed > 0) {
        o.active_first = h[0].active;
        o.active_last = h[executed - 1].active;
        o.energy_first = h[0].energy;
        o.energy_last = h[executed - 1].energy;
        float md;
        unsigned bits = h[executed - 1].max_delta;
        memcpy(&md, &bits, sizeof(md));
        o.max_delta_last = md;
      }
      o.device_ms = ms;
    }
  }
  if (any_diverged) return kf_fail(KF_ERR_DIVERGED, "a problem of the batch diverged (see its statistics)");
  return KF_OK;
}

KF_BOUNDS_TU_API(batch)
