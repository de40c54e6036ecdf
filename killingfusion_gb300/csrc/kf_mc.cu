// Marching cubes in the reference's order (SDF::getMesh, SDF.cpp:396-414;
// ProcessVolumeCell, SDF.cpp:330-378; Polygonise, MarchingCubes.h:366-422).
//
// The triangle soup keeps the reference's order (cells in z, y, x order;
// triangles of a cell in table order): every cell writes its triangles at
// its block's offset plus the triangles of the block's earlier cells.
//
// kf_mc_run (grids the library owns), two passes:
//   1. k_mc_count_list: independent warps stream warp blocks of kWarpCells
//      cells through shared memory (cp.async), classify them and list every
//      cell with triangles: its index, configuration and offset in the warp
//      block.  Warp-block totals are stored and added into the totals of the
//      blocks of kCellsPerBlock cells; the last CTA to finish turns those
//      into offsets.
//   2. k_mc_emit_cells: one thread per listed cell writes its triangles.
//      When a grid has more such cells than the list holds, it falls back
//      to re-classifying every block with triangles (emit_block).
// kf_marching_cubes_noalloc, three passes over caller memory:
//   1. k_mc_count: each CTA classifies a block and writes its total;
//   2. k_mc_scan:  one CTA turns the totals into exclusive offsets, a chunk
//      of kScanChunk totals at a time through registers;
//   3. k_mc_emit:  each CTA re-classifies its block round by round (thread t
//      takes cell r*kThreads + t of round r, so the reads coalesce), scans
//      the round's triangle counts and writes every triangle at its final
//      position.
// A cell whose own value is outside [lo, hi] is skipped after one read
// (SDF.cpp:407), before any index arithmetic; only the band cells gather
// their corners.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "kf_bounds.cuh"
#include "kf_internal.h"
#include "kf_mc_tables.h"

namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 8;
constexpr int kCellsPerBlock = kThreads * kRounds;
constexpr int kCountCtasPerSm = 4;  // resident CTAs of k_mc_count_list per SM
constexpr int kCountStages = 4;     // its ring of warp-block buffers (32 KB per CTA)
constexpr int kWarpCells = kRounds * 32;  // a warp block of k_mc_count_list
constexpr int kSuperWarpBlocks = 64;      // warp blocks per superblock (the unit of its offsets)
constexpr int kScanPerThread = 32;
constexpr int kScanChunk = kThreads * kScanPerThread;

struct McTables {
  signed char tri[256][16];
  unsigned short edge[256];
  unsigned char ntri[256];
  signed char corner[8][3];
  signed char ends[12][2];
};

constexpr int hexv(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }

constexpr McTables build_tables() {
  McTables t{};
  for (int c = 0; c < 256; ++c) {
    const char *s = kfmc::kTriRows[c];
    int k = 0;
    for (; s[k]; ++k) t.tri[c][k] = (signed char)hexv(s[k]);
    t.ntri[c] = (unsigned char)(k / 3);
    for (; k < 16; ++k) t.tri[c][k] = -1;
    int m = 0;
    for (int e = 0; e < 12; ++e) {
      int a = (c >> kfmc::kEdge[e][0]) & 1, b = (c >> kfmc::kEdge[e][1]) & 1;
      if (a != b) m |= 1 << e;
    }
    t.edge[c] = (unsigned short)m;
  }
  for (int k = 0; k < 8; ++k)
    for (int j = 0; j < 3; ++j) t.corner[k][j] = (signed char)kfmc::kCellCorner[k][j];
  for (int e = 0; e < 12; ++e)
    for (int j = 0; j < 2; ++j) t.ends[e][j] = (signed char)kfmc::kEdge[e][j];
  return t;
}

// Uniform lookups (corner offsets, edge ends) read the constant bank; the
// per-cell ones (indexed by each thread's own configuration) read the same
// tables from global memory through L1, which serves a warp's different
// entries together where the constant bank would serialise them.
__constant__ McTables c_mc = build_tables();
__device__ const McTables g_mc = build_tables();

struct McGrid {
  const float *phi;
  int nx, ny, nz;
  int64_t count;
  float hi, lo, oob;  // skip if phi > hi or phi < lo; value outside the grid
  float hx, hy, hz;   // half grid size
};

__device__ __forceinline__ float at(const McGrid &g, int x, int y, int z) {
  if (x < 0 || x >= g.nx || y < 0 || y >= g.ny || z < 0 || z >= g.nz) return g.oob;
  return __ldg(g.phi + ((int64_t)z * g.ny + y) * g.nx + x);
}

// Cube configuration of cell i, or -1 when the cell is skipped (outside the
// grid, or its own value outside [lo, hi]).
__device__ __forceinline__ float own_value(const McGrid &g, int64_t i) {
  return i < g.count ? __ldg(g.phi + i) : g.hi + 1.0f;  // past the end: skipped
}

// d: the cell's own value, own_value(g, i), loaded ahead by the caller so the
// loads of all rounds are in flight together.
__device__ __forceinline__ int classify(const McGrid &g, int64_t i, float d, int &x, int &y, int &z,
                                        float val[8]) {
  if (d > g.hi || d < g.lo) return -1;  // SDF.cpp:407 (a NaN is not skipped)
  if (g.count <= 0xffffffffLL) {  // 32-bit division, several times cheaper
    const unsigned plane = (unsigned)g.nx * (unsigned)g.ny, ui = (unsigned)i;
    z = (int)(ui / plane);
    const unsigned r = ui - (unsigned)z * plane;
    y = (int)(r / (unsigned)g.nx);
    x = (int)(r - (unsigned)y * (unsigned)g.nx);
  } else {
    const int64_t plane = (int64_t)g.nx * g.ny;
    z = (int)(i / plane);
    const int64_t r = i - (int64_t)z * plane;
    y = (int)(r / g.nx);
    x = (int)(r - (int64_t)y * g.nx);
  }
  int cube = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    val[k] = at(g, x + c_mc.corner[k][0], y + c_mc.corner[k][1], z + c_mc.corner[k][2]);
    if (val[k] < 0.0f) cube |= 1 << k;
  }
  return cube;
}

__device__ __forceinline__ int cube_tris(int cube) {
  return (cube < 0 || __ldg(&g_mc.edge[cube]) == 0) ? 0 : (int)__ldg(&g_mc.ntri[cube]);
}

template <typename T>
__device__ T block_exclusive_scan(T v, T *total) {
  __shared__ T warp_sums[kThreads / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T n = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += n;
  }
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    T w = lane < kThreads / 32 ? warp_sums[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T n = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += n;
    }
    if (lane < kThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  T prefix = (wid > 0 ? warp_sums[wid - 1] : T(0)) + inc - v;
  if (total) *total = warp_sums[kThreads / 32 - 1];
  __syncthreads();
  return prefix;
}

__global__ void __launch_bounds__(kThreads) k_mc_count(McGrid g, uint32_t *block_tris) {
  const int64_t base = (int64_t)blockIdx.x * kCellsPerBlock + threadIdx.x;
  float d[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; ++r) d[r] = own_value(g, base + (int64_t)r * kThreads);
  uint32_t n = 0;
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    int x, y, z;
    float val[8];
    n += cube_tris(classify(g, base + (int64_t)r * kThreads, d[r], x, y, z, val));
  }
  uint32_t total;
  block_exclusive_scan<uint32_t>(n, &total);
  if (threadIdx.x == 0) block_tris[blockIdx.x] = total;
}

// Exclusive scan of the per-block totals into 64-bit offsets and the grand
// total, by one CTA (every thread calls it), a chunk of kScanChunk totals at
// a time: the chunk is staged in shared memory with coalesced loads (padded
// by one word per 32, so that thread t's kScanPerThread consecutive totals
// sit in distinct banks), each thread sums its totals, the block scans the
// sums, and each thread writes its offsets.  The totals are read through L2
// (other CTAs of the same launch may have written them).
__device__ void scan_block_totals(const uint32_t *block_tris, int64_t nblocks, int64_t *block_off,
                                  int64_t *grand_total) {
  __shared__ uint32_t s_v[kScanChunk + kScanChunk / 32];
  uint64_t carry = 0;
  for (int64_t c0 = 0; c0 < nblocks; c0 += kScanChunk) {
    const int64_t n = nblocks - c0 < kScanChunk ? nblocks - c0 : kScanChunk;
    for (int i = threadIdx.x; i < kScanChunk; i += kThreads)
      s_v[i + (i >> 5)] = i < n ? __ldcg(block_tris + c0 + i) : 0u;
    __syncthreads();
    const int first = threadIdx.x * kScanPerThread;
    uint64_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanPerThread; ++j) sum += s_v[first + j + ((first + j) >> 5)];
    uint64_t total;
    uint64_t excl = carry + block_exclusive_scan<uint64_t>(sum, &total);
#pragma unroll
    for (int j = 0; j < kScanPerThread; ++j) {
      const int i = first + j;
      if (i < n) block_off[c0 + i] = (int64_t)excl;
      excl += s_v[i + (i >> 5)];
    }
    carry += total;
    __syncthreads();  // the chunk is read before the next one is staged
  }
  if (threadIdx.x == 0) *grand_total = (int64_t)carry;
}

__global__ void __launch_bounds__(kThreads) k_mc_scan(const uint32_t *block_tris, int64_t nblocks,
                                                      int64_t *block_off, int64_t *grand_total) {
  scan_block_totals(block_tris, nblocks, block_off, grand_total);
}

// The same scan for the count pass's last CTA, in registers (no shared
// staging, so that the count pass keeps its shared memory for its rings):
// thread t holds the kPer totals from c0 + t * kPer on (16-byte loads), the
// block scans the sums, and the thread writes their offsets and clears them
// (the count pass adds into zeroed totals).  A thread's chain of dependent
// steps is what the scan costs, so kPer is kept small for small n.  tris and
// off are 16-byte aligned.
template <int kPer>
__device__ void scan_totals_tail(uint32_t *tris, int64_t n, int64_t *off, int64_t *grand_total) {
  static_assert(kPer % 4 == 0, "16-byte groups");
  uint64_t carry = 0;
  for (int64_t c0 = 0; c0 < n; c0 += (int64_t)kThreads * kPer) {
    const int64_t first = c0 + (int64_t)threadIdx.x * kPer;
    const bool whole = first + kPer <= n;
    uint32_t v[kPer];
    if (whole) {
      const uint4 *p = reinterpret_cast<const uint4 *>(tris + first);
#pragma unroll
      for (int j = 0; j < kPer / 4; ++j) {
        const uint4 q = __ldcg(p + j);
        v[4 * j] = q.x, v[4 * j + 1] = q.y, v[4 * j + 2] = q.z, v[4 * j + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < kPer; ++j) v[j] = first + j < n ? __ldcg(tris + first + j) : 0u;
    }
    uint64_t sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) sum += v[j];
    uint64_t total;
    int64_t excl = (int64_t)(carry + block_exclusive_scan<uint64_t>(sum, &total));
    if (whole) {
      longlong2 *o = reinterpret_cast<longlong2 *>(off + first);
#pragma unroll
      for (int j = 0; j < kPer / 2; ++j) {
        o[j] = make_longlong2(excl, excl + v[2 * j]);
        excl += (int64_t)v[2 * j] + v[2 * j + 1];
      }
      uint4 *p = reinterpret_cast<uint4 *>(tris + first);
#pragma unroll
      for (int j = 0; j < kPer / 4; ++j) p[j] = make_uint4(0u, 0u, 0u, 0u);
    } else {
#pragma unroll
      for (int j = 0; j < kPer; ++j)
        if (first + j < n) {
          off[first + j] = excl;
          excl += v[j];
          tris[first + j] = 0u;
        }
    }
    carry += total;
  }
  if (threadIdx.x == 0) *grand_total = (int64_t)carry;
}

// Scratch of kf_mc_run's two passes.
struct McList {
  uint32_t *super_tris;  // triangles per superblock (zero between calls: the scan clears it)
  int64_t *super_off;    // exclusive offsets per superblock, then the grand total
  uint32_t *warp_tris;   // triangles per warp block, kSuperWarpBlocks per superblock
  uint2 *cells;          // per listed cell: index, (offset in its warp block << 8) | configuration
  unsigned *done;        // CTAs of the count pass finished (the last one resets it)
  unsigned *n_cells;     // cells appended by the count pass (the last CTA resets it)
  unsigned *n_listed;    // their final number, for the emit pass
  unsigned cap;          // entries `cells` holds (0: list nothing)
};

// 16-byte asynchronous copy global -> shared (cp.async, L2 only) and its
// group bookkeeping; a thread's wait covers only its own copies.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned dst = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Pass 1 of kf_mc_run, a resident grid of independent warps: each warp
// claims warp blocks (kWarpCells consecutive cells) from its CTA's counter
// and never waits for another warp.  It streams them through a ring of kCountStages
// shared-memory buffers with cp.async, kCountStages - 1 blocks ahead, so
// that the loads in flight cost no registers.  Lane l takes the cell 32 r + l of round r (the band cells
// of a surface spread over the lanes).  The band cells gather their
// corners; a warp scan per round gives each cell its offset among the warp
// block's triangles.  The cells with triangles are appended to the list,
// one atomic per warp block; an entry carries that offset, so the list's
// order does not matter.  The warp block's total is stored and added to its
// superblock's (kSuperWarpBlocks warp blocks); the last CTA to finish turns
// the superblock totals into offsets.
__global__ void __launch_bounds__(kThreads, kCountCtasPerSm)
    k_mc_count_list(McGrid g, McList L, int64_t nsuper) {
  __shared__ __align__(16) float s_ring[kThreads / 32][kCountStages][kWarpCells];
  __shared__ long long s_claimed[kThreads / 32][kCountStages];  // the warp block in each buffer
  __shared__ unsigned s_next;                                    // the CTA's next claim
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_next = 0u;
  __syncthreads();
  float(*ring)[kWarpCells] = s_ring[warp];
  long long *claimed = s_claimed[warp];
  const int64_t nwb = (g.count + kWarpCells - 1) / kWarpCells;
  const int64_t whole = g.count / kWarpCells;  // warp blocks entirely inside the grid
  // lane l copies the 16-byte chunks l and l + 32 of a warp block (kWarpCells = 256
  // cells = 64 chunks); a warp block past the whole ones is read directly
  const auto issue = [&](int64_t wb, int stage) {
    if (wb < whole) {
      const float *src = g.phi + wb * kWarpCells;
      cp_async16(&ring[stage][4 * lane], src + 4 * lane);
      cp_async16(&ring[stage][4 * (lane + 32)], src + 4 * (lane + 32));
    }
    cp_async_commit();  // (an empty group where nothing was copied)
  };
  // CTA c owns the warp blocks c, c + G, c + 2G, ... (G CTAs: the surface
  // spreads evenly over the CTAs); its warps claim them one at a time from a
  // shared-memory counter (the surface makes some much slower than others),
  // one round before their copy is issued
  const auto claim = [&]() -> int64_t {
    return (int64_t)blockIdx.x + (int64_t)atomicAdd(&s_next, 1u) * gridDim.x;
  };
  int64_t pending = 0;
  if (lane == 0) pending = claim();
#pragma unroll
  for (int k = 0; k < kCountStages - 1; ++k) {
    const int64_t wb = __shfl_sync(0xffffffffu, pending, 0);
    if (lane == 0) {
      claimed[k] = wb;
      pending = claim();
    }
    issue(wb, k);
  }
  __syncwarp();
  for (int stage = 0;; stage = stage == kCountStages - 1 ? 0 : stage + 1) {
    const int64_t wb = claimed[stage];
    if (wb >= nwb) break;  // (claims only grow: the later ones are past the end too)
    // the buffer read in the previous round takes the block claimed then
    const int prev = stage == 0 ? kCountStages - 1 : stage - 1;
    const int64_t nb = __shfl_sync(0xffffffffu, pending, 0);
    __syncwarp();
    if (lane == 0) {
      claimed[prev] = nb;
      pending = claim();
    }
    issue(nb, prev);
    cp_async_wait<kCountStages - 1>();  // this lane's copies of the current block
    __syncwarp();                        // ... and every lane's
    const int64_t base = wb * kWarpCells + lane;
    float d[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) d[r] = wb < whole ? ring[stage][32 * r + lane] : own_value(g, base + 32 * r);
    __syncwarp();  // the buffer is read before it is refilled
    unsigned band = 0;
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
      if (!(d[r] > g.hi || d[r] < g.lo)) band |= 1u << r;  // SDF.cpp:407 (a NaN is not skipped)
    uint32_t n = 0, counts = 0;  // counts: 4 bits per round (at most 5 triangles)
    uint64_t cubes = 0;          // 8 bits per round
    for (unsigned rest = band; rest; rest &= rest - 1) {
      const int r = __ffs(rest) - 1;
      const int64_t i = base + 32 * r;
      int x, y, z;
      float val[8];
      const int cube = classify(g, i, __ldg(g.phi + i), x, y, z, val);
      const uint32_t c = (uint32_t)cube_tris(cube);
      n += c;
      counts |= c << (4 * r);
      cubes |= (uint64_t)(cube & 255) << (8 * r);
    }
    const uint32_t total = __reduce_add_sync(0xffffffffu, n);
    if (lane == 0) {
      L.warp_tris[wb] = total;
      if (total) atomicAdd(L.super_tris + wb / kSuperWarpBlocks, total);
    }
    if (total) {
      // one slot per cell with triangles
      unsigned m = 0;
#pragma unroll
      for (int r = 0; r < kRounds; ++r) m += ((counts >> (4 * r)) & 15u) != 0u;
      unsigned incl = m;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      unsigned slot = 0;
      if (lane == 31) slot = atomicAdd(L.n_cells, incl);
      slot = __shfl_sync(0xffffffffu, slot, 31) + incl - m;
      uint32_t run = 0;
#pragma unroll
      for (int r = 0; r < kRounds; ++r) {
        const uint32_t c = (counts >> (4 * r)) & 15u;
        if (!__any_sync(0xffffffffu, c != 0u)) continue;  // a round without triangles
        uint32_t ci = c;  // inclusive scan of the round's counts over the lanes
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(0xffffffffu, ci, o);
          if (lane >= o) ci += t;
        }
        if (c) {
          if (slot < L.cap)
            L.cells[slot] = make_uint2((uint32_t)(base + 32 * r),
                                       ((run + ci - c) << 8) | (uint32_t)((cubes >> (8 * r)) & 255u));
          ++slot;
        }
        run += __shfl_sync(0xffffffffu, ci, 31);
      }
    }
  }
  cp_async_wait<0>();  // no copy outlives the warp (those past the end are empty)
  // the last CTA to finish turns the block totals into offsets (the classic
  // fence-and-count pattern: no CTA waits for another); every warp's
  // additions and appends are done before the CTA counts itself finished
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(L.done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (s_last) {
    __threadfence();
    if (nsuper <= (int64_t)kThreads * 4)
      scan_totals_tail<4>(L.super_tris, nsuper, L.super_off, L.super_off + nsuper);
    else
      scan_totals_tail<16>(L.super_tris, nsuper, L.super_off, L.super_off + nsuper);
    if (threadIdx.x == 0) {
      *L.n_listed = atomicExch(L.n_cells, 0u);
      *L.done = 0u;
    }
  }
}

__device__ __forceinline__ void vinterp(const float p1[3], const float p2[3], float v1, float v2,
                                        float out[3]) {
  float t = (0.0f - v1) / (v1 - v2);
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = p1[k] + t * (p1[k] - p2[k]);
}

// Writes the n triangles of cell i (configuration `cube`) from position out
// on; re-gathers the corners (band cells only, off the common path).  Each
// triangle vertex is interpolated on its edge as VertexInterp does
// (MarchingCubes.h:424-436): the corners' positions take two values per axis
// and their values stay in registers, picked by selects, so nothing is
// indexed by a per-thread value in local memory.
__device__ __noinline__ void emit_cell(const McGrid &g, int64_t i, int cube, int64_t out,
                                       float *__restrict__ verts, int64_t capacity) {
  int x, y, z;
  float val[8];
  classify(g, i, __ldg(g.phi + i), x, y, z, val);
  const float q[3][2] = {{(float)x / g.hx - 1.0f, (float)(x + 1) / g.hx - 1.0f},
                         {(float)y / g.hy - 1.0f, (float)(y + 1) / g.hy - 1.0f},
                         {(float)z / g.hz - 1.0f, (float)(z + 1) / g.hz - 1.0f}};
  const int n = __ldg(&g_mc.ntri[cube]);
  for (int t = 0; t < n; ++t, ++out) {
    if (out >= capacity) break;
    float *o = verts + 9 * out;
#pragma unroll
    for (int j2 = 0; j2 < 3; ++j2) {
      const int e = __ldg(&g_mc.tri[cube][3 * t + j2]);
      const int a = __ldg(&g_mc.ends[e][0]), b = __ldg(&g_mc.ends[e][1]);
      float va = val[0], vb = val[0];
#pragma unroll
      for (int c = 1; c < 8; ++c) {
        va = a == c ? val[c] : va;
        vb = b == c ? val[c] : vb;
      }
      float pa[3], pb[3], v[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pa[k] = __ldg(&g_mc.corner[a][k]) ? q[k][1] : q[k][0];
        pb[k] = __ldg(&g_mc.corner[b][k]) ? q[k][1] : q[k][0];
      }
      vinterp(pa, pb, va, vb, v);
      o[3 * j2 + 0] = v[0];
      o[3 * j2 + 1] = -v[1];
      o[3 * j2 + 2] = v[2];
    }
  }
}

// The triangles of cell block b (cells b*kCellsPerBlock + r*kThreads + t),
// from position out0 on; every cell is classified again.
__device__ __forceinline__ void emit_block(const McGrid &g, int64_t b, int64_t out0, float *__restrict__ verts,
                                           int64_t capacity) {
  const int64_t base = b * kCellsPerBlock + threadIdx.x;
  // classify every round first (the loads in flight together), then scan
  // and emit the rounds that have triangles
  float d[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; ++r) d[r] = own_value(g, base + (int64_t)r * kThreads);
  int cube[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    int x, y, z;
    float val[8];
    cube[r] = classify(g, base + (int64_t)r * kThreads, d[r], x, y, z, val);
  }
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    const uint32_t n = (uint32_t)cube_tris(cube[r]);
    if (!__syncthreads_or(n != 0)) continue;  // no triangle in this round
    uint32_t round_total;
    const int64_t out = out0 + (int64_t)block_exclusive_scan<uint32_t>(n, &round_total);
    out0 += round_total;
    if (n) emit_cell(g, base + (int64_t)r * kThreads, cube[r], out, verts, capacity);
  }
}

// Every cell block, one CTA each.
__global__ void __launch_bounds__(kThreads) k_mc_emit(McGrid g, const int64_t *block_off,
                                                      float *__restrict__ verts, int64_t capacity) {
  emit_block(g, blockIdx.x, block_off[blockIdx.x], verts, capacity);
}

// The first triangle of warp block wb: its superblock's offset plus the
// triangles of the superblock's earlier warp blocks (all of them counted:
// they precede wb, which lies inside the grid).  The superblock's 64 totals
// are loaded together; those from wb on are masked out.
__device__ __forceinline__ int64_t warp_block_offset(const McList &L, int64_t wb) {
  const int64_t sb = wb / kSuperWarpBlocks;
  const int k = (int)(wb - sb * kSuperWarpBlocks);
  const uint4 *wt = reinterpret_cast<const uint4 *>(L.warp_tris + sb * kSuperWarpBlocks);
  uint32_t sum = 0;
#pragma unroll
  for (int j = 0; j < kSuperWarpBlocks / 4; ++j) {
    const uint4 t = __ldg(wt + j);
    sum += (4 * j < k ? t.x : 0u) + (4 * j + 1 < k ? t.y : 0u) + (4 * j + 2 < k ? t.z : 0u) +
           (4 * j + 3 < k ? t.w : 0u);
  }
  return L.super_off[sb] + (int64_t)sum;
}

// Pass 2 of kf_mc_run: a resident grid.  Each thread writes the triangles of
// listed cells; when the list overflowed, each CTA instead takes blocks of
// kCellsPerBlock cells with triangles and re-classifies them (emit_block).
__global__ void __launch_bounds__(kThreads) k_mc_emit_cells(McGrid g, McList L, int64_t nblocks,
                                                            float *__restrict__ verts, int64_t capacity) {
  const unsigned n = *L.n_listed;
  if (n <= L.cap) {
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
      const uint2 c = L.cells[e];
      const int64_t i = c.x;
      if (!KF_IN_BOUNDS(i, g.count, KF_SITE_MC_BLOCK)) continue;
      emit_cell(g, i, (int)(c.y & 255u), warp_block_offset(L, i / kWarpCells) + (int64_t)(c.y >> 8), verts,
                capacity);
    }
  } else {
    constexpr int kPerBlock = kCellsPerBlock / kWarpCells;
    const int64_t nwb = (g.count + kWarpCells - 1) / kWarpCells;
    for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
      uint32_t tris = 0;
      for (int64_t wb = b * kPerBlock; wb < (b + 1) * kPerBlock && wb < nwb; ++wb) tris += __ldg(L.warp_tris + wb);
      if (tris) emit_block(g, b, warp_block_offset(L, b * kPerBlock), verts, capacity);
    }
  }
}

// The count pass wants shared memory for kCountCtasPerSm rings of 32 KB per
// SM: the largest shared-memory carveout (kBesideSolveCarveout), as the
// emit pass, which runs beside the band-only solver too.
void prefer_shared_for_count() {
  static bool done[2][64] = {};
  kf_prefer_carveout((const void *)k_mc_count_list, kBesideSolveCarveout, done[0]);
  kf_prefer_carveout((const void *)k_mc_emit_cells, kBesideSolveCarveout, done[1]);
}

// Resident CTAs of the emit pass.
unsigned emit_grid(int64_t nblocks) {
  return (unsigned)std::min<int64_t>(nblocks, (int64_t)kf_num_sms() * 8);
}

}  // namespace

// ntri_async == NULL: waits for the count, returns it in *ntri and launches
// the emit pass only when there are triangles.  Otherwise nothing waits: the
// count is copied to ntri_async (device or pinned host memory) and the emit
// pass writes the first `capacity` triangles.
int kf_mc_run(kf_grid g, const DevParams &dp, float *verts, int64_t capacity, int64_t *ntri,
              cudaStream_t s, int64_t *ntri_async) {
  McGrid mg;
  mg.phi = g->phi;
  mg.nx = g->n[0];
  mg.ny = g->n[1];
  mg.nz = g->n[2];
  mg.count = g->count;
  mg.hi = dp.mc_hi_f;
  mg.lo = dp.band_lo_f;
  mg.oob = dp.oob_phi_f;
  mg.hx = (float)g->n[0] / 2.0f;
  mg.hy = (float)g->n[1] / 2.0f;
  mg.hz = (float)g->n[2] / 2.0f;
  const int64_t nblocks = (g->count + kCellsPerBlock - 1) / kCellsPerBlock;
  const int64_t nwb = (g->count + kWarpCells - 1) / kWarpCells;
  const int64_t nsuper = (nwb + kSuperWarpBlocks - 1) / kSuperWarpBlocks;
  // scratch, kept with the grid (calls on one grid are stream-ordered): the
  // per-superblock totals (u32), their offsets (i64) and the grand total
  // right after them, three counters, the per-warp-block totals (u32,
  // kSuperWarpBlocks per superblock) and the list of cells with triangles
  // (count / 16 of them, at least 2^18; none for grids of 2^32 cells or
  // more, whose indices the list does not hold)
  const int64_t cap = g->count >= (int64_t)1 << 32
                          ? 0
                          : std::min<int64_t>(g->count, std::max<int64_t>(g->count / 16, 1 << 18));
  const size_t off_off = ((size_t)nsuper * sizeof(uint32_t) + 255) & ~(size_t)255;
  const size_t cnt_off = off_off + (((size_t)nsuper + 1) * sizeof(int64_t) + 15) / 16 * 16;
  const size_t warp_off = cnt_off + 32;
  const size_t list_off = warp_off + (size_t)nsuper * kSuperWarpBlocks * sizeof(uint32_t);
  const size_t bytes = list_off + (size_t)cap * sizeof(uint2);
  bool fresh = false;
  if (g->mc_bytes < bytes) {
    cudaFree(g->mc);
    g->mc = nullptr;
    g->mc_bytes = 0;
    if (cudaMalloc(&g->mc, bytes) != cudaSuccess) {
      cudaGetLastError();
      g->mc = nullptr;
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the marching-cubes scratch failed");
    }
    g->mc_bytes = bytes;
    fresh = true;
  }
  McList L;
  L.super_tris = (uint32_t *)g->mc;
  L.super_off = (int64_t *)((char *)g->mc + off_off);
  int64_t *total_dev = L.super_off + nsuper;
  L.done = (unsigned *)((char *)g->mc + cnt_off);
  L.n_cells = L.done + 1;
  L.n_listed = L.done + 2;
  L.warp_tris = (uint32_t *)((char *)g->mc + warp_off);
  L.cells = (uint2 *)((char *)g->mc + list_off);
  L.cap = (unsigned)cap;
  // the superblock totals and the counters start at zero; the count pass's
  // last CTA leaves them so
  if (fresh) {
    KF_CHECK_CUDA(cudaMemsetAsync(L.super_tris, 0, (size_t)nsuper * sizeof(uint32_t), s));
    KF_CHECK_CUDA(cudaMemsetAsync(L.done, 0, 32, s));
  }
  prefer_shared_for_count();
  const unsigned count_grid = (unsigned)std::min<int64_t>((nwb + kThreads / 32 - 1) / (kThreads / 32),
                                                          (int64_t)kf_num_sms() * kCountCtasPerSm);
  k_mc_count_list<<<count_grid, kThreads, 0, s>>>(mg, L, nsuper);
  KF_CHECK_LAUNCH("k_mc_count_list");
  if (ntri_async) {
    KF_CHECK_CUDA(cudaMemcpyAsync(ntri_async, total_dev, sizeof(int64_t), cudaMemcpyDefault, s));
    if (verts && capacity > 0) {
      k_mc_emit_cells<<<emit_grid(nblocks), kThreads, 0, s>>>(mg, L, nblocks, verts, capacity);
      KF_CHECK_LAUNCH("k_mc_emit_cells");
    }
    return KF_OK;
  }
  // wait for the count only; the emit pass runs on while the caller queues
  // its next work
  int64_t total = 0;
  KF_CHECK_CUDA(cudaMemcpyAsync(&total, total_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  KF_CHECK_CUDA(cudaStreamSynchronize(s));
  *ntri = total;
  if (verts && total > 0 && capacity > 0) {
    k_mc_emit_cells<<<emit_grid(nblocks), kThreads, 0, s>>>(mg, L, nblocks, verts, capacity);
    KF_CHECK_LAUNCH("k_mc_emit_cells");
  }
  if (verts && capacity < total)
    return kf_fail(KF_ERR_CAPACITY, "vertex buffer holds fewer triangles than the mesh has");
  return KF_OK;
}

// ---------------------------------------------------------------------------
// Marching cubes without any allocation (kf_marching_cubes_noalloc).
//
// The scratch of the three passes -- per-block triangle totals (u32), their
// exclusive offsets (i64) and the grand total (i64) -- lives in one
// file-scope device array sized for the largest grid this entry point
// accepts, KF_MC_NOALLOC_MAX_CELLS cells.  Each GPU that loads the library
// holds it until the process exits.  Host code cannot use the array's name as
// a device address, so the address is looked up with cudaGetSymbolAddress
// once per device, with that device current, on the first call there.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocMaxBlocks = (KF_MC_NOALLOC_MAX_CELLS + kCellsPerBlock - 1) / kCellsPerBlock;
constexpr size_t kNoAllocOffBytes = (size_t)(kNoAllocMaxBlocks + 1) * sizeof(int64_t);
constexpr size_t kNoAllocBytes = kNoAllocOffBytes + (size_t)kNoAllocMaxBlocks * sizeof(uint32_t);

static __device__ __align__(256) unsigned char g_mc_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kMaxDevices] = {};

int noalloc_scratch(void **out) {
  int dev = 0;
  KF_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return kf_fail(KF_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_mc_noalloc_scratch);
    if (e != cudaSuccess) return kf_cuda_fail(e, "cudaGetSymbolAddress(marching-cubes scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return KF_OK;
}

}  // namespace

extern "C" int kf_marching_cubes_noalloc(const float *phi, const int dims[3], const kf_params *p,
                                         float *verts, int64_t capacity, int64_t *ntri,
                                         void *stream) {
  KF_REQUIRE(phi && dims && ntri, "NULL argument");
  KF_REQUIRE(capacity >= 0, "capacity must be >= 0");
  KF_REQUIRE(dims[0] > 0 && dims[1] > 0 && dims[2] > 0, "grid dims must be positive");
  const int64_t cells = (int64_t)dims[0] * dims[1] * dims[2];
  if (cells > KF_MC_NOALLOC_MAX_CELLS)
    return kf_fail(KF_ERR_INVALID,
                   "grid has " + std::to_string(cells) + " cells; kf_marching_cubes_noalloc handles "
                   "at most " + std::to_string((long long)KF_MC_NOALLOC_MAX_CELLS) +
                   " (512^3); use kf_marching_cubes");
  int rc = kf_check_params(p);
  if (rc) return rc;
  void *base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc) return rc;
  cudaStream_t s = kf_stream(stream);
  DevParams dp = kf_make_dev_params(dims, p);
  McGrid mg;
  mg.phi = phi;
  mg.nx = dims[0];
  mg.ny = dims[1];
  mg.nz = dims[2];
  mg.count = cells;
  mg.hi = dp.mc_hi_f;
  mg.lo = dp.band_lo_f;
  mg.oob = dp.oob_phi_f;
  mg.hx = (float)dims[0] / 2.0f;
  mg.hy = (float)dims[1] / 2.0f;
  mg.hz = (float)dims[2] / 2.0f;
  const int64_t nblocks = (cells + kCellsPerBlock - 1) / kCellsPerBlock;
  int64_t *off = (int64_t *)base;               // nblocks offsets, then the grand total
  int64_t *total_dev = off + kNoAllocMaxBlocks;
  uint32_t *tris = (uint32_t *)((char *)base + kNoAllocOffBytes);
  // Every word read below is written earlier in this call; the grand total is
  // cleared anyway so a failed launch cannot report a previous call's count.
  KF_CHECK_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(int64_t), s));
  k_mc_count<<<(unsigned)nblocks, kThreads, 0, s>>>(mg, tris);
  k_mc_scan<<<1, kThreads, 0, s>>>(tris, nblocks, off, total_dev);
  if (verts && capacity > 0)
    k_mc_emit<<<(unsigned)nblocks, kThreads, 0, s>>>(mg, off, verts, capacity);
  KF_CHECK_LAUNCH("kf_marching_cubes_noalloc kernels");
  int64_t total = 0;
  KF_CHECK_CUDA(cudaMemcpyAsync(&total, total_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  KF_CHECK_CUDA(cudaStreamSynchronize(s));
  *ntri = total;
  if (verts && capacity < total)
    return kf_fail(KF_ERR_CAPACITY, "vertex buffer holds fewer triangles than the mesh has");
  return KF_OK;
}

KF_BOUNDS_TU_API(mc)
