// Kernels whose outcome hinges on the reference's double-precision rounding.
//
// This translation unit is compiled with -fmad=false: no multiply-add is
// fused, so every float64 expression rounds exactly as the reference's
// (compiled with -ffp-contract=off) does.  It holds
//   - projective integration (the pixel a voxel projects to is decided by a
//     rounding of a double, SDF.cpp:162-172),
//   - the warp / fuse family (the warped weight is a truncation of an
//     interpolated double, SDF.cpp:316-320),
//   - the float64 psi solver that replays the reference bit for bit, and the
//     per-voxel reference-gradient query.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "kf_bounds.cuh"
#include "kf_ffloat.cuh"
#include "kf_internal.h"
#include "kf_ref_math.cuh"

using namespace kfref;

namespace {

constexpr int kBlock = 256;

inline unsigned blocks_for(int64_t n, int per = kBlock) {
  return (unsigned)((n + per - 1) / per);
}

// Coordinates of voxel i; 32-bit division when the index fits (several
// times cheaper than the 64-bit one).
__device__ __forceinline__ void voxel_xyz(int64_t i, int nx, int ny, int &x, int &y, int &z) {
  if (i <= 0xffffffffLL) {
    const unsigned plane = (unsigned)nx * (unsigned)ny, ui = (unsigned)i;
    z = (int)(ui / plane);
    const unsigned r = ui - (unsigned)z * plane;
    y = (int)(r / (unsigned)nx);
    x = (int)(r - (unsigned)y * (unsigned)nx);
    return;
  }
  int64_t plane = (int64_t)nx * ny;
  z = (int)(i / plane);
  int64_t r = i - (int64_t)z * plane;
  y = (int)(r / nx);
  x = (int)(r - (int64_t)y * nx);
}

// ---------------------------------------------------------------------------
// SDF::integrateDepthFrame (SDF.cpp:137-197)
// ---------------------------------------------------------------------------
struct IntegrateArgs {
  double W[16];  // world -> camera, row-major
  double K[9];   // intrinsics, row-major
  float Kf[6];                          // K[0..5] rounded to float
  float e0, e1, e2;                    // error bounds of the float camera rows (launch_integrate)
  float ku0, ku1, kv0, kv1;            // 1.5 |K[0]|, 1.5 |K[1]|, 1.5 |K[3]|, 1.5 |K[4]|
  float c2_min;                        // smallest |camera depth| the float path takes
  float fresh_phi;                     // a fresh grid's phi (k_integrate<D, true>)
  double voxel, min0, min1, min2, unknown_clip, min_depth, max_depth;
  float min_depth_up, max_depth_down;  // float neighbours of the depth range
  double depth_scale;                  // metres per unit of 16-bit depth
  float cliph, clipl;                  // unknown_clip as a float pair
  float tol;                           // bound on |float-float distance - reference's|
  float clip_thr;                      // |dist.hi + cliph| above this decides the clip test
  int width, height;
  int64_t count;                       // voxels of the grid
};

// Pixel coordinates exactly as SDF::integrateDepthFrame computes them, in
// float64 (SDF.cpp:151-164).
__device__ __forceinline__ void project_exact(const IntegrateArgs &a, int x, int y, int z, double &u,
                                              double &v, double &zc) {
  double Z = a.voxel * ((double)z + 0.5) + a.min2;
  double Y = a.voxel * ((double)y + 0.5) + a.min1;
  double X = a.voxel * ((double)x + 0.5) + a.min0;
  double c[3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    c[r] = a.W[4 * r + 0] * X + a.W[4 * r + 1] * Y + a.W[4 * r + 2] * Z + a.W[4 * r + 3] * 1.0;
  double pa = c[0] / c[2], pb = c[1] / c[2];
  u = a.K[0] * pa + a.K[1] * pb + a.K[2] * 1.0;
  v = a.K[3] * pa + a.K[4] * pb + a.K[5] * 1.0;
  zc = c[2];
}

// The reference's pixel index: roundf of the double converted to float
// (SDF.cpp:167,171).  A non-finite value never lands inside the image
// (x86-64 converts it to INT_MIN); -1 stands for "outside".
__device__ __forceinline__ int pixel_of(double u) {
  float f = (float)(u + 0.5);
  if (!isfinite(f)) return -1;
  return (int)roundf(f);
}

// The running-mean update of SDF.cpp:185-193 once the pixel and the camera
// depth zc are known.  With w == 0 and a finite phi the mean
// (phi*0 + dist)/1 is dist itself, so the float64 multiply and divide are
// skipped.  wi and ph are the voxel's weight and value, loaded by the caller.
// False when the voxel is not integrated (nothing written).
__device__ __forceinline__ bool integrate_update(float *__restrict__ phi, int32_t *__restrict__ w, int64_t i,
                                                 double depth, double zc, const IntegrateArgs &a, int32_t wi,
                                                 float ph) {
  const double dist = depth - zc;
  if (dist < -a.unknown_clip) return false;
  if (wi == 0 && isfinite(ph)) {
    phi[i] = (float)dist;
  } else {
    phi[i] = (float)(((double)ph * (double)wi + dist) / (double)(wi + 1));
  }
  w[i] = wi + 1;
  return true;
}

// The depth at pixel k as the reference reads it (a double) and its range
// test `depth < minDepth || depth > maxDepth` (SDF.cpp:176-179; a NaN passes,
// as there).  Float metres: compared through the float neighbours of the
// bounds.  16-bit units: (double)v * scale, as cv::Mat::convertTo with a
// scale produces them (DatasetReader.cpp:131-132).
__device__ __forceinline__ bool depth_at(const float *__restrict__ depth, int64_t k, const IntegrateArgs &a,
                                         double &d) {
  const float df = depth[k];
  d = (double)df;
  return !(df < a.min_depth_up || df > a.max_depth_down);
}

__device__ __forceinline__ bool depth_at(const uint16_t *__restrict__ depth, int64_t k, const IntegrateArgs &a,
                                         double &d) {
  d = (double)depth[k] * a.depth_scale;
  return !(d < a.min_depth || d > a.max_depth);
}

// The whole float64 path of one voxel (SDF.cpp:151-193).
template <typename D>
__device__ __noinline__ void integrate_exact_voxel(float *__restrict__ phi, int32_t *__restrict__ w, int x, int y,
                                                   int z,
                                      int64_t i, const D *__restrict__ depth, const IntegrateArgs &a) {
  double u, v, zc;
  project_exact(a, x, y, z, u, v, zc);
  const int col = pixel_of(u), row = pixel_of(v);
  if (col < 0 || col >= a.width || row < 0 || row >= a.height) return;
  double dd;
  if (!depth_at(depth, (int64_t)row * a.width + col, a, dd)) return;
  integrate_update(phi, w, i, dd, zc, a, w[i], phi[i]);
}

// Per-axis products of the camera-depth row, W[8]*X(x), W[9]*Y(y) and
// W[10]*Z(z), with X = voxel*(x+0.5)+min as SDF.cpp:151-157 computes it:
// zc = ((tx + ty) + tz) + W[11] is then the reference's float64 value.
// The float path's table tp (nx + ny + nz entries, x then y then z) holds
// per axis value: the camera-x and camera-y row products rounded to float
// and the camera-depth product as a float pair, with the rows' constant
// terms W[3], W[7] and W[11] added to the x entries.
//
// The next bw * bh CTAs mark the depth frame's 16 x 16-pixel blocks that
// hold a pixel passing the reference's depth test (SDF.cpp:176-179; a NaN
// passes it): flags[by * bw + bx] = 1.  k_integrate_tiles skips a tile of
// voxels whose possible pixels lie in unmarked blocks only.  For a fresh
// grid (fill != NULL) the remaining CTAs write every voxel's reset values
// (phi = a.fresh_phi, w = 0; 16-byte stores), which only the listed tiles'
// voxels then overwrite.
constexpr int kPixBlock = 16;

template <typename D>
__global__ void __launch_bounds__(kBlock) k_integrate_prep(double *__restrict__ tx, double *__restrict__ ty,
                                                           double *__restrict__ tz, float4 *__restrict__ tp,
                                                           int nx, int ny, int nz, unsigned tab_blocks,
                                                           const D *__restrict__ depth,
                                                           uint8_t *__restrict__ flags, int bw, int bh,
                                                           float *__restrict__ fill_phi,
                                                           int32_t *__restrict__ fill_w, int64_t count,
                                                           IntegrateArgs a) {
  const unsigned flag_end = tab_blocks + (unsigned)(bw * bh);
  if (blockIdx.x >= flag_end) {
    // phi, w come from cudaMalloc (256-byte aligned); the last count % 4 one by one
    const unsigned nfill = gridDim.x - flag_end;
    const int64_t n4 = count >> 2;
    const float4 v4 = make_float4(a.fresh_phi, a.fresh_phi, a.fresh_phi, a.fresh_phi);
    for (int64_t k = (int64_t)(blockIdx.x - flag_end) * blockDim.x + threadIdx.x; k < n4;
         k += (int64_t)nfill * blockDim.x) {
      reinterpret_cast<float4 *>(fill_phi)[k] = v4;
      reinterpret_cast<int4 *>(fill_w)[k] = make_int4(0, 0, 0, 0);
    }
    if (blockIdx.x == flag_end && threadIdx.x < (count & 3)) {
      fill_phi[4 * n4 + threadIdx.x] = a.fresh_phi;
      fill_w[4 * n4 + threadIdx.x] = 0;
    }
    return;
  }
  if (blockIdx.x >= tab_blocks) {
    const int b = (int)(blockIdx.x - tab_blocks), bx = b % bw, by = b / bw;
    const int col = bx * kPixBlock + (int)(threadIdx.x % kPixBlock);
    const int row = by * kPixBlock + (int)(threadIdx.x / kPixBlock);
    double d;
    const bool ok = col < a.width && row < a.height && depth_at(depth, (int64_t)row * a.width + col, a, d);
    const int any = __syncthreads_or(ok);
    if (threadIdx.x == 0) flags[b] = (uint8_t)any;
    return;
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nx + ny + nz; k += tab_blocks * blockDim.x) {
    double c, t, r0, r1;
    if (k < nx) {
      c = a.voxel * ((double)k + 0.5) + a.min0;
      t = tx[k] = a.W[8] * c;
      r0 = a.W[0] * c + a.W[3];
      r1 = a.W[4] * c + a.W[7];
      t += a.W[11];
    } else if (k < nx + ny) {
      const int j = k - nx;
      c = a.voxel * ((double)j + 0.5) + a.min1;
      t = ty[j] = a.W[9] * c;
      r0 = a.W[1] * c;
      r1 = a.W[5] * c;
    } else {
      const int j = k - nx - ny;
      c = a.voxel * ((double)j + 0.5) + a.min2;
      t = tz[j] = a.W[10] * c;
      r0 = a.W[2] * c;
      r1 = a.W[6] * c;
    }
    const FF p = ff_from_double(t);
    tp[k] = make_float4(__double2float_rn(r0), __double2float_rn(r1), p.hi, p.lo);
  }
}

// The float projection of voxel (x, y, z) from the tables and its error
// bounds mu, mv (k_integrate's comment derives them); c2 is the float camera
// depth, px/py/pz the voxel's table entries.
struct FloatProjection {
  float4 px, py, pz;
  float c2, uf, vf, mu, mv;
};

__device__ __forceinline__ FloatProjection project_float(const float4 *__restrict__ tp, int nx, int ny, int x, int y,
                                                         int z, const IntegrateArgs &a) {
  FloatProjection q;
  q.px = __ldg(tp + x);
  q.py = __ldg(tp + nx + y);
  q.pz = __ldg(tp + nx + ny + z);
  const float c0 = __fadd_rn(__fadd_rn(q.px.x, q.py.x), q.pz.x);
  const float c1 = __fadd_rn(__fadd_rn(q.px.y, q.py.y), q.pz.y);
  q.c2 = __fadd_rn(__fadd_rn(q.px.z, q.py.z), q.pz.z);
  const float rc = __fdividef(1.0f, q.c2);
  const float pa = __fmul_rn(c0, rc), pb = __fmul_rn(c1, rc);
  const float ua = __fmul_rn(a.Kf[0], pa), ub = __fmul_rn(a.Kf[1], pb);
  const float va = __fmul_rn(a.Kf[3], pa), vb = __fmul_rn(a.Kf[4], pb);
  q.uf = __fadd_rn(__fadd_rn(ua, ub), a.Kf[2]);
  q.vf = __fadd_rn(__fadd_rn(va, vb), a.Kf[5]);
  const float arc = fabsf(rc);
  const float ea = a.e0 + fabsf(pa) * a.e2, eb = a.e1 + fabsf(pb) * a.e2;
  q.mu = (a.ku0 * ea + a.ku1 * eb) * arc + 0x1p-19f * (fabsf(ua) + fabsf(ub) + (fabsf(a.Kf[2]) + 2.0f));
  q.mv = (a.kv0 * ea + a.kv1 * eb) * arc + 0x1p-19f * (fabsf(va) + fabsf(vb) + (fabsf(a.Kf[5]) + 2.0f));
  return q;
}

// Whether no voxel of the tile [x0, x0 + 32) x [y0, y0 + kTileY) of plane z
// can integrate anything, decided by one warp.  The camera depth is affine
// over the tile and positive at its four corners, so it is positive on the
// whole tile, where u and v are linear-fractional and take their extremes
// at the corners: each corner's float projection, widened by its error
// bound, bounds them.  The tile is skipped when that range of u or v lies
// off the image (every voxel's pixel is rejected by SDF.cpp:167-172), or
// when every 16 x 16-pixel block its pixels can fall in holds no pixel that
// passes the depth test (every voxel is rejected by SDF.cpp:176-179).
constexpr int kTileY = kBlock / 32;  // k_integrate's CTA: 32 x kTileY voxels
constexpr int kIntegrateCtasPerSm = 6;  // resident CTAs of k_integrate (40 registers)

__device__ __forceinline__ bool tile_skippable(const float4 *__restrict__ tp, int nx, int ny, int x0, int y0, int z,
                                               const uint8_t *__restrict__ flags, int bw,
                                               const IntegrateArgs &a) {
  const int x1 = min(x0 + 31, nx - 1), y1 = min(y0 + kTileY - 1, ny - 1);
  float ulo = INFINITY, uhi = -INFINITY, vlo = INFINITY, vhi = -INFINITY;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const FloatProjection q = project_float(tp, nx, ny, c & 1 ? x1 : x0, c & 2 ? y1 : y0, z, a);
    if (!(q.c2 > a.c2_min && isfinite(q.uf) && isfinite(q.vf) && fabsf(q.uf) < 1e7f && fabsf(q.vf) < 1e7f &&
          q.mu < 1e6f && q.mv < 1e6f))
      return false;  // (a NaN bound fails the comparisons too)
    ulo = fminf(ulo, q.uf - q.mu);
    uhi = fmaxf(uhi, q.uf + q.mu);
    vlo = fminf(vlo, q.vf - q.mv);
    vhi = fmaxf(vhi, q.vf + q.mv);
  }
  // col = roundf(u + 0.5) is below 0 for u < -1 and at least width for
  // u > width - 1 (the float rounding of u + 0.5 moves that by 2^-24 of it)
  if (uhi < -1.001f || ulo > (float)a.width - 0.999f || vhi < -1.001f || vlo > (float)a.height - 0.999f)
    return true;
  // the pixels the tile's voxels can read, one more on every side
  const int c_lo = max(0, (int)floorf(ulo + 1.0f) - 1), c_hi = min(a.width - 1, (int)floorf(uhi + 1.0f) + 1);
  const int r_lo = max(0, (int)floorf(vlo + 1.0f) - 1), r_hi = min(a.height - 1, (int)floorf(vhi + 1.0f) + 1);
  // a row of blocks at a time, its flags loaded back to back and or-ed
  for (int by = r_lo / kPixBlock; by <= r_hi / kPixBlock; ++by) {
    const uint8_t *row = flags + by * bw;
    unsigned any = 0;
    for (int bx = c_lo / kPixBlock; bx <= c_hi / kPixBlock; ++bx) any |= __ldg(row + bx);
    if (any) return false;
  }
  return true;
}

// One thread per tile of 32 x kTileY voxels (tiles x-fastest, then y, then
// z): the tiles that can integrate something are appended to `live` (one
// atomic per warp; the order does not matter, every voxel is written by one
// thread).
constexpr int kTileThreads = 64;  // small CTAs: the tile tests are latency chains, spread over every SM

__global__ void __launch_bounds__(kTileThreads)
    k_integrate_tiles(const float4 *__restrict__ tp, int nx, int ny, int nz, const uint8_t *__restrict__ flags,
                      int bw, int *__restrict__ live, unsigned *__restrict__ n_live, IntegrateArgs a) {
  const int tiles_x = (nx + 31) / 32, tiles_y = (ny + kTileY - 1) / kTileY;
  const int64_t ntiles = (int64_t)tiles_x * tiles_y * nz;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool keep = false;
  if (t < ntiles) {
    const int cx = (int)(t % tiles_x), cy = (int)((t / tiles_x) % tiles_y);
    const int z = (int)(t / ((int64_t)tiles_x * tiles_y));
    keep = !tile_skippable(tp, nx, ny, cx * 32, cy * kTileY, z, flags, bw, a);
  }
  const unsigned ball = __ballot_sync(0xffffffffu, keep);
  if (!ball) return;
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (lane == 0) base = atomicAdd(n_live, (unsigned)__popc(ball));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (keep) live[base + __popc(ball & ((1u << lane) - 1u))] = (int)t;
}

// A fresh voxel (w == 0, phi finite) on float depth df, in float-float: the
// distance df - zc with the camera depth zc from the pair tables, the
// unknown-clip test and the float rounding, all decided when they lie
// farther than a.tol from the reference's float64 boundaries.  Returns
// kFfWritten (phi and w written), kFfClipped (not integrated, nothing
// written) or kFfUndecided (nothing written) when one of them is too close
// to call.
enum FfOutcome { kFfUndecided = 0, kFfWritten = 1, kFfClipped = 2 };

__device__ __forceinline__ int integrate_fresh_ff(float *__restrict__ phi, int32_t *__restrict__ w, int64_t i,
                                                  float df, FF zc, const IntegrateArgs &a) {
  const FF dist = ff_add_short(FF{df, 0.f}, ff_neg(zc));
  // dist + unknown_clip < 0: not integrated.  One float add decides it: its
  // error is below 2^-23 (|mf| + |unknown_clip|) plus the distance's, which
  // clip_thr = 2^-18 |unknown_clip| + 2 tol exceeds; the float-float sum
  // decides the rest
  const float mf = __fadd_rn(dist.hi, a.cliph);
  if (!(fabsf(mf) > a.clip_thr)) {
    const FF m = ff_add(dist, FF{a.cliph, a.clipl});
    if (!(fabsf(m.hi) > a.tol)) return kFfUndecided;
    if (m.hi < 0.f) return kFfClipped;
  } else if (mf < 0.f) {
    return kFfClipped;
  }
  bool ambiguous;
  const float r = ff_round_checked(dist, a.tol, ambiguous);
  if (ambiguous) return kFfUndecided;
  phi[i] = r;
  w[i] = 1;
  return kFfWritten;
}

// The voxel on the float64 path once its pixel k is known (the float-float
// decision could not be made, or the voxel holds a weight already): the
// reference's distance, clip test and running mean.  Out of line: it is
// rare, and inline its float64 registers would crowd the common path.
template <typename D, bool kFresh>
__device__ __noinline__ void integrate_f64_tail(float *__restrict__ phi, int32_t *__restrict__ w, int64_t i, int x,
                                                int y, int z, const D *__restrict__ depth, int64_t k,
                                                const double *__restrict__ tx, const double *__restrict__ ty,
                                                const double *__restrict__ tz, const IntegrateArgs &a, int32_t wi,
                                                float ph) {
  double dd;
  const double zd = ((__ldg(tx + x) + __ldg(ty + y)) + __ldg(tz + z)) + a.W[11] * 1.0;
  if (!depth_at(depth, k, a, dd) || !integrate_update(phi, w, i, dd, zd, a, wi, ph)) {
    if (kFresh) {  // nothing integrated
      phi[i] = a.fresh_phi;
      w[i] = 0;
    }
  }
}

// SDF::integrateDepthFrame for one voxel per thread.  The pixel a voxel reads
// flips only where u or v crosses an integer, so the projection runs in float
// from the per-axis tables (project_float) and is left to the float64 path
// when either coordinate lies within its error bound (derived below) of an
// integer, or is not finite.  Those voxels are listed (warp-aggregated) for k_integrate_exact,
// so the slow float64 projection runs on full warps instead of stalling the
// warps they fall in; past the list's capacity a voxel takes the path in
// place.
//
// The bound on |u - u_ref| (u_ref the reference's float64 value):
// * each camera row c_r is the sum of three table entries, each the float64
//   product rounded to float, in two float adds: within E_r = 3 * 2^-24 *
//   T_r of the float64 row, T_r the largest sum of the entries' magnitudes
//   over the grid (the camera depth c2 from the high parts of its pairs);
// * so pa = c0 / c2 is within (E0 + |pa| E2) / |c2| of the float64 quotient
//   to first order (|c2| > 8 E2 is required), and likewise pb;
// * 1/c2 by __fdividef (2 ulp) and the products add 5 * 2^-24 of |pa| and
//   |pb|, and u = K0 pa + K1 pb + K2 four more roundings of at most the sum
//   of its terms' magnitudes S; the float rounding of u_ref + 0.5 in the
//   reference's pixel_of moves the flip by half a float spacing, 2^-24 (S +
//   1.5) at most.
// The margin 1.5 (|K0| (E0 + |pa| E2) + |K1| (E1 + |pb| E2)) |1/c2| + 2^-19
// (S + 2) holds all of that with room for the second-order terms.
// The distance and the running mean are float64 as in the reference, decided
// in float-float for a fresh voxel (integrate_fresh_ff), with the camera
// depth summed from the tables' pairs there.
//
// kFresh: the grid is taken as just reset (phi = a.fresh_phi, w = 0; nothing
// read) and every voxel is written, the reset values where nothing is
// integrated (KillingFusion::computeSDF: a new SDF, then the frame).
template <typename D, bool kFresh>
__device__ __forceinline__ void integrate_voxel(float *__restrict__ phi, int32_t *__restrict__ w, int nx, int ny,
                                                int x, int y, int z, int64_t i, const D *__restrict__ depth,
                                                const double *__restrict__ tx, const double *__restrict__ ty,
                                                const double *__restrict__ tz, const float4 *__restrict__ tp,
                                                int *__restrict__ list, unsigned *__restrict__ list_n,
                                                unsigned list_cap, const IntegrateArgs &a) {
  // the voxel's weight and value, loaded first so that their latency runs
  // under the projection's arithmetic
  const int32_t wi = kFresh ? 0 : w[i];
  const float ph = kFresh ? a.fresh_phi : phi[i];
  const auto leave = [&]() {  // nothing integrated here
    if (kFresh) {
      phi[i] = a.fresh_phi;
      w[i] = 0;
    }
  };
  const FloatProjection q = project_float(tp, nx, ny, x, y, z, a);
  const float4 px = q.px, py = q.py, pz = q.pz;
  const float c2 = q.c2, uf = q.uf, vf = q.vf;
  const bool sure = fabsf(c2) > a.c2_min && fabsf(c2) < 0x1p100f && isfinite(uf) && isfinite(vf) &&
                    fabsf(uf) < 1e7f && fabsf(vf) < 1e7f && fabsf(uf - rintf(uf)) > q.mu &&
                    fabsf(vf - rintf(vf)) > q.mv;
  const unsigned act = __activemask();
  const unsigned need = __ballot_sync(act, !sure);
  if (!sure) {
    leave();  // (before the float64 path reads the voxel)
    const int lane = threadIdx.x & 31;  // blockDim.x == 32
    const int leader = __ffs(need) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(list_n, (unsigned)__popc(need));
    base = __shfl_sync(need, base, leader);
    const unsigned slot = base + (unsigned)__popc(need & ((1u << lane) - 1u));
    if (slot < list_cap)
      list[slot] = (int)i;
    else
      integrate_exact_voxel(phi, w, x, y, z, i, depth, a);
    return;
  }
  int col = (int)floorf(uf + 1.0f);  // == roundf(u + 0.5) away from the flips
  int row = (int)floorf(vf + 1.0f);
  if (uf < -1.0f) col = -1;  // roundf(u + 0.5) < 0: outside
  if (vf < -1.0f) row = -1;
  if (col < 0 || col >= a.width || row < 0 || row >= a.height) {
    leave();
    return;
  }
  const int64_t k = (int64_t)row * a.width + col;
  if constexpr (sizeof(D) == 4) {
    // float depth into a fresh voxel: float-float, float64 only when too close to call
    const float df = depth[k];
    if (df < a.min_depth_up || df > a.max_depth_down) {  // (a NaN passes, as in the reference)
      leave();
      return;
    }
    if (wi == 0 && isfinite(ph) && isfinite(df)) {
      const int r = integrate_fresh_ff(phi, w, i, df,
                                       ff_add_short(ff_add_short(FF{px.z, px.w}, FF{py.z, py.w}), FF{pz.z, pz.w}), a);
      if (r == kFfClipped) leave();
      if (r != kFfUndecided) return;
    }
  }
  integrate_f64_tail<D, kFresh>(phi, w, i, x, y, z, depth, k, tx, ty, tz, a, wi, ph);
}

// The live tiles (k_integrate_tiles), a resident grid of CTAs of 32 x
// kTileY threads, CTA c taking the entries c, c + G, ... of the list.  The
// other tiles hold nothing to integrate; a fresh grid has their reset
// values from k_integrate_prep.
template <typename D, bool kFresh>
__global__ void __launch_bounds__(kBlock, kIntegrateCtasPerSm)
    k_integrate(float *__restrict__ phi, int32_t *__restrict__ w, int nx, int ny, int nz,
                const D *__restrict__ depth, const double *__restrict__ tx, const double *__restrict__ ty,
                const double *__restrict__ tz, const float4 *__restrict__ tp, int *__restrict__ list,
                unsigned *__restrict__ list_n, unsigned list_cap, const int *__restrict__ live,
                const unsigned *__restrict__ n_live, IntegrateArgs a) {
  const unsigned tiles_x = (unsigned)(nx + 31) / 32u, tiles_y = (unsigned)(ny + kTileY - 1) / (unsigned)kTileY;
  const unsigned n = *n_live;
  for (unsigned e = blockIdx.x; e < n; e += gridDim.x) {
    const unsigned t = (unsigned)__ldg(live + e);
    const unsigned txy = t % (tiles_x * tiles_y);
    const int z = (int)(t / (tiles_x * tiles_y));
    const int x = (int)(txy % tiles_x) * 32 + threadIdx.x, y = (int)(txy / tiles_x) * kTileY + threadIdx.y;
    if (x >= nx || y >= ny) continue;
    integrate_voxel<D, kFresh>(phi, w, nx, ny, x, y, z, ((int64_t)z * ny + y) * nx + x, depth, tx, ty, tz, tp,
                               list, list_n, list_cap, a);
  }
}

// The listed voxels of k_integrate, each on the float64 path.
template <typename D>
__global__ void __launch_bounds__(kBlock) k_integrate_exact(float *__restrict__ phi, int32_t *__restrict__ w,
                                                            int nx, int ny, const D *__restrict__ depth,
                                                            const int *__restrict__ list,
                                                            const unsigned *__restrict__ list_n,
                                                            unsigned list_cap, IntegrateArgs a) {
  const unsigned n = min(*list_n, list_cap);
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t i = list[k];
    if (!KF_IN_BOUNDS(i, a.count, KF_SITE_INTEGRATE_LIST)) continue;
    int x, y, z;
    voxel_xyz(i, nx, ny, x, y, z);
    integrate_exact_voxel(phi, w, x, y, z, i, depth, a);
  }
}

}  // namespace

template <typename D>
static int launch_integrate(kf_grid g, const D *depth_dev, double depth_scale, int width, int height,
                            const double w2c[16], const double K[9], double min_depth, double max_depth,
                            const float *fresh_phi, cudaStream_t s) {
  IntegrateArgs a;
  for (int k = 0; k < 16; ++k) a.W[k] = w2c[k];
  for (int k = 0; k < 9; ++k) a.K[k] = K[k];
  for (int k = 0; k < 6; ++k) a.Kf[k] = (float)K[k];
  a.voxel = g->voxel;
  a.min0 = g->min3d[0];
  a.min1 = g->min3d[1];
  a.min2 = g->min3d[2];
  a.unknown_clip = g->unknown_clip;
  a.min_depth = min_depth;
  a.max_depth = max_depth;
  // float x < min_depth  <=>  x < smallest float >= min_depth, and likewise
  float lo = (float)min_depth, hi = (float)max_depth;
  if ((double)lo < min_depth) lo = nextafterf(lo, INFINITY);
  if ((double)hi > max_depth) hi = nextafterf(hi, -INFINITY);
  a.min_depth_up = lo;
  a.max_depth_down = hi;
  a.width = width;
  a.height = height;
  a.count = g->count;
  a.depth_scale = depth_scale;
  a.fresh_phi = fresh_phi ? *fresh_phi : 0.0f;
  ff_split_host(g->unknown_clip, a.cliph, a.clipl);
  {
    // the float-float distance is within a few 2^-46 of the magnitudes it
    // sums (and the reference's within a few 2^-53): 2^-38 of their bound
    double mag = fabs(w2c[11]) + fabs(max_depth);
    for (int c = 0; c < 3; ++c) {
      const double lo_c = g->min3d[c], hi_c = g->min3d[c] + g->voxel * (double)g->n[c];
      mag += fabs(w2c[8 + c]) * std::max(fabs(lo_c), fabs(hi_c));
    }
    a.tol = (float)(ldexp(mag, -38));
    a.clip_thr = (float)(ldexp(fabs(g->unknown_clip), -18) + 2.0 * (double)a.tol);
  }
  {
    // the float projection's error bounds (k_integrate): T_r is the largest
    // sum of the table entries' magnitudes for row r (each entry is affine
    // in its coordinate, so its extremes are at the grid's ends), E_r =
    // 3 * 2^-24 * T_r the bound on the float row's error
    double T[3] = {fabs(w2c[3]), fabs(w2c[7]), fabs(w2c[11])};
    for (int c = 0; c < 3; ++c) {
      const double lo_c = g->voxel * 0.5 + g->min3d[c], hi_c = g->voxel * ((double)g->n[c] - 0.5) + g->min3d[c];
      for (int r = 0; r < 3; ++r) T[r] += fabs(w2c[4 * r + c]) * std::max(fabs(lo_c), fabs(hi_c));
    }
    // (rounded up a little, so that their float values stay bounds)
    const double up = 1.0 + 0x1p-20;
    a.e0 = (float)(ldexp(3.0001 * T[0], -24) * up);
    a.e1 = (float)(ldexp(3.0001 * T[1], -24) * up);
    a.e2 = (float)(ldexp(3.0001 * T[2], -24) * up);
    a.ku0 = (float)(1.5 * fabs(K[0]) * up);
    a.ku1 = (float)(1.5 * fabs(K[1]) * up);
    a.kv0 = (float)(1.5 * fabs(K[3]) * up);
    a.kv1 = (float)(1.5 * fabs(K[4]) * up);
    a.c2_min = (float)std::max(8.0 * (double)a.e2, 0x1p-100);
  }
  // scratch: list counter, the three coordinate tables, the pixel-block
  // flags, the list
  const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
  const unsigned cap = (unsigned)std::min<int64_t>(std::max<int64_t>(g->count / 8, 65536), 0x7fffffff);
  const int bw = (width + kPixBlock - 1) / kPixBlock, bh = (height + kPixBlock - 1) / kPixBlock;
  const size_t tab_off = 256, flag_off = tab_off + (((size_t)(nx + ny + nz) * 24 + 255) & ~(size_t)255);
  const int64_t ntiles = (int64_t)((nx + 31) / 32) * ((ny + kTileY - 1) / kTileY) * nz;
  const size_t live_off = flag_off + (((size_t)bw * bh + 255) & ~(size_t)255);
  const size_t list_off = live_off + (((size_t)ntiles * sizeof(int) + 255) & ~(size_t)255);
  const size_t bytes = list_off + (size_t)cap * sizeof(int);
  if (g->integ_bytes < bytes) {
    cudaFree(g->integ);
    g->integ = nullptr;
    g->integ_bytes = 0;
    if (cudaMalloc(&g->integ, bytes) != cudaSuccess) {
      cudaGetLastError();
      g->integ = nullptr;
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the integration scratch failed");
    }
    g->integ_bytes = bytes;
  }
  char *base = (char *)g->integ;
  unsigned *list_n = (unsigned *)base;
  float4 *tp = (float4 *)(base + tab_off);
  double *tx = (double *)(tp + (nx + ny + nz)), *ty = tx + nx, *tz = ty + ny;
  uint8_t *flags = (uint8_t *)(base + flag_off);
  int *live = (int *)(base + live_off);
  unsigned *n_live = list_n + 1;
  int *list = (int *)(base + list_off);
  KF_CHECK_CUDA(cudaMemsetAsync(list_n, 0, 2 * sizeof(unsigned), s));
  {
    // these passes run beside the band-only solver (kBesideSolveCarveout)
    static bool done[5][64] = {};
    const int c = kBesideSolveCarveout;
    kf_prefer_carveout((const void *)k_integrate_prep<D>, c, done[0]);
    kf_prefer_carveout((const void *)k_integrate_tiles, c, done[1]);
    kf_prefer_carveout((const void *)k_integrate<D, true>, c, done[2]);
    kf_prefer_carveout((const void *)k_integrate<D, false>, c, done[3]);
    kf_prefer_carveout((const void *)k_integrate_exact<D>, c, done[4]);
  }
  const unsigned tab_blocks = blocks_for(nx + ny + nz);
  const unsigned fill_blocks = fresh_phi ? (unsigned)kf_num_sms() * 16 : 0u;
  k_integrate_prep<D><<<tab_blocks + (unsigned)(bw * bh) + fill_blocks, kBlock, 0, s>>>(
      tx, ty, tz, tp, nx, ny, nz, tab_blocks, depth_dev, flags, bw, bh, g->phi, g->w, g->count, a);
  k_integrate_tiles<<<blocks_for(ntiles, kTileThreads), kTileThreads, 0, s>>>(tp, nx, ny, nz, flags, bw, live,
                                                                               n_live, a);
  dim3 block(32, kTileY);
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, (int64_t)kf_num_sms() * kIntegrateCtasPerSm);
  if (fresh_phi)
    k_integrate<D, true><<<grid, block, 0, s>>>(g->phi, g->w, nx, ny, nz, depth_dev, tx, ty, tz, tp, list, list_n,
                                                cap, live, n_live, a);
  else
    k_integrate<D, false><<<grid, block, 0, s>>>(g->phi, g->w, nx, ny, nz, depth_dev, tx, ty, tz, tp, list,
                                                 list_n, cap, live, n_live, a);
  k_integrate_exact<D><<<(unsigned)kf_num_sms() * 4, kBlock, 0, s>>>(g->phi, g->w, nx, ny, depth_dev, list,
                                                                     list_n, cap, a);
  KF_CHECK_LAUNCH("k_integrate");
  return KF_OK;
}

int kf_launch_integrate(kf_grid g, const float *depth_dev, int width, int height, const double w2c[16],
                        const double K[9], double min_depth, double max_depth, const float *fresh_phi,
                        cudaStream_t s) {
  return launch_integrate(g, depth_dev, 0.0, width, height, w2c, K, min_depth, max_depth, fresh_phi, s);
}

int kf_launch_integrate_u16(kf_grid g, const uint16_t *depth_dev, double scale, int width, int height,
                            const double w2c[16], const double K[9], double min_depth, double max_depth,
                            const float *fresh_phi, cudaStream_t s) {
  return launch_integrate(g, depth_dev, scale, width, height, w2c, K, min_depth, max_depth, fresh_phi, s);
}

namespace {

// ---------------------------------------------------------------------------
// warp / fuse
// ---------------------------------------------------------------------------
template <typename P>
struct PsiPlanes {
  const P *x, *y, *z;
};

// Resample (phi, w) of `src` at i+0.5+psi(i) in float64 (SDF::update,
// SDF.cpp:309-321; SDF::getWeight SDF.cpp:584-604).  A voxel with psi == 0
// samples exactly its own cell (zero interpolation weights), so it keeps its
// values without arithmetic.
template <typename P>
__device__ __forceinline__ void warp_sample(const float *__restrict__ phi, const int32_t *__restrict__ w,
                                            int nx, int ny, int nz, double oob, PsiPlanes<P> f,
                                            int64_t i, int x, int y, int z, double &out_phi,
                                            double &out_w, bool &moved) {
  double d0 = (double)f.x[i], d1 = (double)f.y[i], d2 = (double)f.z[i];
  if (d0 == 0.0 && d1 == 0.0 && d2 == 0.0) {
    out_phi = (double)phi[i];
    out_w = (double)w[i];
    moved = false;
    return;
  }
  moved = true;
  double l0 = ((double)x + 0.5) + d0, l1 = ((double)y + 0.5) + d1, l2 = ((double)z + 0.5) + d2;
  double t0 = l0 - 0.5, t1 = l1 - 0.5, t2 = l2 - 0.5;
  int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
  double vp[8], vw[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    int cx = b0 + (c & 1), cy = b1 + ((c >> 1) & 1), cz = b2 + (c >> 2);
    bool in = cx >= 0 && cx < nx && cy >= 0 && cy < ny && cz >= 0 && cz < nz;
    int64_t j = ((int64_t)cz * ny + cy) * nx + cx;
    vp[c] = in ? (double)phi[j] : oob;
    vw[c] = in ? (double)w[j] : 0.0;
  }
  double f0 = t0 - (double)b0, f1 = t1 - (double)b1, f2 = t2 - (double)b2;
  out_w = lerp3(vw, f0, f1, f2);
  out_phi = lerp3(vp, f0, f1, f2);
}

// FUSE_BY_MERGE of (nphi, nw) into canonical voxel i (SDF.cpp:212-236).  The
// running mean is decided in float-float (ff_merge_mean); the rare voxel it
// cannot decide takes the reference's float64 expression.
__device__ __forceinline__ void fuse_voxel(float *__restrict__ cphi, int32_t *__restrict__ cw, int64_t i,
                                           float nphi, int32_t nw) {
  if (nw == 0) return;
  const int32_t w1 = cw[i];
  if (w1 == 0) {
    cphi[i] = nphi;
    cw[i] = nw;
  } else {
    const float f1 = cphi[i];
    float r;
    if (!ff_merge_mean(w1, f1, nw, nphi, r))
      r = (float)(((double)w1 * (double)f1 + (double)nw * (double)nphi) / (double)(w1 + nw));
    cphi[i] = r;
    cw[i] = w1 + nw;
  }
}

// SDF::update followed by canonical->fuse(live) (KillingFusion.cpp:158-159,
// SDF.cpp:199-241, 300-328), in place.  A voxel with psi == 0 keeps its
// values (zero interpolation weights), so only the moved voxels -- the band
// the solver updated -- change.  This pass fuses the others and lists the
// moved ones (warp-aggregated slots); k_warp_moved resamples and fuses those
// in float64, spread over every SM (in the blocks of this pass, which hold
// the surface, their float64 arithmetic was the kernel's tail), and
// k_warp_scatter writes their values back once every moved voxel has read
// its neighbours' old values.  Each thread takes four consecutive voxels
// with 16-byte loads.  When `cphi` is null only the warp is done.  kMoved:
// whether a voxel has moved comes from the bitmap `moved` (k_mark_moved)
// instead of its psi (4 bits a thread, where psi is 12 bytes a voxel).
template <typename P, bool kMoved = false>
__global__ void __launch_bounds__(kBlock) k_warp_fuse(const float *__restrict__ lphi,
                                                      const int32_t *__restrict__ lw,
                                                      float *__restrict__ cphi, int32_t *__restrict__ cw,
                                                      PsiPlanes<P> f, int nx, int ny, int nz, double oob,
                                                      float *__restrict__ side_phi,
                                                      int32_t *__restrict__ side_w,
                                                      int32_t *__restrict__ side_i,
                                                      unsigned *__restrict__ ctr,
                                                      const unsigned *__restrict__ moved_bits = nullptr) {
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i0 = 4 * q;
  float ph[4] = {0.f, 0.f, 0.f, 0.f};
  int32_t wv[4] = {0, 0, 0, 0};
  unsigned moved = 0;
  int valid = 0;
  if (i0 + 3 < N) {
    valid = 4;
    const float4 a = __ldcs(reinterpret_cast<const float4 *>(lphi) + q);
    const int4 b = __ldcs(reinterpret_cast<const int4 *>(lw) + q);
    ph[0] = a.x; ph[1] = a.y; ph[2] = a.z; ph[3] = a.w;
    wv[0] = b.x; wv[1] = b.y; wv[2] = b.z; wv[3] = b.w;
    if (kMoved) {
      moved = (__ldg(moved_bits + (i0 >> 5)) >> (i0 & 31)) & 15u;  // (i0 is a multiple of 4)
    } else if (sizeof(P) == 4) {
      const float4 x = __ldcs(reinterpret_cast<const float4 *>(f.x) + q);
      const float4 y = __ldcs(reinterpret_cast<const float4 *>(f.y) + q);
      const float4 z = __ldcs(reinterpret_cast<const float4 *>(f.z) + q);
      moved = (x.x != 0.f || y.x != 0.f || z.x != 0.f) | (x.y != 0.f || y.y != 0.f || z.y != 0.f) << 1 |
              (x.z != 0.f || y.z != 0.f || z.z != 0.f) << 2 | (x.w != 0.f || y.w != 0.f || z.w != 0.f) << 3;
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (f.x[i0 + e] != P(0) || f.y[i0 + e] != P(0) || f.z[i0 + e] != P(0)) moved |= 1u << e;
    }
  } else if (i0 < N) {
    valid = (int)(N - i0);
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      if (e >= valid) break;
      ph[e] = lphi[i0 + e];
      wv[e] = lw[i0 + e];
      if (kMoved ? ((__ldg(moved_bits + ((i0 + e) >> 5)) >> ((i0 + e) & 31)) & 1u) != 0u
                 : f.x[i0 + e] != P(0) || f.y[i0 + e] != P(0) || f.z[i0 + e] != P(0))
        moved |= 1u << e;
    }
  }
  // one slot range per warp for its moved voxels
  const int lane = threadIdx.x & 31;
  const unsigned nm = (unsigned)__popc(moved);
  unsigned incl = nm;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const unsigned wtotal = __shfl_sync(0xffffffffu, incl, 31);
  unsigned base = 0;
  if (lane == 0 && wtotal) base = atomicAdd(ctr, wtotal);
  unsigned slot = __shfl_sync(0xffffffffu, base, 0) + incl - nm;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    if (e >= valid) break;
    const int64_t i = i0 + e;
    if (moved & (1u << e)) {
      if (KF_IN_BOUNDS(slot, N, KF_SITE_SIDE_LIST)) side_i[slot] = (int32_t)i;
      ++slot;
    }
    else if (cphi)
      fuse_voxel(cphi, cw, i, ph[e], wv[e]);
  }
}

// The moved voxels listed by k_warp_fuse: resample (phi, w) at i+0.5+psi(i)
// in float64 (SDF::update, SDF.cpp:309-321), fuse into the canonical SDF,
// keep the new values in the side list for k_warp_scatter.
template <typename P>
__global__ void __launch_bounds__(kBlock) k_warp_moved(const float *__restrict__ lphi,
                                                       const int32_t *__restrict__ lw,
                                                       float *__restrict__ cphi, int32_t *__restrict__ cw,
                                                       PsiPlanes<P> f, int nx, int ny, int nz, double oob,
                                                       float *__restrict__ side_phi,
                                                       int32_t *__restrict__ side_w,
                                                       const int32_t *__restrict__ side_i,
                                                       const unsigned *__restrict__ ctr) {
  const unsigned n = *ctr;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t i = side_i[k];
    if (!KF_IN_BOUNDS(k, (int64_t)nx * ny * nz, KF_SITE_SIDE_LIST) ||
        !KF_IN_BOUNDS(i, (int64_t)nx * ny * nz, KF_SITE_SIDE_LIST))
      continue;
    int x, y, z;
    voxel_xyz(i, nx, ny, x, y, z);
    double dphi, dw;
    bool m;
    warp_sample(lphi, lw, nx, ny, nz, oob, f, i, x, y, z, dphi, dw, m);
    const float nphi = (float)dphi;
    const int32_t nw = (int32_t)(int64_t)dw;
    side_phi[k] = nphi;
    side_w[k] = nw;
    if (cphi) fuse_voxel(cphi, cw, i, nphi, nw);
  }
}

// Writes the moved voxels' resampled values back (after k_warp_fuse) and
// clears their bits of `moved_bits` (when given), which leaves it clear.
__global__ void __launch_bounds__(kBlock) k_warp_scatter(float *__restrict__ lphi, int32_t *__restrict__ lw,
                                                         const float *__restrict__ side_phi,
                                                         const int32_t *__restrict__ side_w,
                                                         const int32_t *__restrict__ side_i,
                                                         const unsigned *__restrict__ ctr, int64_t count,
                                                         unsigned *__restrict__ moved_bits = nullptr) {
  const unsigned n = *ctr;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int32_t i = side_i[k];
    if (!KF_IN_BOUNDS(k, count, KF_SITE_SIDE_LIST) || !KF_IN_BOUNDS(i, count, KF_SITE_SIDE_LIST)) continue;
    lphi[i] = side_phi[k];
    lw[i] = side_w[k];
    if (moved_bits) atomicAnd(moved_bits + (i >> 5), ~(1u << (i & 31)));
  }
}

// The bits of `moved_bits` of the recorded voxels touched[0, *touched_n)
// whose psi is not zero (psi is zero at every other voxel).
__global__ void __launch_bounds__(kBlock) k_mark_moved(PsiPlanes<float> f, const int *__restrict__ touched,
                                                       const unsigned *__restrict__ touched_n, int64_t count,
                                                       unsigned *__restrict__ moved_bits) {
  const unsigned n = *touched_n;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = touched[k];
    if (!KF_IN_BOUNDS(i, count, KF_SITE_SIDE_LIST)) continue;
    if (f.x[i] != 0.f || f.y[i] != 0.f || f.z[i] != 0.f) atomicOr(moved_bits + (i >> 5), 1u << (i & 31));
  }
}

// SDF::fuse(other) with FUSE_BY_MERGE (SDF.cpp:199-241).
__global__ void __launch_bounds__(kBlock) k_fuse(float *__restrict__ phi1, int32_t *__restrict__ w1,
                                                 const float *__restrict__ phi2,
                                                 const int32_t *__restrict__ w2, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t b = w2[i];
  if (b == 0) return;
  fuse_voxel(phi1, w1, i, phi2[i], b);
}

// SDF::fuse(other, psi) (SDF.cpp:244-297): the other SDF's weight stays an
// interpolated double until it is stored.
template <typename P>
__global__ void __launch_bounds__(kBlock) k_fuse_warped(float *__restrict__ phi1, int32_t *__restrict__ w1,
                                                        const float *__restrict__ phi2,
                                                        const int32_t *__restrict__ w2,
                                                        PsiPlanes<P> f, int nx, int ny, int nz,
                                                        double oob) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nx * ny * nz) return;
  int x, y, z;
  voxel_xyz(i, nx, ny, x, y, z);
  double d2, b;
  bool moved;
  warp_sample(phi2, w2, nx, ny, nz, oob, f, i, x, y, z, d2, b, moved);
  if (fabs(b) < (double)1e-5f) return;
  int32_t a = w1[i];
  if (a == 0) {
    phi1[i] = (float)d2;
    w1[i] = (int32_t)(int64_t)b;
  } else {
    double d1 = (double)phi1[i];
    phi1[i] = (float)(((double)a * d1 + b * d2) / ((double)a + b));
    w1[i] = (int32_t)(int64_t)((double)a + b);
  }
}

// ---------------------------------------------------------------------------
// float64 replay of the Jacobi psi update (KillingFusion.cpp:248-352)
// ---------------------------------------------------------------------------
// With dp.trust each step goes through trust_step; a voxel whose step
// failed keeps its psi and records its x in rows[z * ny + y] (the smallest
// such x of the row wins), for k_exact_trust_rows.
__global__ void __launch_bounds__(kBlock) k_exact_step(PhiView<double> live, PhiView<double> can,
                                                       PsiView<double, double> fin,
                                                       double *__restrict__ ox,
                                                       double *__restrict__ oy,
                                                       double *__restrict__ oz, DevParams dp,
                                                       IterStats *st, int iter, int *__restrict__ rows) {
  if (iteration_gated(st, iter, dp)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st[iter].skipped = 1;
    return;
  }
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool active = false;
  double dn = 0.0;
  if (i < dp.count) {
    int x, y, z;
    voxel_xyz(i, dp.nx, dp.ny, x, y, z);
    double p0 = fin.px[i], p1 = fin.py[i], p2 = fin.pz[i];
    double s = warped_distance(live, fin, x, y, z);
    double d[3] = {0.0, 0.0, 0.0};
    if (in_band(s, dp.band_hi, -dp.unknown_clip)) {
      active = true;
      TParams<double> tp(dp);
      double g[3], u[3];
      energy_gradient(live, can, fin, tp, x, y, z, g);
#pragma unroll
      for (int k = 0; k < 3; ++k) u[k] = -tp.alpha * g[k];
      const double c[3] = {p0, p1, p2};
      if (dp.trust && !trust_step(live, can.at(x, y, z), s, x, y, z, c, g, tp.alpha, u)) {
        atomicMin(rows + ((int64_t)z * dp.ny + y), x);
      } else {
        // the update field starts at zero (KillingFusion.cpp:256, 316)
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k] = d[k] + u[k];
      }
      if (!isfinite(p0) || !isfinite(p1) || !isfinite(p2)) st[iter].diverged = 1;
      dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
    ox[i] = p0 + d[0];
    oy[i] = p1 + d[1];
    oz[i] = p2 + d[2];
  }
  unsigned ballot = __ballot_sync(0xffffffffu, active);
  float m = (float)dn;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && ballot) {
    atomicAdd(&st[iter].active, (unsigned)__popc(ballot));
    atomicMax(&st[iter].max_delta, __float_as_uint(m));
  }
}

// Trust-region step, after k_exact_step: the voxels of a row from its first
// failed step on keep their psi (the reference's break out of the x loop,
// KillingFusion.cpp:312-313).  One warp per row; the warp clears the row's
// entry for the next iteration.
__global__ void __launch_bounds__(kBlock) k_exact_trust_rows(const double *__restrict__ ix,
                                                             const double *__restrict__ iy,
                                                             const double *__restrict__ iz,
                                                             double *__restrict__ ox, double *__restrict__ oy,
                                                             double *__restrict__ oz, int *__restrict__ rows,
                                                             int nx, int nrows) {
  const int row = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nrows) return;
  const int first = rows[row];
  if (first >= nx) return;
  const int64_t base = (int64_t)row * nx;
  for (int x = first + 1 + lane; x < nx; x += 32) {  // psi + the zero update
    ox[base + x] = ix[base + x] + 0.0;
    oy[base + x] = iy[base + x] + 0.0;
    oz[base + x] = iz[base + x] + 0.0;
  }
  __syncwarp();
  if (lane == 0) rows[row] = kRowClear;
}

// Reference gradient at a list of voxels (KillingFusion.cpp:399-442).
template <typename T, typename P>
__global__ void k_gradient_ref(PhiView<T> live, PhiView<T> can, PsiView<T, P> f, DevParams dp,
                               const int32_t *__restrict__ vox, int count, double *__restrict__ out,
                               uint8_t *__restrict__ active) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int x = vox[3 * i], y = vox[3 * i + 1], z = vox[3 * i + 2];
  TParams<T> tp(dp);
  T g[3];
  energy_gradient(live, can, f, tp, x, y, z, g);
  out[3 * i + 0] = (double)g[0];
  out[3 * i + 1] = (double)g[1];
  out[3 * i + 2] = (double)g[2];
  if (active) {
    T s = warped_distance(live, f, x, y, z);
    active[i] = in_band(s, band_hi<T>(dp), band_lo<T>(dp)) ? 1 : 0;
  }
}

template <typename T>
PhiView<T> phi_view(const kf_grid g, const float *phi, double oob) {
  PhiView<T> v;
  v.phi = phi;
  v.nx = g->n[0];
  v.ny = g->n[1];
  v.nz = g->n[2];
  v.oob = (T)oob;
  return v;
}

}  // namespace

int kf_grid_ensure_alt(kf_grid g) {
  if (g->phi_alt) return KF_OK;
  if (cudaMalloc(&g->phi_alt, g->count * sizeof(float)) != cudaSuccess)
    return kf_fail(KF_ERR_OOM, "cudaMalloc of the resampling buffer failed");
  if (cudaMalloc(&g->w_alt, g->count * sizeof(int32_t)) != cudaSuccess) {
    cudaFree(g->phi_alt);
    g->phi_alt = nullptr;
    return kf_fail(KF_ERR_OOM, "cudaMalloc of the resampling buffer failed");
  }
  return KF_OK;
}

template <typename P>
static PsiPlanes<P> planes(kf_field f) {
  return PsiPlanes<P>{(const P *)f->p[0], (const P *)f->p[1], (const P *)f->p[2]};
}

static int warp_fuse_impl(kf_grid can, kf_grid live, kf_field psi, const DevParams &dp,
                          cudaStream_t s) {
  // the moved-voxel list lives in psi's second (ping-pong) buffer, which
  // holds nothing between solves: values, weights and indices, N each
  int st = kf_field_ensure_pair(psi);
  if (st) return st;
  // q zero outside the field's records stays so, with the list's entries
  // [0, *live->ctr) recorded (once between two zeros of the field)
  const bool record = psi->q_state == kPsiRecorded && !psi->side_recorded && !psi->exposed;
  // p zero outside the recorded voxels: which voxels moved comes from a
  // bitmap of those voxels instead of psi at every voxel
  const bool by_bits = psi->p_state == kPsiRecorded && !psi->exposed && psi->prec == KF_F32;
  psi->q_state = kPsiUnknown;
  KfRecords r{};
  if (record || by_bits) {
    st = kf_field_records(psi, s, &r);
    if (st) return st;
  }
  float *side_phi = (float *)psi->q[0];
  int32_t *side_w = (int32_t *)psi->q[1];
  int32_t *side_i = (int32_t *)psi->q[2];
  float *cphi = can ? can->phi : nullptr;
  int32_t *cw = can ? can->w : nullptr;
  KF_CHECK_CUDA(cudaMemsetAsync(live->ctr, 0, sizeof(unsigned), s));
  const unsigned blocks = blocks_for((live->count + 3) / 4);
  const unsigned spread = (unsigned)kf_num_sms() * 4;
  if (by_bits) {
    k_mark_moved<<<spread, kBlock, 0, s>>>(planes<float>(psi), r.touched, r.touched_n, live->count, r.moved);
    k_warp_fuse<float, true><<<blocks, kBlock, 0, s>>>(live->phi, live->w, cphi, cw, planes<float>(psi),
                                                       live->n[0], live->n[1], live->n[2], dp.oob_phi, side_phi,
                                                       side_w, side_i, live->ctr, r.moved);
  } else if (psi->prec == KF_F32)
    k_warp_fuse<float><<<blocks, kBlock, 0, s>>>(live->phi, live->w, cphi, cw, planes<float>(psi), live->n[0],
                                                 live->n[1], live->n[2], dp.oob_phi, side_phi, side_w, side_i,
                                                 live->ctr);
  else
    k_warp_fuse<double><<<blocks, kBlock, 0, s>>>(live->phi, live->w, cphi, cw, planes<double>(psi), live->n[0],
                                                  live->n[1], live->n[2], dp.oob_phi, side_phi, side_w, side_i,
                                                  live->ctr);
  if (psi->prec == KF_F32)
    k_warp_moved<float><<<spread, kBlock, 0, s>>>(live->phi, live->w, cphi, cw, planes<float>(psi), live->n[0],
                                                  live->n[1], live->n[2], dp.oob_phi, side_phi, side_w, side_i,
                                                  live->ctr);
  else
    k_warp_moved<double><<<spread, kBlock, 0, s>>>(live->phi, live->w, cphi, cw, planes<double>(psi),
                                                   live->n[0], live->n[1], live->n[2], dp.oob_phi, side_phi,
                                                   side_w, side_i, live->ctr);
  k_warp_scatter<<<spread, kBlock, 0, s>>>(live->phi, live->w, side_phi, side_w, side_i, live->ctr, live->count,
                                           by_bits ? r.moved : nullptr);
  KF_CHECK_LAUNCH("k_warp_fuse");
  if (record) {
    KF_CHECK_CUDA(cudaMemcpyAsync(r.side_n, live->ctr, sizeof(unsigned), cudaMemcpyDeviceToDevice, s));
    psi->q_state = kPsiRecorded;
    psi->side_recorded = true;
  }
  return KF_OK;
}

int kf_launch_warp(kf_grid g, kf_field psi, const DevParams &dp, cudaStream_t s) {
  return warp_fuse_impl(nullptr, g, psi, dp, s);
}

int kf_launch_warp_fuse(kf_grid can, kf_grid live, kf_field psi, const DevParams &dp,
                        cudaStream_t s) {
  return warp_fuse_impl(can, live, psi, dp, s);
}

int kf_launch_fuse(kf_grid can, kf_grid other, cudaStream_t s) {
  k_fuse<<<blocks_for(can->count), kBlock, 0, s>>>(can->phi, can->w, other->phi, other->w,
                                                   can->count);
  KF_CHECK_LAUNCH("k_fuse");
  return KF_OK;
}

int kf_launch_fuse_warped(kf_grid dst, kf_grid other, kf_field psi, const DevParams &dp,
                          cudaStream_t s) {
  if (psi->prec == KF_F32)
    k_fuse_warped<float><<<blocks_for(dst->count), kBlock, 0, s>>>(
        dst->phi, dst->w, other->phi, other->w, planes<float>(psi), dst->n[0], dst->n[1],
        dst->n[2], dp.oob_phi);
  else
    k_fuse_warped<double><<<blocks_for(dst->count), kBlock, 0, s>>>(
        dst->phi, dst->w, other->phi, other->w, planes<double>(psi), dst->n[0], dst->n[1],
        dst->n[2], dp.oob_phi);
  KF_CHECK_LAUNCH("k_fuse_warped");
  return KF_OK;
}

int kf_solve_exact(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, int iterations,
                   IterStats *st, cudaStream_t s) {
  if (psi->prec != KF_F64)
    return kf_fail(KF_ERR_INVALID, "KF_SOLVER_EXACT needs a KF_F64 displacement field");
  int rc = kf_field_ensure_pair(psi);
  if (rc) return rc;
  PhiView<double> lv = phi_view<double>(live, live->phi, dp.oob_phi);
  PhiView<double> cv = phi_view<double>(can, can->phi, dp.oob_phi);
  void *buf[2][3] = {{psi->p[0], psi->p[1], psi->p[2]}, {psi->q[0], psi->q[1], psi->q[2]}};
  int *rows = nullptr;
  const int nrows = dp.ny * dp.nz;
  if (dp.trust) {
    rc = kf_field_trust_rows(psi, &rows);
    if (rc) return rc;
    KF_CHECK_CUDA(cudaMemsetAsync(rows, 0x7f, (size_t)nrows * sizeof(int), s));
  }
  for (int it = 0; it < iterations; ++it) {
    void **in = buf[it & 1], **out = buf[(it + 1) & 1];
    PsiView<double, double> fin{(const double *)in[0], (const double *)in[1],
                                (const double *)in[2], dp.nx, dp.ny, dp.nz};
    k_exact_step<<<blocks_for(dp.count), kBlock, 0, s>>>(lv, cv, fin, (double *)out[0],
                                                         (double *)out[1], (double *)out[2], dp,
                                                         st, it, rows);
    if (dp.trust)
      k_exact_trust_rows<<<(unsigned)(((int64_t)nrows * 32 + kBlock - 1) / kBlock), kBlock, 0, s>>>(
          (const double *)in[0], (const double *)in[1], (const double *)in[2], (double *)out[0],
          (double *)out[1], (double *)out[2], rows, dp.nx, nrows);
    KF_CHECK_LAUNCH("k_exact_step");
  }
  return KF_OK;
}

int kf_gradient_ref_launch(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                           const int32_t *voxels, int count, double *out, uint8_t *active,
                           cudaStream_t s) {
  if (count <= 0) return KF_OK;
  unsigned nb = (unsigned)((count + 127) / 128);
  if (psi->prec == KF_F32) {
    PsiView<float, float> f{(const float *)psi->p[0], (const float *)psi->p[1],
                            (const float *)psi->p[2], dp.nx, dp.ny, dp.nz};
    k_gradient_ref<float, float><<<nb, 128, 0, s>>>(phi_view<float>(live, live->phi, dp.oob_phi),
                                                    phi_view<float>(can, can->phi, dp.oob_phi), f,
                                                    dp, voxels, count, out, active);
  } else {
    PsiView<double, double> f{(const double *)psi->p[0], (const double *)psi->p[1],
                              (const double *)psi->p[2], dp.nx, dp.ny, dp.nz};
    k_gradient_ref<double, double><<<nb, 128, 0, s>>>(
        phi_view<double>(live, live->phi, dp.oob_phi), phi_view<double>(can, can->phi, dp.oob_phi),
        f, dp, voxels, count, out, active);
  }
  KF_CHECK_LAUNCH("k_gradient_ref");
  return KF_OK;
}

// ---------------------------------------------------------------------------
// point queries and field updates of the host classes (float64, reference
// order): SDF::getDistance / getWeight / getDistanceAtIndex / getWeightAtIndex
// (SDF.cpp:475-604), DisplacementField::getDisplacementAt / getDisplacementAtf
// / update / operator+ / initializeAllVoxels (DisplacementField.cpp:22-88).
// ---------------------------------------------------------------------------
namespace {

// weights through the same sampler: a PhiView over int32 weights
struct WeightView {
  const int32_t *w;
  int nx, ny, nz;
  __device__ __forceinline__ double at(int x, int y, int z) const {
    if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) return 0.0;
    return (double)w[((int64_t)z * ny + y) * nx + x];
  }
};

__global__ void k_grid_sample(PhiView<double> pv, WeightView wv, const double *__restrict__ pts, int n,
                              double *__restrict__ phi, double *__restrict__ weight) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p0 = pts[3 * i], p1 = pts[3 * i + 1], p2 = pts[3 * i + 2];
  if (phi) phi[i] = phi_sample(pv, p0, p1, p2);
  if (weight) {
    double t0 = p0 - 0.5, t1 = p1 - 0.5, t2 = p2 - 0.5;
    int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
    double v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = wv.at(b0 + (c & 1), b1 + ((c >> 1) & 1), b2 + (c >> 2));
    weight[i] = lerp3(v, t0 - (double)b0, t1 - (double)b1, t2 - (double)b2);
  }
}

__global__ void k_grid_get(PhiView<double> pv, WeightView wv, const int32_t *__restrict__ xyz, int n,
                           double *__restrict__ phi, int64_t *__restrict__ weight) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  if (phi) phi[i] = pv.at(x, y, z);
  if (weight) weight[i] = (int64_t)wv.at(x, y, z);
}

template <typename P>
__global__ void k_field_get(PsiView<double, P> f, const int32_t *__restrict__ xyz, int n,
                            double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[3];
  f.at(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], v);
  out[3 * i] = v[0];
  out[3 * i + 1] = v[1];
  out[3 * i + 2] = v[2];
}

template <typename P>
__global__ void k_field_sample(PsiView<double, P> f, const double *__restrict__ pts, int n,
                               double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[3];
  psi_sample(f, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], v);
  out[3 * i] = v[0];
  out[3 * i + 1] = v[1];
  out[3 * i + 2] = v[2];
}

// serial in list order, so repeated voxels accumulate as in the reference
template <typename P>
__global__ void k_field_add_voxels(P *px, P *py, P *pz, int nx, int ny, const int32_t *__restrict__ xyz,
                                   int n, const double *__restrict__ delta) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int i = 0; i < n; ++i) {
    const int64_t j = (int64_t)xyz[3 * i + 2] * nx * ny + (int64_t)xyz[3 * i + 1] * nx + xyz[3 * i];
    px[j] = (P)((double)px[j] + delta[3 * i]);
    py[j] = (P)((double)py[j] + delta[3 * i + 1]);
    pz[j] = (P)((double)pz[j] + delta[3 * i + 2]);
  }
}

template <typename P>
__global__ void k_field_add(P *px, P *py, P *pz, const P *qx, const P *qy, const P *qz, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  px[i] = px[i] + qx[i];
  py[i] = py[i] + qy[i];
  pz[i] = pz[i] + qz[i];
}

template <typename P>
__global__ void k_field_fill(P *px, P *py, P *pz, P a, P b, P c, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  px[i] = a;
  py[i] = b;
  pz[i] = c;
}

// Host staging of a small query: copy `bytes_in` of host input to the
// device, run `launch(dev_in, dev_out)`, copy `bytes_out` back.
template <typename F>
int small_query(const void *in, size_t bytes_in, void *out, size_t bytes_out, cudaStream_t s, F launch) {
  char *d = nullptr;
  KF_CHECK_CUDA(cudaMallocAsync((void **)&d, bytes_in + bytes_out + 256, s));
  char *dout = d + ((bytes_in + 255) & ~(size_t)255);
  // the buffer is released whatever fails after its allocation; the first
  // error is the one reported
  cudaError_t err = cudaSuccess;
  const char *what = nullptr;
  if (bytes_in) {
    err = cudaMemcpyAsync(d, in, bytes_in, cudaMemcpyDefault, s);
    what = "query input copy";
  }
  if (err == cudaSuccess) {
    launch(d, dout);
    err = cudaGetLastError();
    what = "query kernel";
  }
  if (err == cudaSuccess && bytes_out) {
    err = cudaMemcpyAsync(out, dout, bytes_out, cudaMemcpyDefault, s);
    what = "query output copy";
  }
  const cudaError_t fe = cudaFreeAsync(d, s);
  const cudaError_t se = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return kf_cuda_fail(err, what);
  if (fe != cudaSuccess) return kf_cuda_fail(fe, "cudaFreeAsync of the query buffer");
  if (se != cudaSuccess) return kf_cuda_fail(se, "query");
  return KF_OK;
}

}  // namespace

extern "C" int kf_grid_sample(kf_grid g, const kf_params *p, const double *pts, int n, double *phi,
                              double *weight, void *stream) {
  KF_REQUIRE(g && p && (pts || n == 0), "NULL argument");
  KF_REQUIRE(n >= 0, "n must be >= 0");
  if (n == 0) return KF_OK;
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(g->n, p);
  PhiView<double> pv = phi_view<double>(g, g->phi, dp.oob_phi);
  WeightView wv{g->w, g->n[0], g->n[1], g->n[2]};
  const size_t bi = (size_t)n * 3 * sizeof(double), bo = (size_t)n * sizeof(double);
  std::vector<double> buf(2 * (size_t)n);
  rc = small_query(pts, bi, buf.data(), 2 * bo, kf_stream(stream), [&](char *din, char *dout) {
    double *o = (double *)dout;
    k_grid_sample<<<(n + 127) / 128, 128, 0, kf_stream(stream)>>>(pv, wv, (const double *)din, n, o,
                                                                 o + n);
  });
  if (rc) return rc;
  for (int i = 0; i < n; ++i) {
    if (phi) phi[i] = buf[i];
    if (weight) weight[i] = buf[n + i];
  }
  return KF_OK;
}

extern "C" int kf_grid_get_voxels(kf_grid g, const kf_params *p, const int32_t *xyz, int n,
                                  double *phi, int64_t *weight, void *stream) {
  KF_REQUIRE(g && p && (xyz || n == 0), "NULL argument");
  KF_REQUIRE(n >= 0, "n must be >= 0");
  if (n == 0) return KF_OK;
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(g->n, p);
  PhiView<double> pv = phi_view<double>(g, g->phi, dp.oob_phi);
  WeightView wv{g->w, g->n[0], g->n[1], g->n[2]};
  std::vector<char> buf((size_t)n * 16);
  rc = small_query(xyz, (size_t)n * 3 * sizeof(int32_t), buf.data(), buf.size(), kf_stream(stream),
                   [&](char *din, char *dout) {
                     k_grid_get<<<(n + 127) / 128, 128, 0, kf_stream(stream)>>>(
                         pv, wv, (const int32_t *)din, n, (double *)dout, (int64_t *)(dout + (size_t)n * 8));
                   });
  if (rc) return rc;
  if (phi) memcpy(phi, buf.data(), (size_t)n * 8);
  if (weight) memcpy(weight, buf.data() + (size_t)n * 8, (size_t)n * 8);
  return KF_OK;
}

template <typename P>
static PsiView<double, P> psi_view(kf_field f) {
  return PsiView<double, P>{(const P *)f->p[0], (const P *)f->p[1], (const P *)f->p[2], f->n[0], f->n[1],
                            f->n[2]};
}

extern "C" int kf_field_get_voxels(kf_field f, const int32_t *xyz, int n, double *out, void *stream) {
  KF_REQUIRE(f && (xyz || n == 0) && (out || n == 0), "NULL argument");
  KF_REQUIRE(n >= 0, "n must be >= 0");
  if (n == 0) return KF_OK;
  return small_query(xyz, (size_t)n * 3 * sizeof(int32_t), out, (size_t)n * 3 * sizeof(double),
                     kf_stream(stream), [&](char *din, char *dout) {
                       unsigned nb = (n + 127) / 128;
                       if (f->prec == KF_F32)
                         k_field_get<float><<<nb, 128, 0, kf_stream(stream)>>>(psi_view<float>(f),
                                                                             (const int32_t *)din, n,
                                                                             (double *)dout);
                       else
                         k_field_get<double><<<nb, 128, 0, kf_stream(stream)>>>(psi_view<double>(f),
                                                                              (const int32_t *)din, n,
                                                                              (double *)dout);
                     });
}

extern "C" int kf_field_sample(kf_field f, const double *pts, int n, double *out, void *stream) {
  KF_REQUIRE(f && (pts || n == 0) && (out || n == 0), "NULL argument");
  KF_REQUIRE(n >= 0, "n must be >= 0");
  if (n == 0) return KF_OK;
  return small_query(pts, (size_t)n * 3 * sizeof(double), out, (size_t)n * 3 * sizeof(double),
                     kf_stream(stream), [&](char *din, char *dout) {
                       unsigned nb = (n + 127) / 128;
                       if (f->prec == KF_F32)
                         k_field_sample<float><<<nb, 128, 0, kf_stream(stream)>>>(
                             psi_view<float>(f), (const double *)din, n, (double *)dout);
                       else
                         k_field_sample<double><<<nb, 128, 0, kf_stream(stream)>>>(
                             psi_view<double>(f), (const double *)din, n, (double *)dout);
                     });
}

extern "C" int kf_field_add_voxels(kf_field f, const int32_t *xyz, int n, const double *delta,
                                   void *stream) {
  KF_REQUIRE(f && (xyz || n == 0) && (delta || n == 0), "NULL argument");
  KF_REQUIRE(n >= 0, "n must be >= 0");
  kf_field_written(f);
  for (int i = 0; i < n; ++i) {
    int64_t j = (int64_t)xyz[3 * i + 2] * f->n[0] * f->n[1] + (int64_t)xyz[3 * i + 1] * f->n[0] + xyz[3 * i];
    KF_REQUIRE(j >= 0 && j < f->count, "voxel index outside the displacement field");
  }
  if (n == 0) return KF_OK;
  // The deltas (doubles) follow the coordinates at a 16-byte boundary: n * 12 bytes alone is not
  // 8-byte aligned when n is odd.
  const size_t delta_off = ((size_t)n * 12 + 15) & ~(size_t)15;
  std::vector<char> in(delta_off + (size_t)n * 24);
  memcpy(in.data(), xyz, (size_t)n * 12);
  memcpy(in.data() + delta_off, delta, (size_t)n * 24);
  return small_query(in.data(), in.size(), nullptr, 0, kf_stream(stream), [&](char *din, char *) {
    const int32_t *dx = (const int32_t *)din;
    const double *dd = (const double *)(din + delta_off);
    if (f->prec == KF_F32)
      k_field_add_voxels<float><<<1, 1, 0, kf_stream(stream)>>>((float *)f->p[0], (float *)f->p[1],
                                                                (float *)f->p[2], f->n[0], f->n[1], dx, n, dd);
    else
      k_field_add_voxels<double><<<1, 1, 0, kf_stream(stream)>>>(
          (double *)f->p[0], (double *)f->p[1], (double *)f->p[2], f->n[0], f->n[1], dx, n, dd);
  });
}

extern "C" int kf_field_add(kf_field f, kf_field other, void *stream) {
  KF_REQUIRE(f && other, "NULL argument");
  KF_REQUIRE(f->count == other->count && f->n[0] == other->n[0] && f->n[1] == other->n[1],
             "field sizes differ");
  KF_REQUIRE(f->prec == other->prec, "field precisions differ");
  kf_field_written(f);
  unsigned nb = blocks_for(f->count);
  cudaStream_t s = kf_stream(stream);
  if (f->prec == KF_F32)
    k_field_add<float><<<nb, kBlock, 0, s>>>((float *)f->p[0], (float *)f->p[1], (float *)f->p[2],
                                             (const float *)other->p[0], (const float *)other->p[1],
                                             (const float *)other->p[2], f->count);
  else
    k_field_add<double><<<nb, kBlock, 0, s>>>((double *)f->p[0], (double *)f->p[1], (double *)f->p[2],
                                              (const double *)other->p[0], (const double *)other->p[1],
                                              (const double *)other->p[2], f->count);
  KF_CHECK_LAUNCH("k_field_add");
  return KF_OK;
}

extern "C" int kf_field_fill(kf_field f, const double v[3], void *stream) {
  KF_REQUIRE(f && v, "NULL argument");
  kf_field_written(f);
  unsigned nb = blocks_for(f->count);
  cudaStream_t s = kf_stream(stream);
  if (f->prec == KF_F32)
    k_field_fill<float><<<nb, kBlock, 0, s>>>((float *)f->p[0], (float *)f->p[1], (float *)f->p[2],
                                              (float)v[0], (float)v[1], (float)v[2], f->count);
  else
    k_field_fill<double><<<nb, kBlock, 0, s>>>((double *)f->p[0], (double *)f->p[1], (double *)f->p[2],
                                               v[0], v[1], v[2], f->count);
  KF_CHECK_LAUNCH("k_field_fill");
  return KF_OK;
}

KF_BOUNDS_TU_API(exact)
