// Device-side pieces of the fused float32 psi iteration, shared by the
// single-grid solver (kf_fused.cu) and the batched solver (kf_batch.cu): the
// argument block, the gradient of one band voxel (one thread with closed-form
// stencils for the interior, reference-order form for the outer shell), the
// dense passes and the band-voxel update.  Included once per translation unit (internal
// linkage).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <type_traits>

#include "kf_bounds.cuh"
#include "kf_internal.h"
#include "kf_ref_math.cuh"

namespace {

using namespace kfref;

constexpr int kTX = 32, kTY = 8, kThreads = kTX * kTY;
constexpr int kZSlab = 8;
// CTAs of the batch's band pass: 256 threads (chunks of 256 voxels per problem)
constexpr int kBandWarps = 8;
constexpr int kBandThreads = 32 * kBandWarps;
// CTAs of the single-grid band pass and the per-voxel schedule: 64 threads,
// 8 resident per SM (the register file at 128 registers), so that a small
// band -- a few thousand voxels taken in list order -- spreads over all the
// SMs instead of filling a few
constexpr int kLaneWarps = 2;
constexpr int kLaneThreads = 32 * kLaneWarps;
constexpr int kLaneBlocksPerSM = 8;

struct FusedArgs {
  const float *__restrict__ live;
  const float *__restrict__ can;
  const float *__restrict__ ix;
  const float *__restrict__ iy;
  const float *__restrict__ iz;
  float *__restrict__ ox;
  float *__restrict__ oy;
  float *__restrict__ oz;
  IterStats *st;
  int *rows;  // trust-region step: first failed x per row, this iteration
  int iter;
  DevParams dp;
  // float copies of the parameters
  float h, alpha, omega_k, gamma_k, omega_s, clamp, eps, voxel, oob, band_hi, band_lo;
};

// Float arithmetic with every rounding spelled out: fm, fa and fsb never
// merge into a fused multiply-add, ff always is one.  The band update is
// inlined into several kernels (the single-grid band pass, the batch, the
// per-voxel schedule) whose surrounding code differs, and the compiler's
// choice of which products to fuse may follow that code; with the roundings
// explicit, a batch gives each problem the bits its own solve gives.
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsb(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ff(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// utils.h:6-25 in float with explicit roundings: a * (1 - t) + b * t, along
// x, then y, then z.
__device__ __forceinline__ float lerp1f(float a, float b, float t) { return ff(b, t, fm(a, fsb(1.f, t))); }
__device__ __forceinline__ float lerp3f(const float v[8], float x, float y, float z) {
  const float s = lerp1f(lerp1f(v[0], v[1], x), lerp1f(v[2], v[3], x), y);
  const float t = lerp1f(lerp1f(v[4], v[5], x), lerp1f(v[6], v[7], x), y);
  return lerp1f(s, t, z);
}

__device__ __forceinline__ float phi_at(const FusedArgs &a, int x, int y, int z) {
  const DevParams &d = a.dp;
  if (x < 0 || x >= d.nx || y < 0 || y >= d.ny || z < 0 || z >= d.nz) return a.oob;
  return __ldg(a.live + ((int64_t)z * d.ny + y) * d.nx + x);
}

// phi_live at grid coordinate t (SDF::getDistance after its -0.5 shift,
// SDF.cpp:503-524): truncating base, outside corners read MaxSurface+eps.
__device__ __forceinline__ float phi_tri(const FusedArgs &a, float t0, float t1, float t2) {
  const DevParams &d = a.dp;
  int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
  float f0 = fsb(t0, (float)b0), f1 = fsb(t1, (float)b1), f2 = fsb(t2, (float)b2);
  float v[8];
  if ((unsigned)b0 < (unsigned)(d.nx - 1) && (unsigned)b1 < (unsigned)(d.ny - 1) &&
      (unsigned)b2 < (unsigned)(d.nz - 1)) {
    // all eight corners inside: one address, constant strides
    const float *p = a.live + ((int64_t)b2 * d.ny + b1) * d.nx + b0;
    const int64_t sy = d.nx, sz = (int64_t)d.nx * d.ny;
    v[0] = __ldg(p);
    v[1] = __ldg(p + 1);
    v[2] = __ldg(p + sy);
    v[3] = __ldg(p + sy + 1);
    v[4] = __ldg(p + sz);
    v[5] = __ldg(p + sz + 1);
    v[6] = __ldg(p + sz + sy);
    v[7] = __ldg(p + sz + sy + 1);
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = phi_at(a, b0 + (c & 1), b1 + ((c >> 1) & 1), b2 + (c >> 2));
  }
  return lerp3f(v, f0, f1, f2);
}

// The warped value of the band test, SDF::getDistance(i, psi) (SDF.cpp:570-575).
__device__ __noinline__ float warped_value(const FusedArgs &a, int x, int y, int z, float p0, float p1,
                                           float p2) {
  return phi_tri(a, (((float)x + p0) + 0.5f) - 0.5f, (((float)y + p1) + 0.5f) - 0.5f,
                 (((float)z + p2) + 0.5f) - 0.5f);
}

// The 20 psi neighbours of the interior stencil (nb20_off): the 19-point
// Killing stencil and the far corner (1,1,1) of the cell-centre cell.
enum { N000 = 0, NXP, NXM, NYP, NYM, NZP, NZM, NXPYP, NXPYM, NXMYP, NXMYM, NXPZP, NXPZM, NXMZP,
       NXMZM, NYPZP, NYPZM, NYMZP, NYMZM, N111 };

// The stencil offsets as compile-time functions, so that a loop over them
// unrolls into constant-offset code.  off25_at: the 25 sub-voxel offsets
// (units of h) of the cell-centre samples: 0, +-e_k (gradient), +-2e_k and
// +-e_j+-e_k (Hessian).
__host__ __device__ constexpr int nb20_off(int n, int c) {
  constexpr signed char t[20][3] = {
      {0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
      {1, 1, 0},  {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, 0, 1},  {1, 0, -1}, {-1, 0, 1},
      {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1},  {0, -1, -1}, {1, 1, 1}};
  return t[n][c];
}
__host__ __device__ constexpr int off25_at(int j, int c) {
  constexpr signed char t[25][3] = {
      {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},  {0, -1, 0},  {0, 0, 1},  {0, 0, -1},
      {2, 0, 0},   {-2, 0, 0},  {0, 2, 0},   {0, -2, 0}, {0, 0, 2},   {0, 0, -2}, {1, 0, 1},
      {-1, 0, 1},  {0, 1, 1},   {0, -1, 1},  {1, 1, 0},  {-1, 1, 0},  {-1, 0, -1}, {1, 0, -1},
      {0, -1, -1}, {0, 1, -1},  {-1, -1, 0}, {1, -1, 0}};
  return t[j][c];
}

// One interior voxel (1 <= x,y,z <= n-2) by one thread: returns the step
// d = -alpha * g, the warped value s at i + psi(i), the monitored energy e
// and psi(i) in c0.  The thread loads the 20 psi neighbours of each
// component and takes all 26 samples, whose offsets are compile-time
// constants, reading the 25 cell-centre samples' corners once when they
// share one cell; the derivative stencils are the reference's
// (SDF.cpp:726-744, 867-881).  Measured against groups of lanes per voxel that shared the
// neighbours by shuffles (and so replicated the Killing stencil and the
// moments on every lane): one thread per voxel runs 112 warp instructions
// per band voxel against 291 for 4 lanes, 1.7x the band voxels/s on
// band-heavy grids, 2.3x on a 64-problem batch, 3 % faster on the dense
// 256^3 iteration; 4 lanes had been 1.32x 8 lanes and 2x 16.
// How a kernel reads psi: through the read-only path (psi not written during
// the kernel), through L2 only (ld.global.cg; the per-voxel schedule, which
// writes psi in place), or through L1 and L2 (ld.global.ca; the persistent
// passes, which write psi between iterations and order those writes with
// the fences of their grid-wide barrier -- the read-only path is outside
// that ordering, L1 is not).
enum PsiLoad { kPsiReadOnly = 0, kPsiL2 = 1, kPsiL1 = 2 };

template <int kLoad>
__device__ __forceinline__ float load_psi(const float *p) {
  if constexpr (kLoad == kPsiL2)
    return __ldcg(p);
  else if constexpr (kLoad == kPsiL1)
    return __ldca(p);
  else
    return __ldg(p);
}

template <int kLoad = kPsiReadOnly>
__device__ __forceinline__ void gradient_lane(const FusedArgs &a, int x, int y, int z, int64_t idx, float d[3],
                                              float &s_out, float &e_out, float c0[3]) {
  const DevParams &dp = a.dp;
  const int64_t sy = dp.nx, sz = (int64_t)dp.nx * dp.ny;
  const float h = a.h;
  const float *planes[3] = {a.ix, a.iy, a.iz};
  float kg[3], div[3] = {0.f, 0.f, 0.f}, m[3][7], J[3][3];
  const float two_h = fm(2.f, h), hh = fm(h, h);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float *p = planes[c] + idx;
    float v[20];
#pragma unroll
    for (int n = 0; n < 20; ++n) {
      const float *q = p + nb20_off(n, 0) + nb20_off(n, 1) * sy + nb20_off(n, 2) * sz;
      v[n] = load_psi<kLoad>(q);
    }
    const float v000 = v[N000];
    c0[c] = v000;
    // Killing second differences (DisplacementField.cpp:326-331)
    const float xx = fm(two_h, fa(fsb(v[NXP], v000), fsb(v[NXM], v000)));
    const float yy = fm(two_h, fa(fsb(v[NYP], v000), fsb(v[NYM], v000)));
    const float zz = fm(two_h, fa(fsb(v[NZP], v000), fsb(v[NZM], v000)));
    const float xy = fm(hh, fsb(fsb(v[NXPYP], v[NXPYM]), fsb(v[NXMYP], v[NXMYM])));
    const float xz = fm(hh, fsb(fsb(v[NXPZP], v[NXPZM]), fsb(v[NXMZP], v[NXMZM])));
    const float yz = fm(hh, fsb(fsb(v[NYPZP], v[NYPZM]), fsb(v[NYMZP], v[NYMZM])));
    kg[c] = fm(-2.f, fa(fa(xx, yy), zz));
    if (c == 0) { div[0] = fa(div[0], xx); div[1] = fa(div[1], xy); div[2] = fa(div[2], xz); }
    if (c == 1) { div[0] = fa(div[0], xy); div[1] = fa(div[1], yy); div[2] = fa(div[2], yz); }
    if (c == 2) { div[0] = fa(div[0], xz); div[1] = fa(div[1], yz); div[2] = fa(div[2], zz); }
    J[c][0] = fm(0.5f, fsb(v[NXP], v[NXM]));
    J[c][1] = fm(0.5f, fsb(v[NYP], v[NYM]));
    J[c][2] = fm(0.5f, fsb(v[NZP], v[NZM]));
    // moments of the cell [i, i+1]^3 (corner k_abc = psi(i + (a,b,c)))
    const float k000 = v000, k100 = v[NXP], k010 = v[NYP], k110 = v[NXPYP];
    const float k001 = v[NZP], k101 = v[NXPZP], k011 = v[NYPZP], k111 = v[N111];
    const float sx0 = fa(fa(k000, k010), fa(k001, k011)), sx1 = fa(fa(k100, k110), fa(k101, k111));
    const float sy0 = fa(fa(k000, k100), fa(k001, k101)), sy1 = fa(fa(k010, k110), fa(k011, k111));
    const float sz0 = fa(fa(k000, k100), fa(k010, k110)), sz1 = fa(fa(k001, k101), fa(k011, k111));
    m[c][0] = fm(0.125f, fa(sx0, sx1));
    m[c][1] = fm(0.25f, fsb(sx1, sx0));
    m[c][2] = fm(0.25f, fsb(sy1, sy0));
    m[c][3] = fm(0.25f, fsb(sz1, sz0));
    m[c][4] = fm(0.5f, fsb(fa(fsb(fsb(k110, k010), fsb(k100, k000)), fsb(k111, k011)), fsb(k101, k001)));
    m[c][5] = fm(0.5f, fsb(fa(fsb(fsb(k101, k001), fsb(k100, k000)), fsb(k111, k011)), fsb(k110, k010)));
    m[c][6] = fm(0.5f, fsb(fa(fsb(fsb(k011, k001), fsb(k010, k000)), fsb(k111, k101)), fsb(k110, k100)));
  }
  // Killing gradient: damped divergence term, clamp |g| to killing_clamp, /4h^2
  const float m2g = fm(-2.f, a.gamma_k);
#pragma unroll
  for (int c = 0; c < 3; ++c) kg[c] = ff(m2g, div[c], kg[c]);
  {
    const float nrm = sqrtf(ff(kg[2], kg[2], ff(kg[1], kg[1], fm(kg[0], kg[0]))));
    const float sc = nrm > a.clamp ? a.clamp / nrm : 1.f;
    const float den = fm(fm(4.f, h), h);
#pragma unroll
    for (int c = 0; c < 3; ++c) kg[c] = fm(kg[c], sc) / den;
  }
  // the 25 cell-centre samples and the warped value at i + psi(i)
  const float base[3] = {fa((float)x, 0.5f), fa((float)y, 0.5f), fa((float)z, 0.5f)};
  // Shared corner cell.  Along axis c every sample lies within
  // h * (2 + 2 (|m1| + |m2| + |m3|) + h (|m4| + |m5| + |m6|)) of the centre
  // sample base + m0: the offsets are at most 2 and the products of the
  // mixed samples' offsets are +-1.  When that interval, widened for the
  // roundings of the positions (1e-3 voxel plus 2^-20 of the coordinate,
  // several float ulps of it), has one truncated base on every axis and
  // that cell is inside the grid, the 25 samples read the same eight
  // corners: they are loaded once, and each sample interpolates them with
  // its own fractions, the arithmetic phi_tri does after loading them
  // itself.
  int cb[3];
  bool shared = true;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float m1 = fabsf(m[c][1]) + fabsf(m[c][2]) + fabsf(m[c][3]);
    const float m2 = fabsf(m[c][4]) + fabsf(m[c][5]) + fabsf(m[c][6]);
    const float ctr = fa(base[c], m[c][0]);
    const float r = h * (2.f + 2.f * m1 + h * m2) + 1e-3f + fabsf(ctr) * 0x1p-20f;
    const float lo = ctr - r, hi = ctr + r;
    const int b = (int)lo;
    const int n = c == 0 ? dp.nx : (c == 1 ? dp.ny : dp.nz);
    shared = shared && lo >= 0.f && (int)hi == b && (unsigned)b < (unsigned)(n - 1);
    cb[c] = b;
  }
  // sample j's position (SDF::getDistancef at i+0.5+h*o; the half voxel it
  // adds is removed again by getDistance): psi~ there is the cell's
  // trilinear form in its moments, terms with a zero offset dropped at
  // compile time
  auto position = [&](int j, float t[3]) {
    const int o0 = off25_at(j, 0), o1 = off25_at(j, 1), o2 = off25_at(j, 2);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float lin = 0.f, quad = 0.f;
      if (o0) lin = ff((float)o0, m[c][1], lin);
      if (o1) lin = ff((float)o1, m[c][2], lin);
      if (o2) lin = ff((float)o2, m[c][3], lin);
      if (o0 * o1) quad = ff((float)(o0 * o1), m[c][4], quad);
      if (o0 * o2) quad = ff((float)(o0 * o2), m[c][5], quad);
      if (o1 * o2) quad = ff((float)(o1 * o2), m[c][6], quad);
      const int oc = c == 0 ? o0 : (c == 1 ? o1 : o2);
      t[c] = fa(fa(base[c], fm(h, (float)oc)), ff(h, ff(h, quad, lin), m[c][0]));
    }
  };
  float f[25];
  if (shared) {
    const float *p = a.live + ((int64_t)cb[2] * dp.ny + cb[1]) * dp.nx + cb[0];
    float cell[8];
    cell[0] = __ldg(p);
    cell[1] = __ldg(p + 1);
    cell[2] = __ldg(p + sy);
    cell[3] = __ldg(p + sy + 1);
    cell[4] = __ldg(p + sz);
    cell[5] = __ldg(p + sz + 1);
    cell[6] = __ldg(p + sz + sy);
    cell[7] = __ldg(p + sz + sy + 1);
#pragma unroll
    for (int j = 0; j < 25; ++j) {
      float t[3];
      position(j, t);
      f[j] = lerp3f(cell, fsb(t[0], (float)cb[0]), fsb(t[1], (float)cb[1]), fsb(t[2], (float)cb[2]));
    }
  } else {
#pragma unroll
    for (int j = 0; j < 25; ++j) {
      float t[3];
      position(j, t);
      f[j] = phi_tri(a, t[0], t[1], t[2]);
    }
  }
  const float s = phi_tri(a, fsb(fa(fa((float)x, c0[0]), 0.5f), 0.5f), fsb(fa(fa((float)y, c0[1]), 0.5f), 0.5f),
                          fsb(fa(fa((float)z, c0[2]), 0.5f), 0.5f));
  const float cv = __ldg(a.can + idx);
  const float inv2h = 1.f / fm(2.f, h), inv4hh = 1.f / fm(fm(4.f, h), h);
  // SDF.cpp:726-744: (f(p + h e_k) - f(p - h e_k)) / 2h
  const float g[3] = {fm(fsb(f[1], f[2]), inv2h), fm(fsb(f[3], f[4]), inv2h), fm(fsb(f[5], f[6]), inv2h)};
  // SDF.cpp:867-881 on the same samples
  const float f02 = fm(2.f, f[0]);
  const float hxx = fm(fa(fsb(f[7], f02), f[8]), inv4hh);
  const float hyy = fm(fa(fsb(f[9], f02), f[10]), inv4hh);
  const float hzz = fm(fa(fsb(f[11], f02), f[12]), inv4hh);
  const float hxz = fm(fsb(fsb(fa(f[13], f[19]), f[20]), f[14]), inv4hh);
  const float hyz = fm(fsb(fsb(fa(f[15], f[21]), f[22]), f[16]), inv4hh);
  const float hxy = fm(fsb(fsb(fa(f[17], f[23]), f[24]), f[18]), inv4hh);

  float grad[3] = {0.f, 0.f, 0.f};
  float e = 0.f;
  if (dp.use_data) {
    const float r = fsb(s, cv) / a.voxel;
#pragma unroll
    for (int k = 0; k < 3; ++k) grad[k] = ff(r, g[k], grad[k]);
    e = ff(fm(0.5f, r), r, e);
  }
  if (dp.use_killing) {
#pragma unroll
    for (int k = 0; k < 3; ++k) grad[k] = ff(kg[k], a.omega_k, grad[k]);
    float fr = 0.f, tr = 0.f;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        fr = ff(J[p][k], J[p][k], fr);
        tr = ff(J[p][k], J[k][p], tr);
      }
    e = ff(a.omega_k, ff(a.gamma_k, tr, fr), e);
  }
  if (dp.use_levelset) {
    const float gn = sqrtf(ff(g[2], g[2], ff(g[1], g[1], fm(g[0], g[0]))));
    const float hg0 = ff(hxz, g[2], ff(hxy, g[1], fm(hxx, g[0])));
    const float hg1 = ff(hyz, g[2], ff(hyy, g[1], fm(hxy, g[0])));
    const float hg2 = ff(hzz, g[2], ff(hyz, g[1], fm(hxz, g[0])));
    const float sc = fm(fsb(gn, 1.f) / fa(gn, a.eps), a.omega_s);
    grad[0] = ff(hg0, sc, grad[0]);
    grad[1] = ff(hg1, sc, grad[1]);
    grad[2] = ff(hg2, sc, grad[2]);
    const float r = fsb(gn / a.voxel, 1.f);
    e = ff(fm(fm(a.omega_s, 0.5f), r), r, e);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = fm(-a.alpha, grad[k]);
  s_out = s;
  e_out = e;
}

// A psi value read as load_psi<kLoad> reads it: the element type of psi
// views in kernels that write psi themselves.  Same layout as float.
template <int kLoad>
struct PsiElem {
  float v;
  __device__ __forceinline__ operator float() const { return load_psi<kLoad>(&v); }
};

// Generic reference-order gradient for the outer shell (one thread), psi
// read as kLoad says (plain loads for kPsiReadOnly).
template <int kLoad = kPsiReadOnly>
__device__ __noinline__ void gradient_generic(const FusedArgs &a, int x, int y, int z, float d[3],
                                              float &s_out, float &e_out) {
  using P = typename std::conditional<kLoad == kPsiReadOnly, float, PsiElem<kLoad>>::type;
  const DevParams &dp = a.dp;
  const P *px = reinterpret_cast<const P *>(a.ix), *py = reinterpret_cast<const P *>(a.iy),
          *pz = reinterpret_cast<const P *>(a.iz);
  PhiView<float> lv{a.live, dp.nx, dp.ny, dp.nz, a.oob};
  PhiView<float> cv{a.can, dp.nx, dp.ny, dp.nz, a.oob};
  PsiView<float, P> f{px, py, pz, dp.nx, dp.ny, dp.nz};
  TParams<float> tp(dp);
  float g[3], gd[3];
  energy_gradient(lv, cv, f, tp, x, y, z, g);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = -tp.alpha * g[k];
  s_out = warped_distance(lv, f, x, y, z);
  distance_gradient(lv, f, tp.delta_size, x, y, z, gd);
  e_out = monitor_energy(px, py, pz, dp.nx, dp.ny, dp.nz, x, y, z, s_out, cv.at(x, y, z), gd, dp);
}

__device__ __forceinline__ void voxel_xyz(const DevParams &dp, int i, int &x, int &y, int &z) {
  const unsigned plane = (unsigned)dp.nx * (unsigned)dp.ny;
  z = (int)((unsigned)i / plane);
  const unsigned r = (unsigned)i - (unsigned)z * plane;
  y = (int)(r / (unsigned)dp.nx);
  x = (int)(r - (unsigned)y * (unsigned)dp.nx);
}

// Dense pass over one tile (kTX x kTY columns, kSlab planes) of block
// coordinates (bx, by, bz): stream the slab, apply the band test, append the
// band voxels to list (*count counts them).  kPassThrough (ping-pong
// buffers): copy psi of the voxels outside the band to the output buffer;
// without it (psi updated in place) they are only read.
template <bool kPassThrough, int kSlab = kZSlab>
__device__ __forceinline__ void stream_tile(const FusedArgs &a, int bx, int by, int bz,
                                            int *__restrict__ list, unsigned *count) {
  __shared__ int queue[kThreads * kSlab];
  __shared__ int qn, qbase;
  const DevParams &dp = a.dp;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  const int x = bx * kTX + threadIdx.x;
  const int y = by * kTY + threadIdx.y;
  const int z0 = bz * kSlab;
  if (tid == 0) qn = 0;
  __syncthreads();
  const bool col = x < dp.nx && y < dp.ny;
  const int64_t sz = (int64_t)dp.nx * dp.ny;
  const int64_t base = ((int64_t)z0 * dp.ny + y) * dp.nx + x;
  float px[kSlab], py[kSlab], pz[kSlab], ph[kSlab];
#pragma unroll
  for (int j = 0; j < kSlab; ++j) {
    bool ok = col && (z0 + j) < dp.nz;
    int64_t i = base + j * sz;
    px[j] = ok ? __ldcs(a.ix + i) : 0.f;
    py[j] = ok ? __ldcs(a.iy + i) : 0.f;
    pz[j] = ok ? __ldcs(a.iz + i) : 0.f;
    ph[j] = ok ? __ldg(a.live + i) : 0.f;
  }
  // psi == 0 samples its own cell with zero weights: the warped value is
  // phi_live(i) exactly.  Voxels that have moved are tested after the
  // streamed values are dead (their trilinear gather is the rare, long path).
  unsigned moved = 0;
#pragma unroll
  for (int j = 0; j < kSlab; ++j) {
    int z = z0 + j;
    if (!col || z >= dp.nz) continue;
    int64_t i = base + j * sz;
    if (px[j] != 0.f || py[j] != 0.f || pz[j] != 0.f) {
      moved |= 1u << j;
    } else if (in_band(ph[j], a.band_hi, a.band_lo)) {
      const int q = atomicAdd(&qn, 1);
      if (KF_IN_BOUNDS(q, kThreads * kSlab, KF_SITE_STREAM_QUEUE)) queue[q] = (int)i;
    } else if (kPassThrough) {
      __stcs(a.ox + i, 0.f);
      __stcs(a.oy + i, 0.f);
      __stcs(a.oz + i, 0.f);
    }
  }
  while (moved) {
    const int j = __ffs(moved) - 1;
    moved &= moved - 1;
    const int64_t i = base + j * sz;
    const float qx = a.ix[i], qy = a.iy[i], qz = a.iz[i];
    const float s = warped_value(a, x, y, z0 + j, qx, qy, qz);
    if (in_band(s, a.band_hi, a.band_lo)) {
      const int q = atomicAdd(&qn, 1);
      if (KF_IN_BOUNDS(q, kThreads * kSlab, KF_SITE_STREAM_QUEUE)) queue[q] = (int)i;
    } else if (kPassThrough) {
      __stcs(a.ox + i, qx);
      __stcs(a.oy + i, qy);
      __stcs(a.oz + i, qz);
    }
  }
  __syncthreads();
  if (tid == 0 && qn) qbase = (int)atomicAdd(count, (unsigned)qn);
  __syncthreads();
  for (int k = tid; k < min(qn, kThreads * kSlab); k += kThreads)
    if (KF_IN_BOUNDS(qbase + k, dp.count, KF_SITE_STREAM_LIST)) list[qbase + k] = queue[k];
}

// Dense pass over one run of kFlatVoxels consecutive voxels (flat index
// order): thread t streams the float4 groups t and t + kThreads of the run
// from each psi plane and from phi_live, applies the band test and appends
// the band voxels to list (*count counts them).  kPassThrough copies psi of
// all voxels to the output buffer (the band pass overwrites the band
// voxels').  The last count % 4 voxels of the grid are taken by run 0.
constexpr int kFlatGroups = 2;
constexpr int kFlatVoxels = kThreads * kFlatGroups * 4;

__device__ __forceinline__ void flat_test(const FusedArgs &a, int64_t i, float qx, float qy, float qz, float ph,
                                          int *queue, int *qn, unsigned &moved, int bit) {
  if (qx != 0.f || qy != 0.f || qz != 0.f)
    moved |= 1u << bit;
  else if (in_band(ph, a.band_hi, a.band_lo)) {
    const int q = atomicAdd(qn, 1);
    if (KF_IN_BOUNDS(q, kFlatVoxels + 4, KF_SITE_STREAM_QUEUE)) queue[q] = (int)i;
  }
}

// kCheck: the run is only tested, its band voxels are counted in *count and
// not listed (the split schedule's runs without band voxels, where a band
// voxel would break an invariant of the solver).  kPsiZero: psi is zero at
// every voxel (nothing of it is read), so the test reads phi_live alone.
template <bool kPassThrough, bool kCheck = false, bool kPsiZero = false>
__device__ __forceinline__ void stream_flat(const FusedArgs &a, int64_t run, int *__restrict__ list,
                                            unsigned *count, int2 *__restrict__ range = nullptr) {
  __shared__ int queue[kFlatVoxels + 4];
  __shared__ int qn, qbase;
  const DevParams &dp = a.dp;
  const int tid = threadIdx.x;
  if (tid == 0) qn = 0;
  __syncthreads();
  const int64_t n4 = dp.count >> 2;
  const float4 *ix = reinterpret_cast<const float4 *>(a.ix), *iy = reinterpret_cast<const float4 *>(a.iy),
               *iz = reinterpret_cast<const float4 *>(a.iz), *lv = reinterpret_cast<const float4 *>(a.live);
  float4 px[kFlatGroups], py[kFlatGroups], pz[kFlatGroups], ph[kFlatGroups];
  int64_t q[kFlatGroups];
#pragma unroll
  for (int g = 0; g < kFlatGroups; ++g) {
    q[g] = run * (kThreads * kFlatGroups) + g * kThreads + tid;
    const bool ok = q[g] < n4, read_psi = ok && !kPsiZero;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    px[g] = read_psi ? __ldcs(ix + q[g]) : zero;
    py[g] = read_psi ? __ldcs(iy + q[g]) : zero;
    pz[g] = read_psi ? __ldcs(iz + q[g]) : zero;
    ph[g] = ok ? __ldg(lv + q[g]) : zero;
  }
  unsigned moved = 0;  // bit 4g + e: element e of group g has moved
#pragma unroll
  for (int g = 0; g < kFlatGroups; ++g) {
    if (q[g] >= n4) continue;
    const int64_t i = 4 * q[g];
    flat_test(a, i, px[g].x, py[g].x, pz[g].x, ph[g].x, queue, &qn, moved, 4 * g);
    flat_test(a, i + 1, px[g].y, py[g].y, pz[g].y, ph[g].y, queue, &qn, moved, 4 * g + 1);
    flat_test(a, i + 2, px[g].z, py[g].z, pz[g].z, ph[g].z, queue, &qn, moved, 4 * g + 2);
    flat_test(a, i + 3, px[g].w, py[g].w, pz[g].w, ph[g].w, queue, &qn, moved, 4 * g + 3);
    if (kPassThrough) {
      __stcs(reinterpret_cast<float4 *>(a.ox) + q[g], px[g]);
      __stcs(reinterpret_cast<float4 *>(a.oy) + q[g], py[g]);
      __stcs(reinterpret_cast<float4 *>(a.oz) + q[g], pz[g]);
    }
  }
  // the ragged end of the grid, by run 0
  if (run == 0 && tid < (int)(dp.count & 3)) {
    const int64_t i = 4 * n4 + tid;
    const float qx = kPsiZero ? 0.f : a.ix[i], qy = kPsiZero ? 0.f : a.iy[i], qz = kPsiZero ? 0.f : a.iz[i];
    flat_test(a, i, qx, qy, qz, __ldg(a.live + i), queue, &qn, moved, 4 * kFlatGroups);
    if (kPassThrough) {
      a.ox[i] = qx;
      a.oy[i] = qy;
      a.oz[i] = qz;
    }
  }
  // voxels that have moved: the warped value is a trilinear gather
  while (moved) {
    const int bit = __ffs(moved) - 1;
    moved &= moved - 1;
    const int64_t i = bit < 4 * kFlatGroups
                          ? 4 * (run * (kThreads * kFlatGroups) + (bit >> 2) * kThreads + tid) + (bit & 3)
                          : 4 * n4 + tid;
    const unsigned plane = (unsigned)dp.nx * (unsigned)dp.ny, ui = (unsigned)i;
    const int z = (int)(ui / plane);
    const unsigned r = ui - (unsigned)z * plane;
    const int y = (int)(r / (unsigned)dp.nx);
    const int x = (int)(r - (unsigned)y * (unsigned)dp.nx);
    const float s = warped_value(a, x, y, z, a.ix[i], a.iy[i], a.iz[i]);
    if (in_band(s, a.band_hi, a.band_lo)) {
      const int q = atomicAdd(&qn, 1);
      if (KF_IN_BOUNDS(q, kFlatVoxels + 4, KF_SITE_STREAM_QUEUE)) queue[q] = (int)i;
    }
  }
  __syncthreads();
  if (kCheck) {
    if (tid == 0 && qn) atomicAdd(count, (unsigned)qn);
    return;
  }
  if (tid == 0 && qn) qbase = (int)atomicAdd(count, (unsigned)qn);
  __syncthreads();
  for (int k = tid; k < min(qn, kFlatVoxels + 4); k += kThreads)
    if (KF_IN_BOUNDS(qbase + k, dp.count, KF_SITE_STREAM_LIST)) list[qbase + k] = queue[k];
  // where this run's band voxels sit in the list (for the next iteration's
  // write-back of their new psi)
  if (range && tid == 0) *range = make_int2(qn ? qbase : 0, qn);
}

// Appends the voxels `next` (>= 0 on the threads that carry one) of the
// whole block to list_out (of `capacity` entries) with one atomic on
// *count, in thread order; every thread of the block calls it.
template <int kWarps>
__device__ __forceinline__ void block_append(int next, unsigned *count, int *__restrict__ list_out,
                                             int64_t capacity) {
  __shared__ unsigned s_wcnt[kWarps], s_wbase[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool has = next >= 0;
  const unsigned ball = __ballot_sync(0xffffffffu, has);
  if (lane == 0) s_wcnt[warp] = (unsigned)__popc(ball);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = 0;
    for (int w = 0; w < kWarps; ++w) {
      s_wbase[w] = t;
      t += s_wcnt[w];
    }
    const unsigned b = t ? atomicAdd(count, t) : 0u;
    for (int w = 0; w < kWarps; ++w) s_wbase[w] += b;
  }
  __syncthreads();
  if (has) {
    const unsigned pos = s_wbase[warp] + (unsigned)__popc(ball & ((1u << lane) - 1u));
    if (KF_IN_BOUNDS(pos, capacity, KF_SITE_BAND_APPEND)) list_out[pos] = next;
  }
}

// The trust-region step (KillingFusion.cpp:288-314) for the float solvers:
// d = -alpha * g (float) on entry, the accepted step on return; false when
// the step size fell below 1e-7.  The search runs in double, as
// kfref::trust_step: a float position cannot resolve the steps of 1e-7 * g
// that the search reaches before it gives up (near x = 64 one float ulp is
// 7.6e-6 voxel), so in float a step that is too small to move the sample
// reads as "no worse" and the search would accept where the reference
// breaks the row.
__device__ __noinline__ bool trust_step_f(const FusedArgs &a, int x, int y, int z, int64_t i,
                                          const float c[3], float d[3]) {
  const DevParams &dp = a.dp;
  PhiView<double> lv{a.live, dp.nx, dp.ny, dp.nz, dp.oob_phi};
  const double cd[3] = {c[0], c[1], c[2]};
  const double prev = phi_sample(lv, ((double)x + cd[0]) + 0.5, ((double)y + cd[1]) + 0.5,
                                 ((double)z + cd[2]) + 0.5);
  double g[3], dd[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    g[k] = (double)d[k] / -(double)a.alpha;
    dd[k] = -dp.alpha * g[k];
  }
  const bool ok = trust_step(lv, (double)__ldg(a.can + i), prev, x, y, z, cd, g, dp.alpha, dd);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = (float)dd[k];
  return ok;
}

// Update band voxel i (one thread) and write its new psi to entry `slot` of
// the output planes (slot == i for ping-pong buffers; the voxel's list
// position for in-place updates).  The voxel is re-tested with its warped
// value: one outside the band keeps its psi (it left the band in the
// previous iteration).  Returns the voxel for the next iteration's list (-1
// if it left the band) and accumulates the statistics.
// kTrust: the trust-region step (dp.trust set), a separate instantiation so
// that the plain band pass carries no call to it.
// kLoad: how psi is read (PsiLoad); the persistent passes, which write psi
// between iterations, read it with kPsiL1.
template <bool kTrust = false, int kLoad = kPsiReadOnly>
__device__ __forceinline__ int update_band_voxel(const FusedArgs &a, int i, int slot, float &maxd,
                                                 double &energy, unsigned &active, bool &diverged) {
  const DevParams &dp = a.dp;
  if (!KF_IN_BOUNDS(i, dp.count, KF_SITE_BAND_LIST) || !KF_IN_BOUNDS(slot, dp.count, KF_SITE_BAND_LIST)) return -1;
  int x, y, z;
  voxel_xyz(dp, i, x, y, z);
  float d[3] = {0.f, 0.f, 0.f}, s = 0.f, en = 0.f, c0[3] = {0.f, 0.f, 0.f};
  const bool interior = x >= 1 && y >= 1 && z >= 1 && x <= dp.nx - 2 && y <= dp.ny - 2 &&
                        z <= dp.nz - 2;
  if (interior) {
    gradient_lane<kLoad>(a, x, y, z, i, d, s, en, c0);
  } else {
    gradient_generic<kLoad>(a, x, y, z, d, s, en);
    c0[0] = kLoad == kPsiReadOnly ? a.ix[i] : load_psi<kLoad>(a.ix + i);
    c0[1] = kLoad == kPsiReadOnly ? a.iy[i] : load_psi<kLoad>(a.iy + i);
    c0[2] = kLoad == kPsiReadOnly ? a.iz[i] : load_psi<kLoad>(a.iz + i);
  }
  int next = -1;
  if (in_band(s, a.band_hi, a.band_lo)) {
    if (!isfinite(c0[0]) || !isfinite(c0[1]) || !isfinite(c0[2])) diverged = true;
    if (kTrust && !trust_step_f(a, x, y, z, i, c0, d)) {
      // this voxel and the rest of its row keep psi (k_trust_fix)
      atomicMin(a.rows + (z * dp.ny + y), x);
      d[0] = d[1] = d[2] = 0.f;
    }
    a.ox[slot] = c0[0] + d[0];
    a.oy[slot] = c0[1] + d[1];
    a.oz[slot] = c0[2] + d[2];
    maxd = fmaxf(maxd, sqrtf(ff(d[2], d[2], ff(d[1], d[1], fm(d[0], d[0])))));
    energy += en;
    ++active;
    next = i;
  } else {  // left the band: its psi is final, settle the output buffer
    a.ox[slot] = c0[0];
    a.oy[slot] = c0[1];
    a.oz[slot] = c0[2];
  }
  return next;
}

FusedArgs make_args(kf_grid live, kf_grid can, const DevParams &dp, IterStats *st) {
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.live = live->phi;
  a.can = can->phi;
  a.st = st;
  a.dp = dp;
  a.h = (float)dp.delta_size;
  a.alpha = (float)dp.alpha;
  a.omega_k = (float)dp.omega_k;
  a.gamma_k = (float)dp.gamma_k;
  a.omega_s = (float)dp.omega_s;
  a.clamp = (float)dp.killing_clamp;
  a.eps = (float)dp.epsilon;
  a.voxel = (float)dp.voxel_size;
  a.oob = dp.oob_phi_f;
  a.band_hi = dp.band_hi_f;
  a.band_lo = dp.band_lo_f;
  return a;
}

}  // namespace
