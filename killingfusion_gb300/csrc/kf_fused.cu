// Fused float32 psi update (KillingFusion::computeDisplacementField,
// KillingFusion.cpp:248-352, with the gradient of
// KillingFusion::computeEnergyGradient, :399-476) and the CUDA-graph capture
// of the fixed-iteration loop.
//
// An iteration is two passes:
//   k_fused_stream (dense)  streams psi and phi_live and applies the band test
//     of KillingFusion.cpp:272-274.  The warped value phi_live(i + psi(i)) is
//     phi_live(i) itself when psi(i) == 0 (zero interpolation weights), so only
//     voxels that have moved gather their 8 corners.  Voxels outside the band
//     pass psi through; voxels inside are compacted into a list.
//   k_fused_band  evaluates the full gradient for every listed voxel with one
//     warp per voxel: lanes 0-19 load the psi neighbourhood (shared by
//     shuffles), lanes 0-24 each take one of the 25 warped-SDF samples of the
//     gradient and Hessian, lane 25 the warped value, lane 26 phi_can, and the
//     nine derivative sums are warp reductions of +-1-weighted sample
//     differences.
// The band-only solver (KF_SOLVER_BAND) runs the dense pass once: a voxel
// outside the band keeps psi, so its band test keeps failing and the band can
// only shrink.  Each band pass then re-tests its voxels at the new psi and
// hands the survivors to the next iteration; a voxel that leaves the band is
// copied once into the other Jacobi buffer.  Both solvers produce the same psi.
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
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "kf_internal.h"
#include "kf_ref_math.cuh"

using namespace kfref;

namespace {

constexpr int kTX = 32, kTY = 8, kThreads = kTX * kTY;
constexpr int kZSlab = 8;
constexpr int kTile = kThreads * kZSlab;
constexpr int kBandWarps = 8;
constexpr int kBandThreads = 32 * kBandWarps;
constexpr unsigned kFull = 0xffffffffu;

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
  int iter;
  DevParams dp;
  // float copies of the parameters
  float h, alpha, omega_k, gamma_k, omega_s, clamp, eps, voxel, oob, band_hi, band_lo;
};

__device__ __forceinline__ float phi_at(const FusedArgs &a, int x, int y, int z) {
  const DevParams &d = a.dp;
  if (x < 0 || x >= d.nx || y < 0 || y >= d.ny || z < 0 || z >= d.nz) return a.oob;
  return __ldg(a.live + ((int64_t)z * d.ny + y) * d.nx + x);
}

// phi_live at grid coordinate t (SDF::getDistance after its -0.5 shift,
// SDF.cpp:503-524): truncating base, outside corners read MaxSurface+eps.
__device__ __forceinline__ float phi_tri(const FusedArgs &a, float t0, float t1, float t2) {
  int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
  float f0 = t0 - (float)b0, f1 = t1 - (float)b1, f2 = t2 - (float)b2;
  float v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) v[c] = phi_at(a, b0 + (c & 1), b1 + ((c >> 1) & 1), b2 + (c >> 2));
  return lerp3(v, f0, f1, f2);
}

// The warped value of the band test, SDF::getDistance(i, psi) (SDF.cpp:570-575).
__device__ __noinline__ float warped_value(const FusedArgs &a, int x, int y, int z, float p0, float p1,
                                           float p2) {
  return phi_tri(a, (((float)x + p0) + 0.5f) - 0.5f, (((float)y + p1) + 0.5f) - 0.5f,
                 (((float)z + p2) + 0.5f) - 0.5f);
}

// The 25 sub-voxel offsets (units of h) of the cell-centre samples: 0, +-e_k
// (gradient), +-2e_k and +-e_j+-e_k (Hessian), one per lane.
__device__ const signed char kOff25[32][3] = {
    {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},  {0, -1, 0},  {0, 0, 1},  {0, 0, -1},
    {2, 0, 0},   {-2, 0, 0},  {0, 2, 0},   {0, -2, 0}, {0, 0, 2},   {0, 0, -2}, {1, 0, 1},
    {-1, 0, 1},  {0, 1, 1},   {0, -1, 1},  {1, 1, 0},  {-1, 1, 0},  {-1, 0, -1}, {1, 0, -1},
    {0, -1, -1}, {0, 1, -1},  {-1, -1, 0}, {1, -1, 0}, {0, 0, 0},   {0, 0, 0},  {0, 0, 0},
    {0, 0, 0},   {0, 0, 0},   {0, 0, 0},   {0, 0, 0}};

// The 20 psi neighbours of the interior stencil, one per lane: the 19-point
// Killing stencil and the far corner (1,1,1) of the cell-centre cell.
__device__ const signed char kNb20[32][3] = {
    {0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
    {1, 1, 0},  {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, 0, 1},  {1, 0, -1}, {-1, 0, 1},
    {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1},  {0, -1, -1}, {1, 1, 1},  {0, 0, 0},
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},   {0, 0, 0},  {0, 0, 0},  {0, 0, 0},
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0}};
enum { N000 = 0, NXP, NXM, NYP, NYM, NZP, NZM, NXPYP, NXPYM, NXMYP, NXMYM, NXPZP, NXPZM, NXMZP,
       NXMZM, NYPZP, NYPZM, NYMZP, NYMZM, N111 };

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Step d = -alpha * g of an interior voxel (1 <= x,y,z <= n-2), by one warp.
// All lanes return the same d, warped value s, distance gradient g and
// monitored energy e.
__device__ void gradient_warp(const FusedArgs &a, int x, int y, int z, int64_t idx, int lane,
                              float d[3], float &s_out, float g_out[3], float &e_out) {
  const DevParams &dp = a.dp;
  const int64_t sy = dp.nx, sz = (int64_t)dp.nx * dp.ny;
  const float h = a.h;

  // loads: psi at lane's neighbour (lanes 0-19), phi_can (lane 26)
  float q[3] = {0.f, 0.f, 0.f};
  if (lane < 20) {
    int64_t j = idx + __ldg(&kNb20[lane][0]) + __ldg(&kNb20[lane][1]) * sy + __ldg(&kNb20[lane][2]) * sz;
    q[0] = __ldg(a.ix + j);
    q[1] = __ldg(a.iy + j);
    q[2] = __ldg(a.iz + j);
  }
  const float canv = lane == 26 ? __ldg(a.can + idx) : 0.f;

  float kg[3], div[3] = {0.f, 0.f, 0.f}, m[3][7], c0[3], J[3][3];
  const float two_h = 2.f * h, hh = h * h;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[20];
#pragma unroll
    for (int n = 0; n < 20; ++n) v[n] = __shfl_sync(kFull, q[c], n);
    const float v000 = v[N000];
    c0[c] = v000;
    // Killing second differences (DisplacementField.cpp:326-331)
    float xx = two_h * ((v[NXP] - v000) + (v[NXM] - v000));
    float yy = two_h * ((v[NYP] - v000) + (v[NYM] - v000));
    float zz = two_h * ((v[NZP] - v000) + (v[NZM] - v000));
    float xy = hh * ((v[NXPYP] - v[NXPYM]) - (v[NXMYP] - v[NXMYM]));
    float xz = hh * ((v[NXPZP] - v[NXPZM]) - (v[NXMZP] - v[NXMZM]));
    float yz = hh * ((v[NYPZP] - v[NYPZM]) - (v[NYMZP] - v[NYMZM]));
    kg[c] = -2.f * (xx + yy + zz);
    if (c == 0) { div[0] += xx; div[1] += xy; div[2] += xz; }
    if (c == 1) { div[0] += xy; div[1] += yy; div[2] += yz; }
    if (c == 2) { div[0] += xz; div[1] += yz; div[2] += zz; }
    // central differences for the monitored Killing energy
    J[c][0] = 0.5f * (v[NXP] - v[NXM]);
    J[c][1] = 0.5f * (v[NYP] - v[NYM]);
    J[c][2] = 0.5f * (v[NZP] - v[NZM]);
    // moments of the cell [i, i+1]^3 (corner k_abc = psi(i + (a,b,c)))
    float k000 = v000, k100 = v[NXP], k010 = v[NYP], k110 = v[NXPYP];
    float k001 = v[NZP], k101 = v[NXPZP], k011 = v[NYPZP], k111 = v[N111];
    float sx0 = (k000 + k010) + (k001 + k011), sx1 = (k100 + k110) + (k101 + k111);
    float sy0 = (k000 + k100) + (k001 + k101), sy1 = (k010 + k110) + (k011 + k111);
    float sz0 = (k000 + k100) + (k010 + k110), sz1 = (k001 + k101) + (k011 + k111);
    m[c][0] = 0.125f * (sx0 + sx1);
    m[c][1] = 0.25f * (sx1 - sx0);
    m[c][2] = 0.25f * (sy1 - sy0);
    m[c][3] = 0.25f * (sz1 - sz0);
    m[c][4] = 0.5f * ((k110 - k010) - (k100 - k000) + (k111 - k011) - (k101 - k001));
    m[c][5] = 0.5f * ((k101 - k001) - (k100 - k000) + (k111 - k011) - (k110 - k010));
    m[c][6] = 0.5f * ((k011 - k001) - (k010 - k000) + (k111 - k101) - (k110 - k100));
  }
  // Killing gradient: damped divergence term, clamp |g| to killing_clamp, /4h^2
#pragma unroll
  for (int c = 0; c < 3; ++c) kg[c] += (-2.f * a.gamma_k) * div[c];
  {
    float nrm = sqrtf(kg[0] * kg[0] + kg[1] * kg[1] + kg[2] * kg[2]);
    float sc = nrm > a.clamp ? a.clamp / nrm : 1.f;
    float den = 4.f * h * h;
#pragma unroll
    for (int c = 0; c < 3; ++c) kg[c] = kg[c] * sc / den;
  }

  // one trilinear sample per lane: lanes 0-24 the cell-centre samples
  // (SDF::getDistancef at i+0.5+h*o, SDF.cpp:577-582: the half voxel it adds is
  // removed again by getDistance), lanes 25-31 the warped value at i + psi(i)
  const int o0 = __ldg(&kOff25[lane][0]), o1 = __ldg(&kOff25[lane][1]), o2 = __ldg(&kOff25[lane][2]);
  float t[3];
  if (lane < 25) {
    const float of[3] = {(float)o0, (float)o1, (float)o2};
    const float base[3] = {(float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float lin = of[0] * m[c][1] + of[1] * m[c][2] + of[2] * m[c][3];
      float quad = of[0] * of[1] * m[c][4] + of[0] * of[2] * m[c][5] + of[1] * of[2] * m[c][6];
      t[c] = (base[c] + h * of[c]) + (m[c][0] + h * (lin + h * quad));
    }
  } else {
    t[0] = (((float)x + c0[0]) + 0.5f) - 0.5f;
    t[1] = (((float)y + c0[1]) + 0.5f) - 0.5f;
    t[2] = (((float)z + c0[2]) + 0.5f) - 0.5f;
  }
  const float f = phi_tri(a, t[0], t[1], t[2]);
  const float f0 = __shfl_sync(kFull, f, 0);
  const float s = __shfl_sync(kFull, f, 25);
  const float cv = __shfl_sync(kFull, canv, 26);
  // derivative stencils on sample differences (the constant f0 cancels):
  // gradient +-1 on +-e_k, Hessian +1 on +-2e_k, o_j*o_k on the diagonals
  const float df = lane < 25 ? f - f0 : 0.f;
  const int nzc = (o0 != 0) + (o1 != 0) + (o2 != 0);
  const int amax = max(abs(o0), max(abs(o1), abs(o2)));
  const bool first = nzc == 1 && amax == 1, second = nzc == 1 && amax == 2;
  float gx = warp_sum(first ? (float)o0 * df : 0.f);
  float gy = warp_sum(first ? (float)o1 * df : 0.f);
  float gz = warp_sum(first ? (float)o2 * df : 0.f);
  float hxx = warp_sum(second && o0 ? df : 0.f);
  float hyy = warp_sum(second && o1 ? df : 0.f);
  float hzz = warp_sum(second && o2 ? df : 0.f);
  float hxy = warp_sum(nzc == 2 && !o2 ? (float)(o0 * o1) * df : 0.f);
  float hxz = warp_sum(nzc == 2 && !o1 ? (float)(o0 * o2) * df : 0.f);
  float hyz = warp_sum(nzc == 2 && !o0 ? (float)(o1 * o2) * df : 0.f);
  const float inv2h = 1.f / (2.f * h), inv4hh = 1.f / (4.f * h * h);
  const float g[3] = {gx * inv2h, gy * inv2h, gz * inv2h};
  hxx *= inv4hh; hyy *= inv4hh; hzz *= inv4hh; hxy *= inv4hh; hxz *= inv4hh; hyz *= inv4hh;

  float grad[3] = {0.f, 0.f, 0.f};
  float e = 0.f;
  if (dp.use_data) {
    float r = (s - cv) / a.voxel;
#pragma unroll
    for (int k = 0; k < 3; ++k) grad[k] += r * g[k];
    e += 0.5f * r * r;
  }
  if (dp.use_killing) {
#pragma unroll
    for (int k = 0; k < 3; ++k) grad[k] += kg[k] * a.omega_k;
    float fr = 0.f, tr = 0.f;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        fr += J[p][k] * J[p][k];
        tr += J[p][k] * J[k][p];
      }
    e += a.omega_k * (fr + a.gamma_k * tr);
  }
  const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
  if (dp.use_levelset) {
    float hg0 = hxx * g[0] + hxy * g[1] + hxz * g[2];
    float hg1 = hxy * g[0] + hyy * g[1] + hyz * g[2];
    float hg2 = hxz * g[0] + hyz * g[1] + hzz * g[2];
    float sc = (gn - 1.f) / (gn + a.eps) * a.omega_s;
    grad[0] += hg0 * sc;
    grad[1] += hg1 * sc;
    grad[2] += hg2 * sc;
    float r = gn / a.voxel - 1.f;
    e += a.omega_s * 0.5f * r * r;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    d[k] = -a.alpha * grad[k];
    g_out[k] = g[k];
  }
  s_out = s;
  e_out = e;
}

// Generic reference-order gradient for the outer shell (one thread).
__device__ __noinline__ void gradient_generic(const FusedArgs &a, int x, int y, int z, float d[3],
                                              float &s_out, float g_out[3], float &e_out) {
  const DevParams &dp = a.dp;
  PhiView<float> lv{a.live, dp.nx, dp.ny, dp.nz, a.oob};
  PhiView<float> cv{a.can, dp.nx, dp.ny, dp.nz, a.oob};
  PsiView<float, float> f{a.ix, a.iy, a.iz, dp.nx, dp.ny, dp.nz};
  TParams<float> tp(dp);
  float g[3];
  energy_gradient(lv, cv, f, tp, x, y, z, g);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = -tp.alpha * g[k];
  s_out = warped_distance(lv, f, x, y, z);
  distance_gradient(lv, f, tp.delta_size, x, y, z, g_out);
  e_out = monitor_energy(a.ix, a.iy, a.iz, dp.nx, dp.ny, dp.nz, x, y, z, s_out, cv.at(x, y, z),
                         g_out, dp);
}

__device__ __forceinline__ void voxel_xyz(const DevParams &dp, int64_t i, int &x, int &y, int &z) {
  const int64_t sz = (int64_t)dp.nx * dp.ny;
  z = (int)(i / sz);
  int64_t r = i - (int64_t)z * sz;
  y = (int)(r / dp.nx);
  x = (int)(r - (int64_t)y * dp.nx);
}

// Dense pass: stream the slab, pass psi through outside the band, list the
// band voxels (st[iter].list counts them).
__global__ void __launch_bounds__(kThreads) k_fused_stream(FusedArgs a, int *__restrict__ list) {
  if (iteration_gated(a.st, a.iter, a.dp)) {
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
      a.st[a.iter].skipped = 1;
    return;
  }
  __shared__ int queue[kTile];
  __shared__ int qn, qbase;
  const DevParams &dp = a.dp;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  const int x = blockIdx.x * kTX + threadIdx.x;
  const int y = blockIdx.y * kTY + threadIdx.y;
  const int z0 = blockIdx.z * kZSlab;
  if (tid == 0) qn = 0;
  __syncthreads();
  const bool col = x < dp.nx && y < dp.ny;
  const int64_t sz = (int64_t)dp.nx * dp.ny;
  const int64_t base = ((int64_t)z0 * dp.ny + y) * dp.nx + x;
  float px[kZSlab], py[kZSlab], pz[kZSlab], ph[kZSlab];
#pragma unroll
  for (int j = 0; j < kZSlab; ++j) {
    bool ok = col && (z0 + j) < dp.nz;
    int64_t i = base + j * sz;
    px[j] = ok ? __ldcs(a.ix + i) : 0.f;
    py[j] = ok ? __ldcs(a.iy + i) : 0.f;
    pz[j] = ok ? __ldcs(a.iz + i) : 0.f;
    ph[j] = ok ? __ldg(a.live + i) : 0.f;
  }
#pragma unroll
  for (int j = 0; j < kZSlab; ++j) {
    int z = z0 + j;
    if (!col || z >= dp.nz) continue;
    int64_t i = base + j * sz;
    float s = ph[j];
    // psi == 0 samples its own cell with zero weights: phi_live(i) exactly
    if (px[j] != 0.f || py[j] != 0.f || pz[j] != 0.f) s = warped_value(a, x, y, z, px[j], py[j], pz[j]);
    if (in_band(s, a.band_hi, a.band_lo)) {
      queue[atomicAdd(&qn, 1)] = (int)i;
    } else {
      __stcs(a.ox + i, px[j]);
      __stcs(a.oy + i, py[j]);
      __stcs(a.oz + i, pz[j]);
    }
  }
  __syncthreads();
  if (tid == 0 && qn) qbase = (int)atomicAdd(&a.st[a.iter].list, (unsigned)qn);
  __syncthreads();
  for (int k = tid; k < qn; k += kThreads) list[qbase + k] = queue[k];
}

// Band pass: one warp per listed voxel.  kCarry: re-test the band at the new
// psi and list the survivors for the next iteration (list_out, counted in
// st[iter+1].list); a listed entry ~i marks a voxel that left the band, whose
// value is copied into the output buffer.
template <bool kCarry>
__global__ void __launch_bounds__(kBandThreads) k_fused_band(FusedArgs a, const int *__restrict__ list_in,
                                                             int *__restrict__ list_out) {
  if (iteration_gated(a.st, a.iter, a.dp)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st[a.iter].skipped = 1;
    return;
  }
  const DevParams &dp = a.dp;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nq = (int)a.st[a.iter].list;
  const int total_warps = gridDim.x * kBandWarps;
  const int rounds = (nq + total_warps - 1) / total_warps;
  __shared__ int s_next[kBandWarps];
  float maxd = 0.f;
  double energy = 0.0;
  unsigned active = 0;
  bool diverged = false;
  for (int r = 0; r < rounds; ++r) {
    const int k = (r * gridDim.x + blockIdx.x) * kBandWarps + warp;
    int next = INT32_MIN;  // entry this warp hands to the next iteration
    if (k < nq) {
      const int e = list_in[k];
      if (e < 0) {
        if (lane == 0) {  // left the band last iteration: settle both buffers
          const int64_t i = ~e;
          a.ox[i] = a.ix[i];
          a.oy[i] = a.iy[i];
          a.oz[i] = a.iz[i];
        }
      } else {
        const int64_t i = e;
        int x, y, z;
        voxel_xyz(dp, i, x, y, z);
        float d[3], s, g[3], en;
        const bool interior = x >= 1 && y >= 1 && z >= 1 && x <= dp.nx - 2 && y <= dp.ny - 2 &&
                              z <= dp.nz - 2;
        if (interior) {
          gradient_warp(a, x, y, z, i, lane, d, s, g, en);
        } else {
          if (lane == 0) gradient_generic(a, x, y, z, d, s, g, en);
#pragma unroll
          for (int c = 0; c < 3; ++c) d[c] = __shfl_sync(kFull, d[c], 0);
        }
        if (lane == 0) {
          const float p0 = a.ix[i], p1 = a.iy[i], p2 = a.iz[i];
          if (!isfinite(p0) || !isfinite(p1) || !isfinite(p2)) diverged = true;
          const float n0 = p0 + d[0], n1 = p1 + d[1], n2 = p2 + d[2];
          a.ox[i] = n0;
          a.oy[i] = n1;
          a.oz[i] = n2;
          maxd = fmaxf(maxd, sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
          energy += (double)en;
          ++active;
          if (kCarry) {
            const float s1 = warped_value(a, x, y, z, n0, n1, n2);
            next = in_band(s1, a.band_hi, a.band_lo) ? e : ~e;
          }
        }
      }
    }
    if (kCarry) {
      if (lane == 0) s_next[warp] = next;
      __syncthreads();
      if (threadIdx.x == 0) {
        int cnt = 0;
        for (int w = 0; w < kBandWarps; ++w) cnt += s_next[w] != INT32_MIN;
        if (cnt) {
          int b = (int)atomicAdd(&a.st[a.iter + 1].list, (unsigned)cnt);
          for (int w = 0; w < kBandWarps; ++w)
            if (s_next[w] != INT32_MIN) list_out[b++] = s_next[w];
        }
      }
      __syncthreads();
    }
  }
  reduce_iter_stats<kBandThreads>(a.st + a.iter, active, maxd, energy, diverged);
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

// A captured iteration loop, valid for one set of buffers and parameters.
struct FusedGraph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
  const void *key_ptr[10] = {};
  int iterations = 0;
  bool band_only = false;
  DevParams dp;
};

void kf_fused_graph_destroy(FusedGraph *g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->capture) cudaStreamDestroy(g->capture);
  delete g;
}

static void launch_iterations(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                              int iterations, IterStats *st, int *lists, bool band_only,
                              cudaStream_t s) {
  dim3 block(kTX, kTY);
  const unsigned band_blocks = (unsigned)kf_num_sms() * 8;
  dim3 grid((dp.nx + kTX - 1) / kTX, (dp.ny + kTY - 1) / kTY, (dp.nz + kZSlab - 1) / kZSlab);
  FusedArgs a = make_args(live, can, dp, st);
  void *buf[2][3] = {{psi->p[0], psi->p[1], psi->p[2]}, {psi->q[0], psi->q[1], psi->q[2]}};
  int *lst[2] = {lists, lists + dp.count};
  for (int it = 0; it < iterations; ++it) {
    void **in = buf[it & 1], **out = buf[(it + 1) & 1];
    a.ix = (const float *)in[0];
    a.iy = (const float *)in[1];
    a.iz = (const float *)in[2];
    a.ox = (float *)out[0];
    a.oy = (float *)out[1];
    a.oz = (float *)out[2];
    a.iter = it;
    if (!band_only) {
      k_fused_stream<<<grid, block, 0, s>>>(a, lst[0]);
      k_fused_band<false><<<band_blocks, kBandThreads, 0, s>>>(a, lst[0], nullptr);
    } else {
      if (it == 0) k_fused_stream<<<grid, block, 0, s>>>(a, lst[0]);
      k_fused_band<true><<<band_blocks, kBandThreads, 0, s>>>(a, lst[it & 1], lst[(it + 1) & 1]);
    }
  }
}

int kf_solve_fused(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, int iterations,
                   IterStats *st, bool band_only, cudaStream_t s) {
  int rc = kf_field_ensure_pair(psi);
  if (rc) return rc;
  rc = kf_field_band_list(psi, &psi->band);
  if (rc) return rc;
  const void *key[10] = {live->phi, can->phi, psi->p[0], psi->p[1], psi->p[2],
                         psi->q[0], psi->q[1], psi->q[2], st, psi->band};
  FusedGraph *g = psi->graph;
  bool hit = g && g->iterations == iterations && g->band_only == band_only &&
             memcmp(g->key_ptr, key, sizeof(key)) == 0 && memcmp(&g->dp, &dp, sizeof(dp)) == 0;
  if (!hit) {
    kf_fused_graph_destroy(psi->graph);
    psi->graph = g = new FusedGraph();
    KF_CHECK_CUDA(cudaStreamCreateWithFlags(&g->capture, cudaStreamNonBlocking));
    cudaGraph_t graph;
    KF_CHECK_CUDA(cudaStreamBeginCapture(g->capture, cudaStreamCaptureModeThreadLocal));
    launch_iterations(live, can, psi, dp, iterations, st, psi->band, band_only, g->capture);
    cudaError_t le = cudaGetLastError();
    KF_CHECK_CUDA(cudaStreamEndCapture(g->capture, &graph));
    if (le != cudaSuccess) {
      cudaGraphDestroy(graph);
      return kf_cuda_fail(le, "fused kernel launch during capture");
    }
    cudaError_t ie = cudaGraphInstantiate(&g->exec, graph, 0);
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
