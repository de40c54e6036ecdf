// Device-side restatement of the reference's per-voxel arithmetic, templated
// on the arithmetic type T (float or double).  Every function follows the
// operation order of the reference method it names, so that the double
// instantiation, compiled without fused multiply-add (kf_exact.cu), rounds
// exactly as the reference does.  The float instantiation is the arithmetic of
// the plain per-term solver and of the reference-gradient query.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kf_internal.h"

namespace kfref {

// SDF storage (float32 on the device) read as T.  Outside the grid:
// MaxSurfaceVoxelDistance + epsilon (SDF::getDistanceAtIndex, SDF.cpp:475-487).
template <typename T>
struct PhiView {
  const float *phi;
  int nx, ny, nz;
  T oob;
  __device__ __forceinline__ T at(int x, int y, int z) const {
    if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) return oob;
    return (T)__ldg(phi + ((int64_t)z * ny + y) * nx + x);
  }
};

// Displacement field planes of type P read as T.  Only the linear index is
// range-checked, so x/y overflow wraps into the next row or plane
// (DisplacementField::getDisplacementAt, DisplacementField.cpp:22-38).
template <typename T, typename P>
struct PsiView {
  const P *px, *py, *pz;
  int nx, ny, nz;
  __device__ __forceinline__ void at(int x, int y, int z, T out[3]) const {
    int index = z * (nx * ny) + y * nx + x;
    int total = nx * ny * nz;
    if (index < 0 || index >= total) {
      out[0] = out[1] = out[2] = T(0);
      return;
    }
    out[0] = (T)px[index];
    out[1] = (T)py[index];
    out[2] = (T)pz[index];
  }
};

// utils.h:6-25: lerp along x, then y, then z.
template <typename T>
__device__ __forceinline__ T lerp1(T a, T b, T t) {
  return a * (T(1) - t) + b * t;
}
template <typename T>
__device__ __forceinline__ T lerp3(const T v[8], T x, T y, T z) {
  T s = lerp1(lerp1(v[0], v[1], x), lerp1(v[2], v[3], x), y);
  T t = lerp1(lerp1(v[4], v[5], x), lerp1(v[6], v[7], x), y);
  return lerp1(s, t, z);
}

// SDF::getDistance(gridLocation) (SDF.cpp:503-524): sample at p-0.5, base by
// truncation toward zero.
template <typename T>
__device__ T phi_sample(const PhiView<T> &g, T p0, T p1, T p2) {
  T t0 = p0 - T(0.5), t1 = p1 - T(0.5), t2 = p2 - T(0.5);
  int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
  T v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) v[c] = g.at(b0 + (c & 1), b1 + ((c >> 1) & 1), b2 + (c >> 2));
  return lerp3(v, t0 - (T)b0, t1 - (T)b1, t2 - (T)b2);
}

// DisplacementField::getDisplacementAtf (DisplacementField.cpp:40-58).
template <typename T, typename P>
__device__ void psi_sample(const PsiView<T, P> &f, T p0, T p1, T p2, T out[3]) {
  int b0 = (int)p0, b1 = (int)p1, b2 = (int)p2;
  T v[8][3];
#pragma unroll
  for (int c = 0; c < 8; ++c) f.at(b0 + (c & 1), b1 + ((c >> 1) & 1), b2 + (c >> 2), v[c]);
  T f0 = p0 - (T)b0, f1 = p1 - (T)b1, f2 = p2 - (T)b2;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T s[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) s[c] = v[c][k];
    out[k] = lerp3(s, f0, f1, f2);
  }
}

// SDF::getDistance(spatialIndex, psi) (SDF.cpp:570-575).
template <typename T, typename P>
__device__ T warped_distance(const PhiView<T> &live, const PsiView<T, P> &f, int x, int y, int z) {
  T d[3];
  f.at(x, y, z, d);
  return phi_sample(live, ((T)x + d[0]) + T(0.5), ((T)y + d[1]) + T(0.5), ((T)z + d[2]) + T(0.5));
}

// SDF::getDistancef(gridLocation, psi) (SDF.cpp:577-582).
template <typename T, typename P>
__device__ T warped_distance_f(const PhiView<T> &live, const PsiView<T, P> &f, T p0, T p1, T p2) {
  T d[3];
  psi_sample(f, p0, p1, p2, d);
  return phi_sample(live, (p0 + d[0]) + T(0.5), (p1 + d[1]) + T(0.5), (p2 + d[2]) + T(0.5));
}

// The 19 offsets (units of h) of the second-difference stencils in the
// reference's order (SDF.cpp:847-865, DisplacementField.cpp:305-323).
__device__ __constant__ static const signed char kHessOff[19][3] = {
    {0, 0, 0},  {2, 0, 0},  {-2, 0, 0},  {0, 2, 0},   {0, -2, 0}, {0, 0, 2},   {0, 0, -2},
    {1, 0, 1},  {-1, 0, 1}, {0, 1, 1},   {0, -1, 1},  {1, 1, 0},  {-1, 1, 0},  {-1, 0, -1},
    {1, 0, -1}, {0, -1, -1}, {0, 1, -1}, {-1, -1, 0}, {1, -1, 0}};
enum { H0 = 0, HXP2, HXM2, HYP2, HYM2, HZP2, HZM2, HXPZP, HXMZP, HYPZP, HYMZP,
       HXPYP, HXMYP, HXMZM, HXPZM, HYMZM, HYPZM, HXMYM, HXPYM };

// Second differences from the 19 samples (SDF.cpp:867-881), row-major H.
template <typename T>
__device__ __forceinline__ void hess_assemble(const T f[19], T H[9]) {
  T fxx = (f[HXP2] - T(2) * f[H0] + f[HXM2]);
  T fyy = (f[HYP2] - T(2) * f[H0] + f[HYM2]);
  T fzz = (f[HZP2] - T(2) * f[H0] + f[HZM2]);
  T fxz = (f[HXPZP] + f[HXMZM] - f[HXPZM] - f[HXMZP]);
  T fyz = (f[HYPZP] + f[HYMZM] - f[HYPZM] - f[HYMZP]);
  T fxy = (f[HXPYP] + f[HXMYM] - f[HXPYM] - f[HXMYP]);
  H[0] = fxx; H[4] = fyy; H[8] = fzz;
  H[1] = H[3] = fxy;
  H[2] = H[6] = fxz;
  H[5] = H[7] = fyz;
}

// SDF::computeDistanceGradient(spatialIndex, psi) (SDF.cpp:726-744).
template <typename T, typename P>
__device__ void distance_gradient(const PhiView<T> &live, const PsiView<T, P> &f, T h, int x,
                                  int y, int z, T out[3]) {
  T g[3] = {(T)x + T(0.5), (T)y + T(0.5), (T)z + T(0.5)};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T a[3], b[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T d = h * (T)(j == k);
      a[j] = g[j] + d;
      b[j] = g[j] - d;
    }
    out[k] = warped_distance_f(live, f, a[0], a[1], a[2]) - warped_distance_f(live, f, b[0], b[1], b[2]);
  }
  T den = (T(2) * h);
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = out[k] / den;
}

// SDF::computeDistanceHessian(spatialIndex, psi) (SDF.cpp:842-886).
template <typename T, typename P>
__device__ void distance_hessian(const PhiView<T> &live, const PsiView<T, P> &f, T h, int x,
                                 int y, int z, T out[9]) {
  T g[3] = {(T)x + T(0.5), (T)y + T(0.5), (T)z + T(0.5)};
  T s[19];
  for (int i = 0; i < 19; ++i)
    s[i] = warped_distance_f(live, f, g[0] + h * (T)kHessOff[i][0], g[1] + h * (T)kHessOff[i][1],
                             g[2] + h * (T)kHessOff[i][2]);
  hess_assemble(s, out);
  T den = (T(4) * h * h);
#pragma unroll
  for (int j = 0; j < 9; ++j) out[j] = out[j] / den;
}

template <typename T>
__device__ __forceinline__ T norm3(const T v[3]) {
  return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

// DisplacementField::computeKillingEnergyGradient2 (DisplacementField.cpp:301-347).
template <typename T, typename P>
__device__ void killing_gradient(const PsiView<T, P> &f, T h, T gamma, T clamp, int x, int y,
                                 int z, T out[3]) {
  T g[3] = {(T)x, (T)y, (T)z};
  T d[19][3];
  for (int i = 0; i < 19; ++i)
    psi_sample(f, g[0] + h * (T)kHessOff[i][0], g[1] + h * (T)kHessOff[i][1],
               g[2] + h * (T)kHessOff[i][2], d[i]);
  T xx[3], yy[3], zz[3], xy[3], xz[3], yz[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    xx[c] = (d[HXP2][c] - T(2) * d[H0][c] + d[HXM2][c]);
    yy[c] = (d[HYP2][c] - T(2) * d[H0][c] + d[HYM2][c]);
    zz[c] = (d[HZP2][c] - T(2) * d[H0][c] + d[HZM2][c]);
    xz[c] = (d[HXPZP][c] + d[HXMZM][c] - d[HXPZM][c] - d[HXMZP][c]);
    yz[c] = (d[HYPZP][c] + d[HYMZM][c] - d[HYPZM][c] - d[HYMZP][c]);
    xy[c] = (d[HXPYP][c] + d[HXMYM][c] - d[HXPYM][c] - d[HXMYP][c]);
  }
  T div[3] = {xx[0] + xy[1] + xz[2], xy[0] + yy[1] + yz[2], xz[0] + yz[1] + zz[2]};
  T gk = T(-2) * gamma;
  T kg[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) kg[c] = T(-2) * (xx[c] + yy[c] + zz[c]) + gk * div[c];
  T den = (T(4) * h * h);
  T nrm = norm3(kg);
  if (nrm > clamp) {
    T s = sqrt(kg[0] * kg[0] + kg[1] * kg[1] + kg[2] * kg[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) kg[c] = (kg[c] / s) * clamp;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = kg[c] / den;
}

// Parameters of the gradient in type T.
template <typename T>
struct TParams {
  T voxel_size, epsilon, delta_size, alpha, omega_k, gamma_k, omega_s, killing_clamp;
  int use_data, use_levelset, use_killing;
  __host__ __device__ explicit TParams(const DevParams &p)
      : voxel_size((T)p.voxel_size), epsilon((T)p.epsilon), delta_size((T)p.delta_size),
        alpha((T)p.alpha), omega_k((T)p.omega_k), gamma_k((T)p.gamma_k), omega_s((T)p.omega_s),
        killing_clamp((T)p.killing_clamp), use_data(p.use_data), use_levelset(p.use_levelset),
        use_killing(p.use_killing) {}
};

// KillingFusion::computeEnergyGradient with its three terms
// (KillingFusion.cpp:399-476).  The distance gradient, which the reference
// evaluates twice (data and level-set terms), is computed once: both
// evaluations are the same deterministic function of the same inputs.
template <typename T, typename P>
__device__ void energy_gradient(const PhiView<T> &live, const PhiView<T> &can,
                                const PsiView<T, P> &f, const TParams<T> &tp, int x, int y, int z,
                                T out[3]) {
  T dg[3] = {T(0), T(0), T(0)}, lg[3] = {T(0), T(0), T(0)}, kg[3] = {T(0), T(0), T(0)};
  T g[3];
  if (tp.use_data || tp.use_levelset) distance_gradient(live, f, tp.delta_size, x, y, z, g);
  if (tp.use_data) {
    T s = warped_distance(live, f, x, y, z);
    T dd = can.at(x, y, z);
    T c = (s - dd) / tp.voxel_size;
#pragma unroll
    for (int k = 0; k < 3; ++k) dg[k] = c * g[k];
  }
  if (tp.use_levelset) {
    T H[9];
    distance_hessian(live, f, tp.delta_size, x, y, z, H);
    T hg[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) hg[r] = H[3 * r + 0] * g[0] + H[3 * r + 1] * g[1] + H[3 * r + 2] * g[2];
    T nm1 = norm3(g) - T(1);
    T np = norm3(g) + tp.epsilon;
#pragma unroll
    for (int r = 0; r < 3; ++r) lg[r] = ((hg[r] * nm1) / np) * tp.omega_s;
  }
  if (tp.use_killing) {
    T k3[3];
    killing_gradient(f, tp.delta_size, tp.gamma_k, tp.killing_clamp, x, y, z, k3);
#pragma unroll
    for (int r = 0; r < 3; ++r) kg[r] = k3[r] * tp.omega_k;
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) out[r] = (dg[r] + kg[r]) + lg[r];
}

// The trust-region step of the Jacobi sweep (KillingFusion.cpp:288-314),
// taken with the data term alone.  On entry d = -alpha * g.  While the step
// does not bring phi_live at ((i + psi(i)) + d) + 0.5 closer to dest =
// phi_can(i) than prev = phi_live at the voxel's own warped position, the
// step size a is divided by 1.5 and d = -a * g.  Returns false when a fell
// below 1e-7: the reference then breaks out of the voxel's x loop, so this
// voxel and the rest of its row keep their psi for the iteration.
template <typename T>
__device__ bool trust_step(const PhiView<T> &live, T dest, T prev, int x, int y, int z, const T c[3],
                           const T g[3], T alpha, T d[3]) {
  T a = alpha;
  bool decreased = false;
  do {
    const T s = phi_sample(live, (((T)x + c[0]) + d[0]) + T(0.5), (((T)y + c[1]) + d[1]) + T(0.5),
                           (((T)z + c[2]) + d[2]) + T(0.5));
    const T worse = fabs(s - dest) - fabs(prev - dest);
    if (worse > T(0)) {
      a /= T(1.5);
#pragma unroll
      for (int k = 0; k < 3; ++k) d[k] = -a * g[k];
    } else {
      decreased = true;
    }
  } while (!decreased && a > T(1e-7));
  return !(a < T(1e-7));
}

// Band test of the Jacobi sweep (KillingFusion.cpp:272-274) in T.  The float
// thresholds are the float neighbours of the double ones that make the float
// comparison equivalent to comparing the value as a double.
template <typename T>
__device__ __forceinline__ bool in_band(T s, T hi, T lo) {
  return !(s > hi || s < lo);
}
template <typename T>
__device__ __forceinline__ T band_hi(const DevParams &dp) {
  if constexpr (sizeof(T) == 4) return dp.band_hi_f; else return dp.band_hi;
}
template <typename T>
__device__ __forceinline__ T band_lo(const DevParams &dp) {
  if constexpr (sizeof(T) == 4) return dp.band_lo_f; else return -dp.unknown_clip;
}

// Monitored energy of an active voxel, reported per iteration by the float
// solvers (the reference prints no energy): data + omega_s * level-set +
// omega_k * Killing, with
//   data      0.5 * ((s - phi_can) / v)^2,
//   level set 0.5 * (|grad| / v - 1)^2      (grad in metres per voxel),
//   Killing   |J|_F^2 + gamma <J, J^T>,  J[a][k] = (psi_a(i+e_k) - psi_a(i-e_k)) / 2
// (neighbours clamped to the grid).
template <typename P>
__device__ float monitor_energy(const P *px, const P *py, const P *pz, int nx, int ny, int nz,
                                int x, int y, int z, float s, float can, const float g[3],
                                const DevParams &dp) {
  float v = (float)dp.voxel_size;
  float e = 0.f;
  if (dp.use_data) {
    float r = (s - can) / v;
    e += 0.5f * r * r;
  }
  if (dp.use_levelset) {
    float r = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) / v - 1.0f;
    e += (float)dp.omega_s * 0.5f * r * r;
  }
  if (dp.use_killing) {
    float J[3][3];
    int c[3] = {x, y, z};
    int n[3] = {nx, ny, nz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
      p[k] = min(c[k] + 1, n[k] - 1);
      m[k] = max(c[k] - 1, 0);
      int64_t ip = ((int64_t)p[2] * ny + p[1]) * nx + p[0];
      int64_t im = ((int64_t)m[2] * ny + m[1]) * nx + m[0];
      J[0][k] = 0.5f * ((float)px[ip] - (float)px[im]);
      J[1][k] = 0.5f * ((float)py[ip] - (float)py[im]);
      J[2][k] = 0.5f * ((float)pz[ip] - (float)pz[im]);
    }
    float f = 0.f, t = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        f += J[a][k] * J[a][k];
        t += J[a][k] * J[k][a];
      }
    e += (float)dp.omega_k * (f + (float)dp.gamma_k * t);
  }
  return e;
}

// A block's totals of one iteration's statistics.
struct BlockStats {
  double energy;
  unsigned active;
  float max_delta;
  bool diverged;
};

// Adds a block's totals into st (one atomic per quantity).
__device__ __forceinline__ void commit_iter_stats(IterStats *st, const BlockStats &b) {
  if (b.active || b.max_delta > 0.f || b.energy != 0.0) {
    if (b.active) atomicAdd(&st->active, b.active);
    atomicMax(&st->max_delta, __float_as_uint(b.max_delta));
    atomicAdd(&st->energy, b.energy);
  }
  if (b.diverged) st->diverged = 1;
}

// Block-wide reduction of the per-iteration statistics into st (one atomic
// per block and quantity).  Every thread of the block must call it.  With
// `out`, thread 0 receives the block's totals there instead, and commits
// them itself.
template <int kThreads>
__device__ void reduce_iter_stats(IterStats *st, unsigned active, float max_delta, double energy,
                                  bool diverged, BlockStats *out = nullptr) {
  __shared__ double s_e[kThreads / 32];
  __shared__ float s_m[kThreads / 32];
  __shared__ unsigned s_a[kThreads / 32];
  __shared__ int s_d;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  if (tid == 0) s_d = 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    energy += __shfl_xor_sync(0xffffffffu, energy, o);
    max_delta = fmaxf(max_delta, __shfl_xor_sync(0xffffffffu, max_delta, o));
    active += __shfl_xor_sync(0xffffffffu, active, o);
  }
  int lane = tid & 31, wid = tid >> 5;
  __syncthreads();
  if (diverged) s_d = 1;
  if (lane == 0) {
    s_e[wid] = energy;
    s_m[wid] = max_delta;
    s_a[wid] = active;
  }
  __syncthreads();
  if (wid == 0) {
    energy = lane < kThreads / 32 ? s_e[lane] : 0.0;
    max_delta = lane < kThreads / 32 ? s_m[lane] : 0.f;
    active = lane < kThreads / 32 ? s_a[lane] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      energy += __shfl_xor_sync(0xffffffffu, energy, o);
      max_delta = fmaxf(max_delta, __shfl_xor_sync(0xffffffffu, max_delta, o));
      active += __shfl_xor_sync(0xffffffffu, active, o);
    }
    if (lane == 0) {
      const BlockStats b{energy, active, max_delta, s_d != 0};
      if (out)
        *out = b;
      else
        commit_iter_stats(st, b);
    }
  }
}

// Convergence gate at the start of an iteration: skip when the previous
// iteration was skipped, diverged, or (early_exit) moved psi by at most
// `threshold`.
__device__ __forceinline__ bool iteration_gated(const IterStats *st, int iter, const DevParams &dp) {
  if (iter == 0) return false;
  const IterStats &p = st[iter - 1];
  if (p.skipped || p.diverged) return true;
  return dp.early_exit && __uint_as_float(p.max_delta) <= (float)dp.threshold;
}

}  // namespace kfref
