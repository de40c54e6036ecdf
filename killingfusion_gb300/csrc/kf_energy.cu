// Project energy of a displacement field and its exact adjoint.
//
// The reference never evaluates an energy: its solver descends the
// Euler-Lagrange gradients of KillingFusion::computeEnergyGradient
// (KillingFusion.cpp:399-476) directly.  This file evaluates a discrete
// energy with the same three terms, written so that its gradient with respect
// to psi can be taken exactly and checked against finite differences:
//
//   E = sum over active voxels i of
//         1/2 ((phi_w(i) - phi_can(i)) / v)^2                           data
//       + w_s 1/2 (|g(i)|_e / v - 1)^2                                  level set
//       + w_k (|J(i)|^2 + gamma <J(i), J(i)^T>)                         Killing
//
//   phi_w(j) = live sampled at j + psi(j) (grid units; trilinear with the
//              reference's truncating base, SDF.cpp:503-524),
//   g(i)_k   = (phi_w(i + e_k) - phi_w(i - e_k)) / 2, neighbours clamped,
//   |g|_e    = sqrt(g.g + (v eps)^2),
//   J(i)_ak  = (psi_a(i + e_k) - psi_a(i - e_k)) / 2, neighbours clamped.
//
// Kernels:
//   k_energy       one thread per voxel of a box, FP32 or FP64 arithmetic,
//                  per-block FP64 partial sums summed in a fixed order
//                  (deterministic);
//   k_ls_coef +    the adjoint as a gather: each voxel j collects the
//   k_adjoint      partial derivatives of every active voxel whose energy
//                  reads psi(j) (itself and its six clamped neighbours), so
//                  no atomics and a deterministic result;
//   k_energy_fd    central differences of the energy of the 3x3x3 window
//                  around sampled voxels with one psi component moved by
//                  +-h (the only voxels whose energy depends on it).
// Compiled without contracted multiply-add so the float64 form rounds as the
// oracle's C restatement does.
#include <cuda_runtime.h>

#include <algorithm>

#include "kf_internal.h"
#include "kf_ref_math.cuh"

namespace {

constexpr int kThreads = 256;

template <typename T>
struct EnergyTerms {
  T data, ls, killing;
};

template <typename T, typename P>
struct EArgs {
  const float *live;
  const float *can;
  const P *px, *py, *pz;
  const uint8_t *active;  // NULL: every voxel
  int nx, ny, nz;
  T v, ve, oob, omega_s, omega_k, gamma_k;
  int use_data, use_ls, use_k;
  // a virtual change of one psi entry (k_energy_fd): psi_comp(pj) += pdelta
  int64_t pj;
  int pcomp;
  T pdelta;
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <typename T, typename P>
__device__ __forceinline__ int64_t lin(const EArgs<T, P> &a, int x, int y, int z) {
  return ((int64_t)z * a.ny + y) * a.nx + x;
}

template <typename T, typename P>
__device__ __forceinline__ T psi_c(const EArgs<T, P> &a, int64_t j, int c) {
  const P *p = c == 0 ? a.px : (c == 1 ? a.py : a.pz);
  T v = (T)p[j];
  if (j == a.pj && c == a.pcomp) v = v + a.pdelta;
  return v;
}

template <typename T, typename P>
__device__ __forceinline__ T live_at(const EArgs<T, P> &a, int x, int y, int z) {
  if (x < 0 || x >= a.nx || y < 0 || y >= a.ny || z < 0 || z >= a.nz) return a.oob;
  return (T)__ldg(a.live + lin(a, x, y, z));
}

// Trilinear sample of live at t (grid units) and its derivative with
// respect to t inside the cell chosen by truncation.
template <typename T, typename P>
__device__ T sample_grad(const EArgs<T, P> &a, const T t[3], T dv[3]) {
  const int b0 = (int)t[0], b1 = (int)t[1], b2 = (int)t[2];
  T v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) v[c] = live_at(a, b0 + (c & 1), b1 + ((c >> 1) & 1), b2 + (c >> 2));
  const T fx = t[0] - (T)b0, fy = t[1] - (T)b1, fz = t[2] - (T)b2;
  const T one = T(1);
  dv[0] = (one - fz) * ((one - fy) * (v[1] - v[0]) + fy * (v[3] - v[2])) +
          fz * ((one - fy) * (v[5] - v[4]) + fy * (v[7] - v[6]));
  dv[1] = (one - fz) * ((one - fx) * (v[2] - v[0]) + fx * (v[3] - v[1])) +
          fz * ((one - fx) * (v[6] - v[4]) + fx * (v[7] - v[5]));
  using kfref::lerp1;
  const T top = lerp1(lerp1(v[4], v[5], fx), lerp1(v[6], v[7], fx), fy);
  const T bot = lerp1(lerp1(v[0], v[1], fx), lerp1(v[2], v[3], fx), fy);
  dv[2] = top - bot;
  return lerp1(bot, top, fz);
}

template <typename T, typename P>
__device__ T warped(const EArgs<T, P> &a, int x, int y, int z, T dv[3]) {
  const int64_t j = lin(a, x, y, z);
  const T t[3] = {(T)x + psi_c(a, j, 0), (T)y + psi_c(a, j, 1), (T)z + psi_c(a, j, 2)};
  return sample_grad(a, t, dv);
}

template <typename T, typename P>
__device__ bool is_active(const EArgs<T, P> &a, int64_t i) {
  return a.active == nullptr || a.active[i] != 0;
}

// J(i)_ak = (psi_a(p_k) - psi_a(m_k)) / 2 with clamped neighbours.
template <typename T, typename P>
__device__ void jacobian(const EArgs<T, P> &a, int x, int y, int z, T J[3][3]) {
  const int c[3] = {x, y, z}, n[3] = {a.nx, a.ny, a.nz};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
    p[k] = clampi(c[k] + 1, 0, n[k] - 1);
    m[k] = clampi(c[k] - 1, 0, n[k] - 1);
    const int64_t ip = lin(a, p[0], p[1], p[2]), im = lin(a, m[0], m[1], m[2]);
#pragma unroll
    for (int q = 0; q < 3; ++q) J[q][k] = T(0.5) * (psi_c(a, ip, q) - psi_c(a, im, q));
  }
}

// Level-set gradient g(i) (clamped central differences of phi_w).
template <typename T, typename P>
__device__ void ls_gradient(const EArgs<T, P> &a, int x, int y, int z, T g[3]) {
  const int c[3] = {x, y, z}, n[3] = {a.nx, a.ny, a.nz};
  T dv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
    p[k] = clampi(c[k] + 1, 0, n[k] - 1);
    m[k] = clampi(c[k] - 1, 0, n[k] - 1);
    g[k] = T(0.5) * (warped(a, p[0], p[1], p[2], dv) - warped(a, m[0], m[1], m[2], dv));
  }
}

// Energy of voxel (x,y,z), assumed active.
template <typename T, typename P>
__device__ EnergyTerms<T> voxel_energy(const EArgs<T, P> &a, int x, int y, int z) {
  EnergyTerms<T> e{T(0), T(0), T(0)};
  const int64_t i = lin(a, x, y, z);
  if (a.use_data) {
    T dv[3];
    const T r = (warped(a, x, y, z, dv) - (T)__ldg(a.can + i)) / a.v;
    e.data = T(0.5) * r * r;
  }
  if (a.use_ls) {
    T g[3];
    ls_gradient(a, x, y, z, g);
    const T nr = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + a.ve * a.ve);
    const T r = nr / a.v - T(1);
    e.ls = a.omega_s * T(0.5) * r * r;
  }
  if (a.use_k) {
    T J[3][3];
    jacobian(a, x, y, z, J);
    T f = T(0), s = T(0);
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        f += J[q][k] * J[q][k];
        s += J[q][k] * J[k][q];
      }
    e.killing = a.omega_k * (f + a.gamma_k * s);
  }
  return e;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sums three doubles over the block; thread 0 gets the totals.
__device__ void block_sum3(double v[3]) {
  __shared__ double red[3][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) red[k][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) {
      double s = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) s += red[k][w];
      v[k] = s;
    }
  }
}

template <typename T, typename P>
__global__ void __launch_bounds__(kThreads) k_energy(EArgs<T, P> a, int x0, int y0, int z0, int bx, int by,
                                                     int64_t count, double *partial) {
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t u = (int64_t)blockIdx.x * kThreads + threadIdx.x; u < count; u += (int64_t)gridDim.x * kThreads) {
    const int x = x0 + (int)(u % bx);
    const int y = y0 + (int)((u / bx) % by);
    const int z = z0 + (int)(u / ((int64_t)bx * by));
    if (!is_active(a, lin(a, x, y, z))) continue;
    EnergyTerms<T> e = voxel_energy(a, x, y, z);
    acc[0] += (double)e.data;
    acc[1] += (double)e.ls;
    acc[2] += (double)e.killing;
  }
  block_sum3(acc);
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) partial[3 * blockIdx.x + k] = acc[k];
}

__global__ void k_sum_partials(const double *partial, int blocks, double *out) {
  // one warp; lane l sums blocks l, l+32, ... then a fixed shuffle tree
  double s[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < blocks; b += 32)
    for (int k = 0; k < 3; ++k) s[k] += partial[3 * b + k];
  for (int k = 0; k < 3; ++k) {
    double t = warp_sum(s[k]);
    if (threadIdx.x == 0) out[k] = t;
  }
}

// Level-set coefficient of voxel i: d E_ls(i) / d g_k(i) / 2, i.e. the
// weight of d phi_w(p_k(i)) (+) and d phi_w(m_k(i)) (-).
template <typename P>
__global__ void __launch_bounds__(kThreads) k_ls_coef(EArgs<double, P> a, double *S) {
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < N; i += (int64_t)gridDim.x * kThreads) {
    double s[3] = {0.0, 0.0, 0.0};
    if (is_active(a, i)) {
      const int x = (int)(i % a.nx), y = (int)((i / a.nx) % a.ny), z = (int)(i / ((int64_t)a.nx * a.ny));
      double g[3];
      ls_gradient(a, x, y, z, g);
      const double nr = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + a.ve * a.ve);
      const double coef = a.omega_s * (nr / a.v - 1.0) / (a.v * nr);
      for (int k = 0; k < 3; ++k) s[k] = coef * g[k] * 0.5;
    }
    S[i] = s[0];
    S[N + i] = s[1];
    S[2 * N + i] = s[2];
  }
}

// d E / d psi(j) by gathering from the voxels whose energy reads psi(j).
template <typename P>
__global__ void __launch_bounds__(kThreads) k_adjoint(EArgs<double, P> a, const double *S, double *grad) {
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  const int n[3] = {a.nx, a.ny, a.nz};
  for (int64_t j = (int64_t)blockIdx.x * kThreads + threadIdx.x; j < N; j += (int64_t)gridDim.x * kThreads) {
    const int c[3] = {(int)(j % a.nx), (int)((j / a.nx) % a.ny), (int)(j / ((int64_t)a.nx * a.ny))};
    double dv[3];
    const double w = warped(a, c[0], c[1], c[2], dv);
    double out[3] = {0.0, 0.0, 0.0};
    if (a.use_data && is_active(a, j)) {
      const double r = (w - (double)__ldg(a.can + j)) / a.v;
      for (int q = 0; q < 3; ++q) out[q] += r / a.v * dv[q];
    }
    double ls = 0.0;
    for (int k = 0; k < 3; ++k) {
      // voxels i with p_k(i) == j (+) and m_k(i) == j (-)
      int cand[2][3];
      int sign[2], nc = 0;
      if (c[k] >= 1) {
        cand[nc][0] = c[0]; cand[nc][1] = c[1]; cand[nc][2] = c[2];
        cand[nc][k] -= 1;
        sign[nc++] = 1;
      }
      if (c[k] <= n[k] - 2) {
        cand[nc][0] = c[0]; cand[nc][1] = c[1]; cand[nc][2] = c[2];
        cand[nc][k] += 1;
        sign[nc++] = -1;
      }
      // clamped neighbours: i = j reads itself as p_k (top face) and/or m_k
      // (bottom face)
      int self = (c[k] == n[k] - 1 ? 1 : 0) - (c[k] == 0 ? 1 : 0);
      for (int u = 0; u < nc + 1; ++u) {
        int ix, iy, iz, sg;
        if (u < nc) {
          ix = cand[u][0]; iy = cand[u][1]; iz = cand[u][2]; sg = sign[u];
        } else {
          if (self == 0) break;
          ix = c[0]; iy = c[1]; iz = c[2]; sg = self;
        }
        const int64_t i = lin(a, ix, iy, iz);
        if (!is_active(a, i)) continue;
        if (a.use_ls) ls += sg * S[(int64_t)k * N + i];
        if (a.use_k) {
          double J[3][3];
          jacobian(a, ix, iy, iz, J);
          for (int q = 0; q < 3; ++q) {
            const double dJ = a.omega_k * (2 * J[q][k] + 2 * a.gamma_k * J[k][q]);
            out[q] += sg * (0.5 * dJ);
          }
        }
      }
    }
    if (a.use_ls)
      for (int q = 0; q < 3; ++q) out[q] += ls * dv[q];
    grad[3 * j] = out[0];
    grad[3 * j + 1] = out[1];
    grad[3 * j + 2] = out[2];
  }
}

// Central difference of the energy of the 3x3x3 window around each sampled
// voxel, one warp per (voxel, component).
template <typename P>
__global__ void k_energy_fd(EArgs<double, P> a, const int32_t *voxels, int count, double h, double *out) {
  const int pair = blockIdx.x;
  if (pair >= 3 * count) return;
  const int s = pair / 3, comp = pair % 3;
  const int jx = voxels[3 * s], jy = voxels[3 * s + 1], jz = voxels[3 * s + 2];
  if (jx < 0 || jx >= a.nx || jy < 0 || jy >= a.ny || jz < 0 || jz >= a.nz) {
    if (threadIdx.x == 0) out[3 * s + comp] = 0.0;
    return;
  }
  const int l = threadIdx.x;
  double d = 0.0;
  if (l < 27) {
    const int x = jx + l % 3 - 1, y = jy + (l / 3) % 3 - 1, z = jz + l / 9 - 1;
    if (x >= 0 && x < a.nx && y >= 0 && y < a.ny && z >= 0 && z < a.nz && is_active(a, lin(a, x, y, z))) {
      EArgs<double, P> b = a;
      b.pj = lin(a, jx, jy, jz);
      b.pcomp = comp;
      b.pdelta = h;
      EnergyTerms<double> ep = voxel_energy(b, x, y, z);
      b.pdelta = -h;
      EnergyTerms<double> em = voxel_energy(b, x, y, z);
      d = ((ep.data + ep.ls) + ep.killing) - ((em.data + em.ls) + em.killing);
    }
  }
  d = warp_sum(d);
  if (l == 0) out[3 * s + comp] = d / (2.0 * h);
}

template <typename T, typename P>
EArgs<T, P> make_args(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, const uint8_t *active) {
  EArgs<T, P> a;
  a.live = live->phi;
  a.can = can->phi;
  a.px = (const P *)psi->p[0];
  a.py = (const P *)psi->p[1];
  a.pz = (const P *)psi->p[2];
  a.active = active;
  a.nx = live->n[0];
  a.ny = live->n[1];
  a.nz = live->n[2];
  a.v = (T)dp.voxel_size;
  a.ve = (T)(dp.voxel_size * dp.epsilon);
  a.oob = (T)dp.oob_phi;
  a.omega_s = (T)dp.omega_s;
  a.omega_k = (T)dp.omega_k;
  a.gamma_k = (T)dp.gamma_k;
  a.use_data = dp.use_data;
  a.use_ls = dp.use_levelset;
  a.use_k = dp.use_killing;
  a.pj = -1;
  a.pcomp = -1;
  a.pdelta = T(0);
  return a;
}

int check_common(kf_grid live, kf_grid can, kf_field psi, const kf_params *p) {
  KF_REQUIRE(live && can && psi && p, "NULL argument");
  for (int k = 0; k < 3; ++k)
    KF_REQUIRE(live->n[k] == can->n[k] && live->n[k] == psi->n[k], "grid and field sizes differ");
  return kf_check_params(p);
}

template <typename T, typename P>
int run_energy(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, const uint8_t *active,
               const int box[6], double terms[3], cudaStream_t s) {
  const int x0 = box[0], y0 = box[1], z0 = box[2];
  const int bx = box[3] - box[0], by = box[4] - box[1], bz = box[5] - box[2];
  const int64_t count = (int64_t)bx * by * bz;
  double *buf = nullptr;
  int blocks = (int)std::min<int64_t>((count + kThreads - 1) / kThreads, (int64_t)kf_num_sms() * 8);
  if (blocks < 1) blocks = 1;
  KF_CHECK_CUDA(cudaMallocAsync((void **)&buf, sizeof(double) * (3 * (size_t)blocks + 3), s));
  EArgs<T, P> a = make_args<T, P>(live, can, psi, dp, active);
  k_energy<T, P><<<blocks, kThreads, 0, s>>>(a, x0, y0, z0, bx, by, count, buf + 3);
  k_sum_partials<<<1, 32, 0, s>>>(buf + 3, blocks, buf);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(terms, buf, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t f = cudaFreeAsync(buf, s);
  if (e == cudaSuccess) e = f;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return kf_cuda_fail(e, "kf_energy");
  return KF_OK;
}

template <typename P>
int run_adjoint(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, const uint8_t *active,
                double *grad, cudaStream_t s) {
  const int64_t N = live->count;
  EArgs<double, P> a = make_args<double, P>(live, can, psi, dp, active);
  double *S = nullptr;
  const int blocks = (int)std::min<int64_t>((N + kThreads - 1) / kThreads, (int64_t)kf_num_sms() * 8);
  KF_CHECK_CUDA(cudaMallocAsync((void **)&S, sizeof(double) * 3 * (size_t)N, s));
  if (dp.use_levelset) k_ls_coef<P><<<blocks, kThreads, 0, s>>>(a, S);
  k_adjoint<P><<<blocks, kThreads, 0, s>>>(a, S, grad);
  cudaError_t e = cudaGetLastError();
  cudaError_t f = cudaFreeAsync(S, s);
  if (e == cudaSuccess) e = f;
  if (e != cudaSuccess) return kf_cuda_fail(e, "kf_energy_adjoint");
  return KF_OK;
}

}  // namespace

extern "C" int kf_energy(kf_grid live, kf_grid can, kf_field psi, const kf_params *p, const uint8_t *active,
                         const int box[6], kf_precision arith, double terms[3], void *stream) {
  int rc = check_common(live, can, psi, p);
  if (rc) return rc;
  KF_REQUIRE(terms, "NULL terms");
  KF_REQUIRE(arith == KF_F32 || arith == KF_F64, "bad arithmetic precision");
  int b[6] = {0, 0, 0, live->n[0], live->n[1], live->n[2]};
  if (box) {
    for (int k = 0; k < 3; ++k) {
      KF_REQUIRE(box[k] >= 0 && box[k] <= box[k + 3] && box[k + 3] <= live->n[k], "box outside the grid");
      b[k] = box[k];
      b[k + 3] = box[k + 3];
    }
  }
  DevParams dp = kf_make_dev_params(live->n, p);
  cudaStream_t s = kf_stream(stream);
  if (b[3] == b[0] || b[4] == b[1] || b[5] == b[2]) {
    terms[0] = terms[1] = terms[2] = 0.0;
    return KF_OK;
  }
  if (psi->prec == KF_F32)
    return arith == KF_F64 ? run_energy<double, float>(live, can, psi, dp, active, b, terms, s)
                           : run_energy<float, float>(live, can, psi, dp, active, b, terms, s);
  return arith == KF_F64 ? run_energy<double, double>(live, can, psi, dp, active, b, terms, s)
                         : run_energy<float, double>(live, can, psi, dp, active, b, terms, s);
}

extern "C" int kf_energy_adjoint(kf_grid live, kf_grid can, kf_field psi, const kf_params *p,
                                 const uint8_t *active, double *grad, void *stream) {
  int rc = check_common(live, can, psi, p);
  if (rc) return rc;
  KF_REQUIRE(grad, "NULL grad");
  DevParams dp = kf_make_dev_params(live->n, p);
  cudaStream_t s = kf_stream(stream);
  return psi->prec == KF_F32 ? run_adjoint<float>(live, can, psi, dp, active, grad, s)
                             : run_adjoint<double>(live, can, psi, dp, active, grad, s);
}

extern "C" int kf_energy_fd(kf_grid live, kf_grid can, kf_field psi, const kf_params *p,
                            const uint8_t *active, const int32_t *voxels, int count, double h, double *out,
                            void *stream) {
  int rc = check_common(live, can, psi, p);
  if (rc) return rc;
  KF_REQUIRE(count >= 0 && (count == 0 || (voxels && out)), "bad voxel list");
  KF_REQUIRE(h > 0.0, "h must be positive");
  if (count == 0) return KF_OK;
  KF_REQUIRE((int64_t)count * 3 <= 0x7fffffff, "too many voxels");
  DevParams dp = kf_make_dev_params(live->n, p);
  cudaStream_t s = kf_stream(stream);
  if (psi->prec == KF_F32) {
    k_energy_fd<float><<<3 * count, 32, 0, s>>>(make_args<double, float>(live, can, psi, dp, active), voxels,
                                                 count, h, out);
  } else {
    k_energy_fd<double><<<3 * count, 32, 0, s>>>(make_args<double, double>(live, can, psi, dp, active), voxels,
                                                  count, h, out);
  }
  KF_CHECK_LAUNCH("kf_energy_fd");
  return KF_OK;
}
