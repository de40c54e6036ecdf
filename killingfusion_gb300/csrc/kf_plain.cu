// Plain per-term psi update: one kernel per quantity of the reference's
// per-voxel gradient (KillingFusion.cpp:260-350, 399-476), with every
// intermediate field written to and read back from HBM.  This is the direct
// GPU form of the reference's structure -- the baseline the fused solver
// (kf_fused.cu) is measured against.  Float32 arithmetic through the
// reference-order device functions of kf_ref_math.cuh.
//
//   P1 mask      s = phi_live(i + psi(i)), band flag           (SDF.cpp:570)
//   P2 gradient  grad phi~ at the cell centre (6 warped samples) (SDF.cpp:726)
//   P3 hessian   Hessian of phi~ (19 warped samples)            (SDF.cpp:842)
//   P4 data      (s - phi_can)/v * grad                         (KillingFusion.cpp:444)
//   P5 levelset  omega_s * H grad (|grad|-1)/(|grad|+eps)       (KillingFusion.cpp:464)
//   P6 killing   omega_k * Killing gradient (19 psi samples)    (DisplacementField.cpp:301)
//   P7 step      psi += -alpha * (data + killing + levelset)    (KillingFusion.cpp:286,346)
#include <cuda_runtime.h>
#include <stdint.h>

#include "kf_internal.h"
#include "kf_ref_math.cuh"

using namespace kfref;

namespace {

constexpr int kBlock = 256;

struct PlainFields {
  float *s;        // warped value
  uint8_t *act;    // band flag
  float *g[3];     // distance gradient
  float *H[6];     // Hessian xx yy zz xy xz yz
  float *gd[3];    // data term
  float *gl[3];    // level-set term
  float *gk[3];    // Killing term
};

struct PlainArgs {
  PhiView<float> live, can;
  PsiView<float, float> psi;
  float *ox, *oy, *oz;
  DevParams dp;
  PlainFields F;
  IterStats *st;
  int iter;
};

__device__ __forceinline__ bool voxel_of(const DevParams &dp, int64_t &i, int &x, int &y, int &z) {
  i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dp.count) return false;
  int64_t plane = (int64_t)dp.nx * dp.ny;
  z = (int)(i / plane);
  int64_t r = i - (int64_t)z * plane;
  y = (int)(r / dp.nx);
  x = (int)(r - (int64_t)y * dp.nx);
  return true;
}

#define PLAIN_GATE()                                                  \
  if (iteration_gated(a.st, a.iter, a.dp)) {                          \
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st[a.iter].skipped = 1; \
    return;                                                           \
  }

__global__ void __launch_bounds__(kBlock) k_plain_mask(PlainArgs a) {
  PLAIN_GATE();
  int64_t i;
  int x, y, z;
  if (!voxel_of(a.dp, i, x, y, z)) return;
  float s = warped_distance(a.live, a.psi, x, y, z);
  a.F.s[i] = s;
  a.F.act[i] = in_band(s, a.dp.band_hi_f, a.dp.band_lo_f) ? 1 : 0;
}

__global__ void __launch_bounds__(kBlock) k_plain_gradient(PlainArgs a) {
  PLAIN_GATE();
  int64_t i;
  int x, y, z;
  if (!voxel_of(a.dp, i, x, y, z)) return;
  float g[3] = {0.f, 0.f, 0.f};
  if (a.F.act[i]) distance_gradient(a.live, a.psi, (float)a.dp.delta_size, x, y, z, g);
#pragma unroll
  for (int k = 0; k < 3; ++k) a.F.g[k][i] = g[k];
}

__global__ void __launch_bounds__(kBlock) k_plain_hessian(PlainArgs a) {
  PLAIN_GATE();
  int64_t i;
  int x, y, z;
  if (!voxel_of(a.dp, i, x, y, z)) return;
  float H[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (a.F.act[i] && a.dp.use_levelset)
    distance_hessian(a.live, a.psi, (float)a.dp.delta_size, x, y, z, H);
  a.F.H[0][i] = H[0];
  a.F.H[1][i] = H[4];
  a.F.H[2][i] = H[8];
  a.F.H[3][i] = H[1];
  a.F.H[4][i] = H[2];
  a.F.H[5][i] = H[5];
}

__global__ void __launch_bounds__(kBlock) k_plain_data(PlainArgs a) {
  PLAIN_GATE();
  int64_t i;
  int x, y, z;
  if (!voxel_of(a.dp, i, x, y, z)) return;
  float d[3] = {0.f, 0.f, 0.f};
  if (a.F.act[i] && a.dp.use_data) {
    float c = (a.F.s[i] - a.can.at(x, y, z)) / (float)a.dp.voxel_size;
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = c * a.F.g[k][i];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) a.F.gd[k][i] = d[k];
}

__global__ void __launch_bounds__(kBlock) k_plain_levelset(PlainArgs a) {
  PLAIN_GATE();
  int64_t i;
  int x, y, z;
  if (!voxel_of(a.dp, i, x, y, z)) return;
  float l[3] = {0.f, 0.f, 0.f};
  if (a.F.act[i] && a.dp.use_levelset) {
    float g[3] = {a.F.g[0][i], a.F.g[1][i], a.F.g[2][i]};
    float xx = a.F.H[0][i], yy = a.F.H[1][i], zz = a.F.H[2][i];
    float xy = a.F.H[3][i], xz = a.F.H[4][i], yz = a.F.H[5][i];
    float hg[3] = {xx * g[0] + xy * g[1] + xz * g[2], xy * g[0] + yy * g[1] + yz * g[2],
                   xz * g[0] + yz * g[1] + zz * g[2]};
    float nm1 = norm3(g) - 1.f, np = norm3(g) + (float)a.dp.epsilon;
#pragma unroll
    for (int k = 0; k < 3; ++k) l[k] = ((hg[k] * nm1) / np) * (float)a.dp.omega_s;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) a.F.gl[k][i] = l[k];
}

__global__ void __launch_bounds__(kBlock) k_plain_killing(PlainArgs a) {
  PLAIN_GATE();
  int64_t i;
  int x, y, z;
  if (!voxel_of(a.dp, i, x, y, z)) return;
  float kg[3] = {0.f, 0.f, 0.f};
  if (a.F.act[i] && a.dp.use_killing) {
    killing_gradient(a.psi, (float)a.dp.delta_size, (float)a.dp.gamma_k,
                     (float)a.dp.killing_clamp, x, y, z, kg);
#pragma unroll
    for (int k = 0; k < 3; ++k) kg[k] = kg[k] * (float)a.dp.omega_k;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) a.F.gk[k][i] = kg[k];
}

__global__ void __launch_bounds__(kBlock) k_plain_step(PlainArgs a) {
  PLAIN_GATE();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool act = false, diverged = false;
  float dn = 0.f;
  double e = 0.0;
  if (i < a.dp.count) {
    int64_t plane = (int64_t)a.dp.nx * a.dp.ny;
    int z = (int)(i / plane);
    int64_t r = i - (int64_t)z * plane;
    int y = (int)(r / a.dp.nx);
    int x = (int)(r - (int64_t)y * a.dp.nx);
    float p[3] = {a.psi.px[i], a.psi.py[i], a.psi.pz[i]};
    float d[3] = {0.f, 0.f, 0.f};
    act = a.F.act[i] != 0;
    if (act) {
#pragma unroll
      for (int k = 0; k < 3; ++k)
        d[k] = d[k] + -(float)a.dp.alpha * ((a.F.gd[k][i] + a.F.gk[k][i]) + a.F.gl[k][i]);
      diverged = !isfinite(p[0]) || !isfinite(p[1]) || !isfinite(p[2]);
      dn = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      float g[3] = {a.F.g[0][i], a.F.g[1][i], a.F.g[2][i]};
      e = (double)monitor_energy(a.psi.px, a.psi.py, a.psi.pz, a.dp.nx, a.dp.ny, a.dp.nz, x, y, z,
                                 a.F.s[i], a.can.at(x, y, z), g, a.dp);
    }
    a.ox[i] = p[0] + d[0];
    a.oy[i] = p[1] + d[1];
    a.oz[i] = p[2] + d[2];
  }
  reduce_iter_stats<kBlock>(a.st + a.iter, act ? 1u : 0u, dn, e, diverged);
}

}  // namespace

int kf_solve_plain(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp, int iterations,
                   IterStats *st, cudaStream_t s) {
  int rc = kf_field_ensure_pair(psi);
  if (rc) return rc;
  const int64_t N = dp.count;
  // s (4) + flag (1, padded to 4) + grad (12) + hessian (24) + three terms (36)
  size_t need = (size_t)N * (4 + 4 + 12 + 24 + 36) + 256;
  if (psi->plain_bytes < need) {
    cudaFree(psi->plain_scratch);
    psi->plain_scratch = nullptr;
    psi->plain_bytes = 0;
    if (cudaMalloc(&psi->plain_scratch, need) != cudaSuccess) {
      cudaGetLastError();
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the per-term solver fields failed");
    }
    psi->plain_bytes = need;
  }
  float *f = (float *)psi->plain_scratch;
  PlainArgs a;
  a.F.s = f;
  f += N;
  a.F.act = (uint8_t *)f;
  f += N;  // 4 bytes reserved per flag keeps the float fields aligned
  for (int k = 0; k < 3; ++k, f += N) a.F.g[k] = f;
  for (int k = 0; k < 6; ++k, f += N) a.F.H[k] = f;
  for (int k = 0; k < 3; ++k, f += N) a.F.gd[k] = f;
  for (int k = 0; k < 3; ++k, f += N) a.F.gl[k] = f;
  for (int k = 0; k < 3; ++k, f += N) a.F.gk[k] = f;
  a.live = PhiView<float>{live->phi, dp.nx, dp.ny, dp.nz, dp.oob_phi_f};
  a.can = PhiView<float>{can->phi, dp.nx, dp.ny, dp.nz, dp.oob_phi_f};
  a.dp = dp;
  a.st = st;
  unsigned nb = (unsigned)((N + kBlock - 1) / kBlock);
  void *buf[2][3] = {{psi->p[0], psi->p[1], psi->p[2]}, {psi->q[0], psi->q[1], psi->q[2]}};
  for (int it = 0; it < iterations; ++it) {
    void **in = buf[it & 1], **out = buf[(it + 1) & 1];
    a.psi = PsiView<float, float>{(const float *)in[0], (const float *)in[1], (const float *)in[2],
                                  dp.nx, dp.ny, dp.nz};
    a.ox = (float *)out[0];
    a.oy = (float *)out[1];
    a.oz = (float *)out[2];
    a.iter = it;
    k_plain_mask<<<nb, kBlock, 0, s>>>(a);
    k_plain_gradient<<<nb, kBlock, 0, s>>>(a);
    k_plain_hessian<<<nb, kBlock, 0, s>>>(a);
    k_plain_data<<<nb, kBlock, 0, s>>>(a);
    k_plain_levelset<<<nb, kBlock, 0, s>>>(a);
    k_plain_killing<<<nb, kBlock, 0, s>>>(a);
    k_plain_step<<<nb, kBlock, 0, s>>>(a);
    KF_CHECK_LAUNCH("plain per-term kernels");
  }
  return KF_OK;
}
