// The per-frame pipeline of KillingFusion::processNextFrame
// (KillingFusion.cpp:109-175) on the device: canonical SDF, live SDF and psi
// stay resident; a frame goes in as a depth image and up to three triangle
// soups come out in pinned host memory.
#include <cuda_runtime.h>
#include <string.h>

#include "kf_internal.h"

struct kf_fusion_s {
  kf_fusion_config cfg;
  kf_grid can = nullptr, live = nullptr, scratch = nullptr;
  kf_field psi = nullptr;
  int frames = 0;
  float *dmesh[3] = {nullptr, nullptr, nullptr};
  int64_t dcap[3] = {0, 0, 0};
  float *hmesh[3] = {nullptr, nullptr, nullptr};
  int64_t hcap[3] = {0, 0, 0};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

static void release(kf_fusion f) {
  kf_grid_destroy(f->can);
  kf_grid_destroy(f->live);
  kf_grid_destroy(f->scratch);
  kf_field_destroy(f->psi);
  for (int k = 0; k < 3; ++k) {
    cudaFree(f->dmesh[k]);
    cudaFreeHost(f->hmesh[k]);
  }
  if (f->e0) cudaEventDestroy(f->e0);
  if (f->e1) cudaEventDestroy(f->e1);
}

extern "C" int kf_fusion_destroy(kf_fusion f) {
  if (!f) return KF_OK;
  release(f);
  delete f;
  return KF_OK;
}

extern "C" int kf_fusion_create(const kf_fusion_config *cfg, kf_fusion *out) {
  KF_REQUIRE(cfg && out, "NULL argument");
  *out = nullptr;
  KF_REQUIRE(cfg->width > 0 && cfg->height > 0, "depth frame size must be positive");
  KF_REQUIRE(cfg->iterations >= 0, "iterations must be >= 0");
  KF_REQUIRE(cfg->solver == KF_SOLVER_FUSED || cfg->solver == KF_SOLVER_PLAIN ||
                 cfg->solver == KF_SOLVER_EXACT || cfg->solver == KF_SOLVER_BAND,
             "unknown solver");
  int rc = kf_check_params(&cfg->params);
  if (rc) return rc;
  kf_fusion f = new kf_fusion_s();
  f->cfg = *cfg;
  rc = kf_grid_create(cfg->dims, cfg->voxel_size, cfg->min3d, cfg->params.unknown_clip, &cfg->params,
                      &f->can);
  if (!rc)
    rc = kf_grid_create(cfg->dims, cfg->voxel_size, cfg->min3d, cfg->params.unknown_clip,
                        &cfg->params, &f->live);
  if (!rc)
    rc = kf_field_create(cfg->dims, cfg->solver == KF_SOLVER_EXACT ? KF_F64 : KF_F32, &f->psi);
  if (!rc && (cudaEventCreate(&f->e0) != cudaSuccess || cudaEventCreate(&f->e1) != cudaSuccess))
    rc = kf_fail(KF_ERR_CUDA, "cudaEventCreate failed");
  if (rc) {
    kf_fusion_destroy(f);
    return rc;
  }
  *out = f;
  return KF_OK;
}

extern "C" int kf_fusion_state(kf_fusion f, kf_grid *canonical, kf_grid *live, kf_field *psi) {
  KF_REQUIRE(f, "pipeline is NULL");
  if (canonical) *canonical = f->can;
  if (live) *live = f->live;
  if (psi) *psi = f->psi;
  return KF_OK;
}

// SDF::getMesh into the pipeline's buffers; the host copy is queued on s.
static int mesh_to_host(kf_fusion f, kf_grid g, int k, int64_t *ntri, cudaStream_t s) {
  DevParams dp = kf_make_dev_params(g->n, &f->cfg.params);
  int64_t n = 0;
  int rc = kf_mc_run(g, dp, f->dmesh[k], f->dcap[k], &n, s);
  if (rc == KF_ERR_CAPACITY || (rc == KF_OK && f->dmesh[k] == nullptr && n > 0)) {
    cudaFree(f->dmesh[k]);
    f->dcap[k] = n + n / 4 + 1024;
    if (cudaMalloc(&f->dmesh[k], f->dcap[k] * 9 * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      f->dmesh[k] = nullptr;
      f->dcap[k] = 0;
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the mesh buffer failed");
    }
    rc = kf_mc_run(g, dp, f->dmesh[k], f->dcap[k], &n, s);
  }
  if (rc) return rc;
  if (f->hcap[k] < n) {
    cudaFreeHost(f->hmesh[k]);
    f->hcap[k] = n + n / 4 + 1024;
    if (cudaMallocHost(&f->hmesh[k], f->hcap[k] * 9 * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      f->hmesh[k] = nullptr;
      f->hcap[k] = 0;
      return kf_fail(KF_ERR_OOM, "pinned allocation of the mesh buffer failed");
    }
  }
  if (n > 0)
    KF_CHECK_CUDA(cudaMemcpyAsync(f->hmesh[k], f->dmesh[k], n * 9 * sizeof(float),
                                  cudaMemcpyDeviceToHost, s));
  *ntri = n;
  return KF_OK;
}

extern "C" int kf_fusion_process_frame(kf_fusion f, const float *depth, const double c2w[16],
                                       int meshes, kf_frame_result *res, void *stream) {
  KF_REQUIRE(f && depth, "NULL argument");
  cudaStream_t s = kf_stream(stream);
  const kf_fusion_config &c = f->cfg;
  const kf_params *p = &c.params;
  static const double kEye[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  const double *pose = c2w ? c2w : kEye;
  kf_frame_result r;
  memset(&r, 0, sizeof(r));
  KF_CHECK_CUDA(cudaEventRecord(f->e0, s));
  int rc = KF_OK;
  if (f->frames == 0) {
    // the first frame becomes the canonical SDF (KillingFusion.cpp:115-121)
    rc = kf_compute_sdf(f->can, p, depth, c.width, c.height, pose, c.K, c.min_depth, c.max_depth, s);
    if (!rc) rc = kf_field_zero(f->psi, s);
    if (!rc && (meshes & KF_MESH_LIVE)) rc = mesh_to_host(f, f->can, 0, &r.ntri[0], s);
    if (!rc && (meshes & KF_MESH_REGISTERED)) {
      // canonical->getMesh(psi): fuse through psi into a fresh SDF (SDF.cpp:416-421)
      if (!f->scratch)
        rc = kf_grid_create(c.dims, c.voxel_size, c.min3d, p->unknown_clip, p, &f->scratch);
      if (!rc) rc = kf_grid_reset(f->scratch, p, s);
      if (!rc) rc = kf_fuse_warped(f->scratch, f->can, f->psi, p, s);
      if (!rc) rc = mesh_to_host(f, f->scratch, 1, &r.ntri[1], s);
    }
  } else {
    // computeSDF, zero psi, register, mesh, warp + fuse (KillingFusion.cpp:130-160)
    rc = kf_compute_sdf(f->live, p, depth, c.width, c.height, pose, c.K, c.min_depth, c.max_depth, s);
    if (!rc) rc = kf_field_zero(f->psi, s);
    // the live mesh queues behind the solve without the host waiting in
    // between; the solve's status is read before warp + fuse changes the
    // canonical SDF, so a diverged solve leaves it untouched, as the
    // reference's throw does
    const bool async = !(p->early_exit && c.solver != KF_SOLVER_FUSED && c.solver != KF_SOLVER_PERVOXEL);
    if (!rc)
      rc = async ? kf_psi_solve_async(f->live, f->can, f->psi, p, c.iterations, c.solver, stream)
                 : kf_psi_solve(f->live, f->can, f->psi, p, c.iterations, c.solver, &r.solve, stream);
    if (!rc && (meshes & KF_MESH_LIVE)) rc = mesh_to_host(f, f->live, 0, &r.ntri[0], s);
    if (async && c.iterations > 0) {
      const int wrc = kf_psi_solve_wait(f->psi, &r.solve);
      if (!rc) rc = wrc;
    }
    if (!rc) rc = kf_warp_fuse(f->can, f->live, f->psi, p, s);
    if (!rc && (meshes & KF_MESH_REGISTERED)) rc = mesh_to_host(f, f->live, 1, &r.ntri[1], s);
  }
  if (!rc && (meshes & KF_MESH_CANONICAL)) rc = mesh_to_host(f, f->can, 2, &r.ntri[2], s);
  if (rc) return rc;
  KF_CHECK_CUDA(cudaEventRecord(f->e1, s));
  KF_CHECK_CUDA(cudaEventSynchronize(f->e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, f->e0, f->e1);
  r.device_ms = ms;
  ++f->frames;
  r.frame = f->frames;
  for (int k = 0; k < 3; ++k)
    r.mesh[k] = (meshes & (1 << k)) ? f->hmesh[k] : nullptr;
  if (res) *res = r;
  return KF_OK;
}

extern "C" int kf_fusion_save(kf_fusion f, const char *path, void *stream) {
  KF_REQUIRE(f && path, "NULL argument");
  return kf_state_save(path, f->can, f->psi, f->frames, stream);
}

extern "C" int kf_fusion_load(kf_fusion f, const char *path, void *stream) {
  KF_REQUIRE(f && path, "NULL argument");
  int32_t frames = 0;
  int rc = kf_state_load(path, f->can, f->psi, &frames, stream);
  if (rc) return rc;
  KF_REQUIRE(frames >= 0, "negative frame count in the state file");
  f->frames = frames;
  return KF_OK;
}
