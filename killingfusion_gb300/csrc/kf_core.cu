// Library core: error state, parameters, grid and field handles, and the
// host side of the hot-path entry points declared in include/killingfusion.h.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <string>

#include "kf_internal.h"
#include "kf_mc_tables.h"

// ---------------------------------------------------------------------------
// error state
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

int kf_fail(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}

int kf_cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return e == cudaErrorMemoryAllocation ? KF_ERR_OOM : KF_ERR_CUDA;
}

extern "C" int kf_version(void) { return KF_ABI_VERSION; }

// Limit of a device-side wait (the grid-wide barrier of the persistent
// kernels); one second unless kf_set_wait_limit changes it.
static std::atomic<double> g_wait_limit_s{1.0};

extern "C" double kf_set_wait_limit(double seconds) {
  if (!(seconds >= 0.0) || seconds > 60.0) return -1.0;
  return g_wait_limit_s.exchange(seconds);
}

unsigned long long kf_wait_limit_ns() { return (unsigned long long)(g_wait_limit_s.load() * 1e9); }

// Bounds-check build mode: the records of the translation units with
// checked kernels, summed; the first failed check of the first unit that
// has one.
extern "C" int kf_bounds_status(int *enabled, int64_t *violations, int *site, int64_t *index, int64_t *bound) {
#ifdef KF_BOUNDS_CHECK
  if (enabled) *enabled = 1;
#else
  if (enabled) *enabled = 0;
#endif
  int (*readers[])(KfBoundsRecord *) = {kf_bounds_tu_read_fused, kf_bounds_tu_read_batch, kf_bounds_tu_read_exact,
                                        kf_bounds_tu_read_mc};
  int64_t total = 0;
  KfBoundsRecord first = {0u, 0, 0, 0};
  for (auto rd : readers) {
    KfBoundsRecord r;
    KF_CHECK_CUDA((cudaError_t)rd(&r));
    if (r.count && !first.count) first = r;
    total += r.count;
  }
  if (violations) *violations = total;
  if (site) *site = first.site;
  if (index) *index = first.index;
  if (bound) *bound = first.bound;
  return KF_OK;
}

extern "C" int kf_bounds_reset(int64_t limit) {
  const long long l = limit > 0 ? (long long)limit : 0x7fffffffffffffffLL;
  int (*resets[])(long long) = {kf_bounds_tu_reset_fused, kf_bounds_tu_reset_batch, kf_bounds_tu_reset_exact,
                                kf_bounds_tu_reset_mc};
  for (auto rs : resets) KF_CHECK_CUDA((cudaError_t)rs(l));
  return KF_OK;
}

extern "C" const char *kf_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
extern "C" void kf_params_reference(kf_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->voxel_size = 0.012;
  p->unknown_clip = 0.012 * 4;
  p->max_surface = 0.012 * 4;
  p->epsilon = 0.00001;
  p->delta_size = 0.05;
  p->alpha = 0.025;
  p->omega_k = 0.04;
  p->gamma_k = 0.0;
  p->omega_s = 0.1;
  p->threshold = 0.000001;
  p->killing_clamp = 0.1;
  p->use_data = p->use_levelset = p->use_killing = 1;
  p->early_exit = 0;
}

extern "C" void kf_params_paper(kf_params *p, double voxel_size, double trunc_voxels) {
  kf_params_reference(p);
  if (!p) return;
  p->voxel_size = voxel_size;
  p->unknown_clip = voxel_size * trunc_voxels;
  p->max_surface = voxel_size * trunc_voxels;
  p->alpha = 0.1;
  p->omega_k = 0.5;
  p->gamma_k = 0.1;
  p->omega_s = 0.2;
}

int kf_check_params(const kf_params *p) {
  KF_REQUIRE(p, "params is NULL");
  KF_REQUIRE(p->voxel_size > 0 && isfinite(p->voxel_size), "voxel_size must be > 0");
  KF_REQUIRE(p->delta_size > 0 && p->delta_size < 0.25, "delta_size must lie in (0, 0.25)");
  KF_REQUIRE(isfinite(p->unknown_clip) && isfinite(p->max_surface) && isfinite(p->epsilon),
             "non-finite band parameters");
  KF_REQUIRE(p->killing_clamp > 0, "killing_clamp must be > 0");
  return KF_OK;
}

// Largest float <= v and smallest float >= v.
static float float_down(double v) {
  float f = (float)v;
  if ((double)f > v) f = nextafterf(f, -INFINITY);
  return f;
}
static float float_up(double v) {
  float f = (float)v;
  if ((double)f < v) f = nextafterf(f, INFINITY);
  return f;
}

DevParams kf_make_dev_params(const int n[3], const kf_params *p) {
  DevParams d;
  memset(&d, 0, sizeof(d));
  d.nx = n[0];
  d.ny = n[1];
  d.nz = n[2];
  d.count = (int64_t)n[0] * n[1] * n[2];
  d.voxel_size = p->voxel_size;
  d.unknown_clip = p->unknown_clip;
  d.max_surface = p->max_surface;
  d.epsilon = p->epsilon;
  d.delta_size = p->delta_size;
  d.alpha = p->alpha;
  d.omega_k = p->omega_k;
  d.gamma_k = p->gamma_k;
  d.omega_s = p->omega_s;
  d.killing_clamp = p->killing_clamp;
  d.oob_phi = p->max_surface + p->epsilon;
  d.band_hi = p->max_surface - p->epsilon;
  d.band_hi_f = float_down(d.band_hi);
  d.band_lo_f = float_up(-p->unknown_clip);
  d.pv_lo_f = float_up(-p->max_surface + p->epsilon);
  d.mc_hi_f = float_down(p->max_surface);
  d.oob_phi_f = (float)d.oob_phi;
  d.use_data = p->use_data;
  d.use_levelset = p->use_levelset;
  d.use_killing = p->use_killing;
  d.early_exit = p->early_exit;
  d.threshold = p->threshold;
  d.trust = p->use_trust && p->use_data && !p->use_levelset && !p->use_killing;
  return d;
}

int kf_num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

extern "C" int kf_mc_case(int cube, int *edge_mask, int tri_edges[16]) {
  KF_REQUIRE(cube >= 0 && cube < 256, "cube index out of range");
  if (edge_mask) *edge_mask = kf_mc_edge_mask_host(cube);
  if (tri_edges) kf_mc_tri_row_host(cube, tri_edges);
  return KF_OK;
}

// ---------------------------------------------------------------------------
// grids
// ---------------------------------------------------------------------------
static bool dims_ok(const int n[3]) {
  if (!n) return false;
  for (int k = 0; k < 3; ++k)
    if (n[k] <= 0) return false;
  // the reference indexes with int (DisplacementField.cpp:24-34)
  return (int64_t)n[0] * n[1] * n[2] < (int64_t)INT32_MAX;
}

// phi = v, w = 0 with 16-byte stores (the planes come from cudaMalloc,
// 256-byte aligned); the last n % 4 entries one by one.
__global__ void k_fill(float *phi, int32_t *w, int64_t n, float v) {
  const int64_t n4 = n >> 2;
  const float4 v4 = make_float4(v, v, v, v);
  const int4 z4 = make_int4(0, 0, 0, 0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    reinterpret_cast<float4 *>(phi)[i] = v4;
    reinterpret_cast<int4 *>(w)[i] = z4;
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    phi[4 * n4 + threadIdx.x] = v;
    w[4 * n4 + threadIdx.x] = 0;
  }
}

extern "C" int kf_grid_reset(kf_grid g, const kf_params *p, void *stream) {
  KF_REQUIRE(g, "grid is NULL");
  int rc = kf_check_params(p);
  if (rc) return rc;
  float v = (float)(p->max_surface + p->epsilon);
  const int64_t blocks = std::min<int64_t>((g->count / 4 + 255) / 256 + 1, (int64_t)kf_num_sms() * 16);
  k_fill<<<(unsigned)blocks, 256, 0, kf_stream(stream)>>>(g->phi, g->w, g->count, v);
  KF_CHECK_LAUNCH("k_fill");
  return KF_OK;
}

extern "C" int kf_grid_create(const int dims[3], double voxel_size, const double min3d[3],
                              double unknown_clip, const kf_params *p, kf_grid *out) {
  KF_REQUIRE(out, "out is NULL");
  *out = nullptr;
  KF_REQUIRE(dims_ok(dims), "grid dims must be positive with fewer than 2^31 voxels");
  KF_REQUIRE(voxel_size > 0, "voxel_size must be > 0");
  int rc = kf_check_params(p);
  if (rc) return rc;
  kf_grid g = new kf_grid_s();
  memset(g, 0, sizeof(*g));
  for (int k = 0; k < 3; ++k) {
    g->n[k] = dims[k];
    g->min3d[k] = min3d ? min3d[k] : 0.0;
  }
  g->count = (int64_t)dims[0] * dims[1] * dims[2];
  g->voxel = voxel_size;
  g->unknown_clip = unknown_clip;
  if (cudaMalloc(&g->phi, g->count * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&g->w, g->count * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&g->ctr, 256) != cudaSuccess) {
    cudaGetLastError();
    kf_grid_destroy(g);
    return kf_fail(KF_ERR_OOM, "cudaMalloc of the SDF grid failed");
  }
  rc = kf_grid_reset(g, p, nullptr);
  if (rc) {
    kf_grid_destroy(g);
    return rc;
  }
  *out = g;
  return KF_OK;
}

extern "C" int kf_grid_destroy(kf_grid g) {
  if (!g) return KF_OK;
  cudaFree(g->phi);
  cudaFree(g->w);
  cudaFree(g->phi_alt);
  cudaFree(g->w_alt);
  cudaFree(g->depth);
  cudaFree(g->integ);
  cudaFree(g->mc);
  cudaFree(g->ctr);
  delete g;
  return KF_OK;
}

extern "C" int kf_grid_info(kf_grid g, int dims[3], double *voxel_size, double min3d[3],
                            double *unknown_clip) {
  KF_REQUIRE(g, "grid is NULL");
  for (int k = 0; k < 3; ++k) {
    if (dims) dims[k] = g->n[k];
    if (min3d) min3d[k] = g->min3d[k];
  }
  if (voxel_size) *voxel_size = g->voxel;
  if (unknown_clip) *unknown_clip = g->unknown_clip;
  return KF_OK;
}

extern "C" int kf_grid_upload(kf_grid g, const float *phi, const int32_t *weight, void *stream) {
  KF_REQUIRE(g, "grid is NULL");
  cudaStream_t s = kf_stream(stream);
  if (phi) KF_CHECK_CUDA(cudaMemcpyAsync(g->phi, phi, g->count * sizeof(float), cudaMemcpyDefault, s));
  if (weight)
    KF_CHECK_CUDA(cudaMemcpyAsync(g->w, weight, g->count * sizeof(int32_t), cudaMemcpyDefault, s));
  KF_CHECK_CUDA(cudaStreamSynchronize(s));
  return KF_OK;
}

extern "C" int kf_grid_download(kf_grid g, float *phi, int32_t *weight, void *stream) {
  KF_REQUIRE(g, "grid is NULL");
  cudaStream_t s = kf_stream(stream);
  if (phi) KF_CHECK_CUDA(cudaMemcpyAsync(phi, g->phi, g->count * sizeof(float), cudaMemcpyDefault, s));
  if (weight)
    KF_CHECK_CUDA(cudaMemcpyAsync(weight, g->w, g->count * sizeof(int32_t), cudaMemcpyDefault, s));
  KF_CHECK_CUDA(cudaStreamSynchronize(s));
  return KF_OK;
}

extern "C" int kf_grid_device(kf_grid g, float **phi, int32_t **weight) {
  KF_REQUIRE(g, "grid is NULL");
  if (phi) *phi = g->phi;
  if (weight) *weight = g->w;
  return KF_OK;
}

// ---------------------------------------------------------------------------
// displacement fields
// ---------------------------------------------------------------------------
size_t kf_prec_size(kf_precision p) { return p == KF_F64 ? sizeof(double) : sizeof(float); }

extern "C" int kf_field_destroy(kf_field f) {
  if (!f) return KF_OK;
  for (int k = 0; k < 3; ++k) {
    cudaFree(f->p[k]);
    cudaFree(f->q[k]);
  }
  kf_field_release_solver(f);
  delete f;
  return KF_OK;
}

extern "C" int kf_field_create(const int dims[3], kf_precision prec, kf_field *out) {
  KF_REQUIRE(out, "out is NULL");
  *out = nullptr;
  KF_REQUIRE(dims_ok(dims), "field dims must be positive with fewer than 2^31 voxels");
  KF_REQUIRE(prec == KF_F32 || prec == KF_F64, "unknown precision");
  kf_field f = new kf_field_s();
  memset(f, 0, sizeof(*f));
  for (int k = 0; k < 3; ++k) f->n[k] = dims[k];
  f->count = (int64_t)dims[0] * dims[1] * dims[2];
  f->prec = prec;
  for (int k = 0; k < 3; ++k) {
    if (cudaMalloc(&f->p[k], f->count * kf_prec_size(prec)) != cudaSuccess) {
      cudaGetLastError();
      kf_field_destroy(f);
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the displacement field failed");
    }
  }
  int rc = kf_field_zero(f, nullptr);
  if (rc) {
    kf_field_destroy(f);
    return rc;
  }
  KF_CHECK_CUDA(cudaDeviceSynchronize());
  *out = f;
  return KF_OK;
}

int kf_field_stats(kf_field f, int iterations, IterStats **dev) {
  if (f->stats_cap < iterations) {
    cudaFree(f->stats);
    cudaFreeHost(f->stats_host);
    f->stats = nullptr;
    f->stats_host = nullptr;
    f->stats_cap = 0;
    int cap = iterations < 64 ? 64 : iterations;
    if (cudaMalloc(&f->stats, sizeof(IterStats) * cap) != cudaSuccess ||
        cudaMallocHost(&f->stats_host, sizeof(IterStats) * cap) != cudaSuccess) {
      cudaGetLastError();
      return kf_fail(KF_ERR_OOM, "allocation of the solver statistics failed");
    }
    f->stats_cap = cap;
  }
  *dev = f->stats;
  return KF_OK;
}

int kf_field_band_list(kf_field f, int **out) {
  if (!f->band && cudaMalloc(&f->band, 2 * f->count * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    f->band = nullptr;
    return kf_fail(KF_ERR_OOM, "cudaMalloc of the band voxel list failed");
  }
  *out = f->band;
  return KF_OK;
}

int kf_field_trust_rows(kf_field f, int **out) {
  if (!f->rows &&
      cudaMalloc(&f->rows, 2 * (size_t)f->n[1] * f->n[2] * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    f->rows = nullptr;
    return kf_fail(KF_ERR_OOM, "cudaMalloc of the trust-region row table failed");
  }
  *out = f->rows;
  return KF_OK;
}

int kf_field_sync(kf_field f, void **out) {
  if (!f->sync && cudaMalloc(&f->sync, 256) != cudaSuccess) {
    cudaGetLastError();
    f->sync = nullptr;
    return kf_fail(KF_ERR_OOM, "cudaMalloc of the persistent pass's barrier failed");
  }
  *out = f->sync;
  return KF_OK;
}

int kf_field_records(kf_field f, cudaStream_t s, KfRecords *r) {
  // touched[count], 64 words of counters, the bitmap
  const size_t words = (size_t)(f->count + 31) / 32;
  if (!f->touched) {
    if (cudaMalloc(&f->touched, ((size_t)f->count + 64 + words) * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      f->touched = nullptr;
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the field's records failed");
    }
    KF_CHECK_CUDA(cudaMemsetAsync(f->touched + f->count + 64, 0, words * sizeof(int), s));
  }
  r->touched = f->touched;
  r->touched_n = reinterpret_cast<unsigned *>(f->touched + f->count);
  r->side_n = r->touched_n + 1;
  r->moved = reinterpret_cast<unsigned *>(f->touched + f->count + 64);
  return KF_OK;
}

void kf_field_release_solver(kf_field f) {
  cudaFree(f->sync);
  f->sync = nullptr;
  cudaFree(f->touched);
  f->touched = nullptr;
  f->p_state = f->p_state == kPsiRecorded ? kPsiUnknown : f->p_state;
  f->q_state = f->q_state == kPsiRecorded ? kPsiUnknown : f->q_state;
  cudaFree(f->band);
  cudaFree(f->runs);
  f->runs = nullptr;
  f->runs_cap = 0;
  cudaFree(f->rows);
  f->rows = nullptr;
  for (int k = 0; k < 3; ++k) {
    if (f->ev[k]) cudaEventDestroy(f->ev[k]);
    f->ev[k] = nullptr;
  }
  f->pending = 0;
  f->band = nullptr;
  cudaFree(f->stats);
  cudaFreeHost(f->stats_host);
  cudaFree(f->plain_scratch);
  kf_fused_graph_destroy(f->graph);
  f->stats = nullptr;
  f->stats_host = nullptr;
  f->plain_scratch = nullptr;
  f->graph = nullptr;
  f->stats_cap = 0;
  f->plain_bytes = 0;
}

int kf_field_ensure_pair(kf_field f) {
  if (f->q[0]) return KF_OK;
  for (int k = 0; k < 3; ++k)
    if (cudaMalloc(&f->q[k], f->count * kf_prec_size(f->prec)) != cudaSuccess) {
      cudaGetLastError();
      for (int j = 0; j < 3; ++j) {
        cudaFree(f->q[j]);
        f->q[j] = nullptr;
      }
      return kf_fail(KF_ERR_OOM, "cudaMalloc of the displacement ping-pong buffer failed");
    }
  return KF_OK;
}

// kf_field_zero of float buffers that are zero outside the field's records:
// every plane of p and/or q (NULL: left alone) at the voxels touched[0, n),
// and q's planes at their entries [0, *side_n).
__global__ void k_zero_records(float *p0, float *p1, float *p2, float *q0, float *q1, float *q2,
                               const int *__restrict__ touched, const unsigned *touched_n,
                               const unsigned *side_n, int64_t count) {
  const int64_t n = *touched_n, m = q0 ? *side_n : 0u;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n + m; k += (int64_t)gridDim.x * blockDim.x) {
    if (k < n) {
      const int64_t v = touched[k];
      if (v < 0 || v >= count) continue;
      if (p0) p0[v] = p1[v] = p2[v] = 0.f;
      if (q0) q0[v] = q1[v] = q2[v] = 0.f;
    } else if (k - n < count) {
      q0[k - n] = q1[k - n] = q2[k - n] = 0.f;
    }
  }
}

extern "C" int kf_field_zero(kf_field f, void *stream) {
  KF_REQUIRE(f, "field is NULL");
  cudaStream_t s = kf_stream(stream);
  const int ps = f->exposed ? kPsiUnknown : f->p_state, qs = f->exposed ? kPsiUnknown : f->q_state;
  // the band-only solver's ping-pong buffer too, once that solver has used
  // the field: its first pass then reads phi_live alone (no copy of psi)
  const bool q_too = f->q[0] && f->q_zero_wanted;
  kf_field_written(f);  // (until every clear is queued)
  if (ps == kPsiRecorded || (q_too && qs == kPsiRecorded)) {
    KfRecords r;
    int rc = kf_field_records(f, s, &r);
    if (rc) return rc;
    const bool zp = ps == kPsiRecorded, zq = q_too && qs == kPsiRecorded;
    static bool carveout[64] = {};
    kf_prefer_carveout((const void *)k_zero_records, kBesideSolveCarveout, carveout);
    k_zero_records<<<(unsigned)kf_num_sms() * 4, 256, 0, s>>>(
        zp ? (float *)f->p[0] : nullptr, (float *)f->p[1], (float *)f->p[2], zq ? (float *)f->q[0] : nullptr,
        (float *)f->q[1], (float *)f->q[2], r.touched, r.touched_n, r.side_n, f->count);
    KF_CHECK_LAUNCH("k_zero_records");
  }
  const size_t bytes = f->count * kf_prec_size(f->prec);
  for (int k = 0; ps == kPsiUnknown && k < 3; ++k) KF_CHECK_CUDA(cudaMemsetAsync(f->p[k], 0, bytes, s));
  for (int k = 0; q_too && qs == kPsiUnknown && k < 3; ++k) KF_CHECK_CUDA(cudaMemsetAsync(f->q[k], 0, bytes, s));
  f->p_state = kPsiZero;
  f->q_state = q_too ? kPsiZero : qs;
  return KF_OK;
}

template <typename T>
__global__ void k_aos_to_soa(const T *__restrict__ aos, T *x, T *y, T *z, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    x[i] = aos[3 * i];
    y[i] = aos[3 * i + 1];
    z[i] = aos[3 * i + 2];
  }
}
template <typename T>
__global__ void k_soa_to_aos(T *__restrict__ aos, const T *x, const T *y, const T *z, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    aos[3 * i] = x[i];
    aos[3 * i + 1] = y[i];
    aos[3 * i + 2] = z[i];
  }
}

static int field_copy(kf_field f, void *xyz, bool upload, cudaStream_t s) {
  size_t bytes = 3 * f->count * kf_prec_size(f->prec);
  void *tmp = nullptr;
  KF_CHECK_CUDA(cudaMallocAsync(&tmp, bytes, s));
  unsigned nb = (unsigned)((f->count + 255) / 256);
  if (upload) {
    KF_CHECK_CUDA(cudaMemcpyAsync(tmp, xyz, bytes, cudaMemcpyDefault, s));
    if (f->prec == KF_F32)
      k_aos_to_soa<float><<<nb, 256, 0, s>>>((const float *)tmp, (float *)f->p[0], (float *)f->p[1],
                                              (float *)f->p[2], f->count);
    else
      k_aos_to_soa<double><<<nb, 256, 0, s>>>((const double *)tmp, (double *)f->p[0],
                                               (double *)f->p[1], (double *)f->p[2], f->count);
  } else {
    if (f->prec == KF_F32)
      k_soa_to_aos<float><<<nb, 256, 0, s>>>((float *)tmp, (const float *)f->p[0],
                                              (const float *)f->p[1], (const float *)f->p[2], f->count);
    else
      k_soa_to_aos<double><<<nb, 256, 0, s>>>((double *)tmp, (const double *)f->p[0],
                                               (const double *)f->p[1], (const double *)f->p[2],
                                               f->count);
    KF_CHECK_CUDA(cudaMemcpyAsync(xyz, tmp, bytes, cudaMemcpyDefault, s));
  }
  KF_CHECK_LAUNCH("field layout conversion");
  KF_CHECK_CUDA(cudaFreeAsync(tmp, s));
  KF_CHECK_CUDA(cudaStreamSynchronize(s));
  return KF_OK;
}

extern "C" int kf_field_upload(kf_field f, const void *xyz, void *stream) {
  KF_REQUIRE(f && xyz, "field or buffer is NULL");
  kf_field_written(f);
  return field_copy(f, const_cast<void *>(xyz), true, kf_stream(stream));
}

extern "C" int kf_field_download(kf_field f, void *xyz, void *stream) {
  KF_REQUIRE(f && xyz, "field or buffer is NULL");
  return field_copy(f, xyz, false, kf_stream(stream));
}

extern "C" int kf_field_device(kf_field f, void **px, void **py, void **pz) {
  KF_REQUIRE(f, "field is NULL");
  f->exposed = true;  // the caller may write the planes from now on
  kf_field_written(f);
  if (px) *px = f->p[0];
  if (py) *py = f->p[1];
  if (pz) *pz = f->p[2];
  return KF_OK;
}

// ---------------------------------------------------------------------------
// hot path
// ---------------------------------------------------------------------------
static bool same_dims(const int a[3], const int b[3]) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
}

// Gauss-Jordan inverse with partial pivoting of a row-major 4x4 matrix.
static bool invert4(const double m[16], double out[16]) {
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? m[4 * r + c] : (c - 4 == r ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int p = c;
    for (int r = c + 1; r < 4; ++r)
      if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
    if (a[p][c] == 0.0) return false;
    if (p != c)
      for (int k = 0; k < 8; ++k) {
        double t = a[c][k];
        a[c][k] = a[p][k];
        a[p][k] = t;
      }
    double piv = a[c][c];
    for (int k = 0; k < 8; ++k) a[c][k] = a[c][k] / piv;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      if (f == 0.0) continue;
      for (int k = 0; k < 8; ++k) a[r][k] = a[r][k] - f * a[c][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[4 * r + c] = a[r][c + 4];
  return true;
}

// The depth frame on the device: itself when it is device (or managed)
// memory, else copied into the grid's staging buffer.
static int stage_depth(kf_grid g, const void *depth, size_t bytes, cudaStream_t s, const void **dev) {
  cudaPointerAttributes attr;
  *dev = depth;
  if (cudaPointerGetAttributes(&attr, depth) != cudaSuccess || attr.type == cudaMemoryTypeUnregistered ||
      attr.type == cudaMemoryTypeHost) {
    cudaGetLastError();
    if (g->depth_cap < bytes) {
      cudaFree(g->depth);
      g->depth = nullptr;
      g->depth_cap = 0;
      if (cudaMalloc(&g->depth, bytes) != cudaSuccess) {
        cudaGetLastError();
        return kf_fail(KF_ERR_OOM, "cudaMalloc of the depth staging buffer failed");
      }
      g->depth_cap = bytes;
    }
    KF_CHECK_CUDA(cudaMemcpyAsync(g->depth, depth, bytes, cudaMemcpyHostToDevice, s));
    *dev = g->depth;
  }
  return KF_OK;
}

// Both depth formats of integration, into the grid as it is (fresh == NULL)
// or into a fresh grid of phi = *fresh, w = 0.
static int integrate_entry(kf_grid g, const void *depth, size_t pixel_bytes, int width, int height, double scale,
                           const double c2w[16], const double K[9], double min_depth, double max_depth,
                           const float *fresh, void *stream) {
  KF_REQUIRE(g && depth && c2w && K, "NULL argument");
  KF_REQUIRE(width > 0 && height > 0, "depth frame size must be positive");
  KF_REQUIRE(pixel_bytes == sizeof(float) || scale > 0.0, "depth scale must be positive");
  cudaStream_t s = kf_stream(stream);
  double w2c[16];
  KF_REQUIRE(invert4(c2w, w2c), "camera pose is singular");
  const void *dev = nullptr;
  int rc = stage_depth(g, depth, (size_t)width * height * pixel_bytes, s, &dev);
  if (rc) return rc;
  if (pixel_bytes == sizeof(float))
    return kf_launch_integrate(g, (const float *)dev, width, height, w2c, K, min_depth, max_depth, fresh, s);
  return kf_launch_integrate_u16(g, (const uint16_t *)dev, scale, width, height, w2c, K, min_depth, max_depth,
                                 fresh, s);
}

extern "C" int kf_integrate_depth(kf_grid g, const float *depth, int width, int height,
                                  const double c2w[16], const double K[9], double min_depth,
                                  double max_depth, void *stream) {
  return integrate_entry(g, depth, sizeof(float), width, height, 0.0, c2w, K, min_depth, max_depth, nullptr,
                         stream);
}

extern "C" int kf_integrate_depth_u16(kf_grid g, const uint16_t *depth, int width, int height, double scale,
                                      const double c2w[16], const double K[9], double min_depth,
                                      double max_depth, void *stream) {
  return integrate_entry(g, depth, sizeof(uint16_t), width, height, scale, c2w, K, min_depth, max_depth, nullptr,
                         stream);
}

extern "C" int kf_compute_sdf(kf_grid g, const kf_params *p, const float *depth, int width, int height,
                              const double c2w[16], const double K[9], double min_depth, double max_depth,
                              void *stream) {
  int rc = kf_check_params(p);
  if (rc) return rc;
  const float fresh = (float)(p->max_surface + p->epsilon);  // kf_grid_reset's value
  return integrate_entry(g, depth, sizeof(float), width, height, 0.0, c2w, K, min_depth, max_depth, &fresh,
                         stream);
}

extern "C" int kf_compute_sdf_u16(kf_grid g, const kf_params *p, const uint16_t *depth, int width, int height,
                                  double scale, const double c2w[16], const double K[9], double min_depth,
                                  double max_depth, void *stream) {
  int rc = kf_check_params(p);
  if (rc) return rc;
  const float fresh = (float)(p->max_surface + p->epsilon);
  return integrate_entry(g, depth, sizeof(uint16_t), width, height, scale, c2w, K, min_depth, max_depth, &fresh,
                         stream);
}

extern "C" int kf_warp(kf_grid g, kf_field psi, const kf_params *p, void *stream) {
  KF_REQUIRE(g && psi, "NULL argument");
  KF_REQUIRE(same_dims(g->n, psi->n), "grid and field sizes differ");
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(g->n, p);
  return kf_launch_warp(g, psi, dp, kf_stream(stream));
}

extern "C" int kf_fuse(kf_grid canonical, kf_grid other, void *stream) {
  KF_REQUIRE(canonical && other, "NULL argument");
  KF_REQUIRE(same_dims(canonical->n, other->n), "grid sizes differ");
  return kf_launch_fuse(canonical, other, kf_stream(stream));
}

extern "C" int kf_warp_fuse(kf_grid canonical, kf_grid live, kf_field psi, const kf_params *p,
                            void *stream) {
  KF_REQUIRE(canonical && live && psi, "NULL argument");
  KF_REQUIRE(canonical != live, "canonical and live must differ");
  KF_REQUIRE(same_dims(canonical->n, live->n) && same_dims(live->n, psi->n), "sizes differ");
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(live->n, p);
  return kf_launch_warp_fuse(canonical, live, psi, dp, kf_stream(stream));
}

extern "C" int kf_fuse_warped(kf_grid dst, kf_grid other, kf_field psi, const kf_params *p,
                              void *stream) {
  KF_REQUIRE(dst && other && psi, "NULL argument");
  KF_REQUIRE(dst != other, "dst and other must differ");
  KF_REQUIRE(same_dims(dst->n, other->n) && same_dims(dst->n, psi->n), "sizes differ");
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(dst->n, p);
  return kf_launch_fuse_warped(dst, other, psi, dp, kf_stream(stream));
}

extern "C" int kf_psi_gradient_ref(kf_grid live, kf_grid canonical, kf_field psi,
                                   const kf_params *p, const int32_t *voxels, int count,
                                   double *out, uint8_t *active, void *stream) {
  KF_REQUIRE(live && canonical && psi && out && (voxels || count == 0), "NULL argument");
  KF_REQUIRE(count >= 0, "count must be >= 0");
  KF_REQUIRE(same_dims(live->n, canonical->n) && same_dims(live->n, psi->n), "sizes differ");
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(live->n, p);
  return kf_gradient_ref_launch(live, canonical, psi, dp, voxels, count, out, active,
                                kf_stream(stream));
}

extern "C" int kf_marching_cubes(kf_grid g, const kf_params *p, float *verts, int64_t capacity,
                                 int64_t *ntri, void *stream) {
  KF_REQUIRE(g && ntri, "NULL argument");
  KF_REQUIRE(capacity >= 0, "capacity must be >= 0");
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(g->n, p);
  return kf_mc_run(g, dp, verts, capacity, ntri, kf_stream(stream));
}

extern "C" int kf_marching_cubes_async(kf_grid g, const kf_params *p, float *verts, int64_t capacity,
                                       int64_t *ntri, void *stream) {
  KF_REQUIRE(g && ntri, "NULL argument");
  KF_REQUIRE(capacity >= 0, "capacity must be >= 0");
  cudaPointerAttributes at;
  KF_REQUIRE(cudaPointerGetAttributes(&at, ntri) == cudaSuccess &&
                 (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeHost ||
                  at.type == cudaMemoryTypeManaged),
             "ntri must be device, pinned host or managed memory");
  int rc = kf_check_params(p);
  if (rc) return rc;
  DevParams dp = kf_make_dev_params(g->n, p);
  int64_t unused = 0;
  return kf_mc_run(g, dp, verts, capacity, &unused, kf_stream(stream), ntri);
}

extern "C" int kf_mesh_host(kf_grid g, const kf_params *p, float *verts, int64_t capacity,
                            int64_t *ntri, void *stream) {
  KF_REQUIRE(g && ntri, "NULL argument");
  KF_REQUIRE(capacity >= 0, "capacity must be >= 0");
  int rc = kf_check_params(p);
  if (rc) return rc;
  cudaStream_t s = kf_stream(stream);
  DevParams dp = kf_make_dev_params(g->n, p);
  if (!verts || capacity == 0) return kf_mc_run(g, dp, nullptr, 0, ntri, s);
  float *dev = nullptr;
  KF_CHECK_CUDA(cudaMallocAsync((void **)&dev, (size_t)capacity * 9 * sizeof(float), s));
  rc = kf_mc_run(g, dp, dev, capacity, ntri, s);
  if (rc == KF_OK || rc == KF_ERR_CAPACITY) {
    int64_t n = *ntri < capacity ? *ntri : capacity;
    if (n > 0) {
      cudaError_t e = cudaMemcpyAsync(verts, dev, (size_t)n * 9 * sizeof(float), cudaMemcpyDefault, s);
      if (e != cudaSuccess) rc = kf_cuda_fail(e, "mesh copy to host");
    }
  }
  cudaFreeAsync(dev, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess && rc == KF_OK) rc = kf_cuda_fail(e, "kf_mesh_host");
  if (rc == KF_ERR_CAPACITY)
    return kf_fail(KF_ERR_CAPACITY, "vertex buffer holds fewer triangles than the mesh has");
  return rc;
}

// ---------------------------------------------------------------------------
// psi solve
// ---------------------------------------------------------------------------
// Queues a solve and the copy of its statistics to the field's pinned
// mirror; *launched = 0 when there was nothing to queue (iterations == 0).
static int solve_launch(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p, int iterations,
                        kf_solver solver, cudaStream_t s, int *launched) {
  *launched = 0;
  KF_REQUIRE(live && canonical && psi, "NULL argument");
  KF_REQUIRE(live != canonical, "live and canonical must differ");
  KF_REQUIRE(same_dims(live->n, canonical->n) && same_dims(live->n, psi->n), "sizes differ");
  KF_REQUIRE(iterations >= 0, "iterations must be >= 0");
  int rc = kf_check_params(p);
  if (rc) return rc;
  KF_REQUIRE(solver == KF_SOLVER_FUSED || solver == KF_SOLVER_PLAIN || solver == KF_SOLVER_EXACT ||
                 solver == KF_SOLVER_BAND || solver == KF_SOLVER_PERVOXEL,
             "unknown solver");
  KF_REQUIRE((solver == KF_SOLVER_EXACT) == (psi->prec == KF_F64),
             "KF_SOLVER_EXACT runs on KF_F64 fields and the other solvers on KF_F32 fields");
  KF_REQUIRE(!(p->use_trust && p->use_data && !p->use_levelset && !p->use_killing &&
               solver == KF_SOLVER_PLAIN),
             "the trust-region step (use_trust) runs in KF_SOLVER_FUSED, _BAND and _EXACT, not _PLAIN");
  if (iterations == 0) return KF_OK;
  DevParams dp = kf_make_dev_params(live->n, p);
  IterStats *st = nullptr;
  // one extra record: the band solver counts the next iteration's list there
  rc = kf_field_stats(psi, iterations + 1, &st);
  if (rc) return rc;
  KF_CHECK_CUDA(cudaMemsetAsync(st, 0, sizeof(IterStats) * (iterations + 1), s));
  for (int k = 0; k < 3; ++k)
    if (!psi->ev[k]) KF_CHECK_CUDA(cudaEventCreate(&psi->ev[k]));
  KF_CHECK_CUDA(cudaEventRecord(psi->ev[0], s));
  // every solver writes psi's planes; the band-only solver's first pass
  // reads phi_live alone when both start at zero, and from now on
  // kf_field_zero clears its ping-pong buffer too
  const bool p_zero = !psi->exposed && psi->p_state == kPsiZero;
  const bool q_zero = !psi->exposed && psi->q_state == kPsiZero;
  kf_field_written(psi);
  if (solver == KF_SOLVER_BAND) psi->q_zero_wanted = true;
  if (solver == KF_SOLVER_PERVOXEL)
    rc = kf_solve_pervoxel(live, canonical, psi, dp, iterations, st, s);
  else if (solver == KF_SOLVER_FUSED || solver == KF_SOLVER_BAND)
    rc = kf_solve_fused(live, canonical, psi, dp, iterations, st, solver == KF_SOLVER_BAND, p_zero, q_zero, s);
  else if (solver == KF_SOLVER_PLAIN)
    rc = kf_solve_plain(live, canonical, psi, dp, iterations, st, s);
  else
    rc = kf_solve_exact(live, canonical, psi, dp, iterations, st, s);
  if (rc) return rc;
  KF_CHECK_CUDA(cudaEventRecord(psi->ev[1], s));
  KF_CHECK_CUDA(cudaMemcpyAsync(psi->stats_host, st, sizeof(IterStats) * (iterations + 1),
                                cudaMemcpyDeviceToHost, s));
  KF_CHECK_CUDA(cudaEventRecord(psi->ev[2], s));
  psi->last_iterations = iterations;
  psi->last_solver = solver;
  psi->pending = 1;
  *launched = 1;
  return KF_OK;
}

// Waits for the statistics of the last solve launched on psi and reads
// them.  presumed_swapped: the buffers were exchanged at launch on the
// assumption that every iteration runs (kf_psi_solve_async).
static int solve_finish(kf_field psi, kf_solve_stats *stats, bool presumed_swapped) {
  KF_CHECK_CUDA(cudaEventSynchronize(psi->ev[2]));
  psi->pending = 0;
  const IterStats *host = psi->stats_host;
  const int iterations = psi->last_iterations;
  const kf_solver solver = psi->last_solver;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, psi->ev[0], psi->ev[1]);
  if (solver == KF_SOLVER_PERVOXEL) {
    // record 0: voxels visited (list), their last monitored energy and
    // step, divergence; record 1: voxels that hit the cap (active), most
    // steps of a voxel (list)
    const int diverged = host[0].diverged;
    if (stats) {
      float md;
      unsigned bits = host[0].max_delta;
      memcpy(&md, &bits, sizeof(md));
      stats->iterations_run = (int32_t)host[1].list;
      stats->converged = (!diverged && host[1].active == 0) ? 1 : 0;
      stats->capped = (int32_t)host[1].active;
      stats->diverged = diverged;
      stats->active_first = stats->active_last = host[0].list;
      stats->energy_last = host[0].energy;
      stats->max_delta_last = md;
      stats->device_ms = ms;
    }
    if (diverged)
      return kf_fail(KF_ERR_DIVERGED, "deformation field diverged (non-finite psi inside the band)");
    return KF_OK;
  }
  if (host[0].timeout) {
    if (stats) stats->device_ms = ms;
    return kf_fail(KF_ERR_TIMEOUT, "a grid-wide wait of the persistent band pass gave up (limit " +
                                       std::to_string(kf_wait_limit_ns() / 1e9) + " s); psi is undefined");
  }
  for (int k = 0; k < iterations; ++k)
    if (host[k].cold)
      return kf_fail(KF_ERR_INTERNAL, "the split dense schedule found a band voxel in a run without band "
                                      "voxels at the first iteration");
  int executed = 0;
  int diverged = 0;
  for (int k = 0; k < iterations; ++k) {
    if (host[k].skipped) break;
    ++executed;
    if (host[k].diverged) {
      diverged = 1;
      break;
    }
  }
  // Iteration k reads buffer k%2 and writes (k+1)%2 (the dense fused solver
  // updates in place); a diverged iteration still wrote its output.  Put
  // the result into the primary planes.
  if (solver != KF_SOLVER_FUSED && !presumed_swapped && (executed & 1))
    for (int k = 0; k < 3; ++k) {
      void *t = psi->p[k];
      psi->p[k] = psi->q[k];
      psi->q[k] = t;
    }
  if (stats) {
    stats->iterations_run = executed;
    stats->converged = (!diverged && executed < iterations) ? 1 : 0;
    stats->diverged = diverged;
    if (executed > 0) {
      stats->active_first = host[0].active;
      stats->active_last = host[executed - 1].active;
      stats->energy_first = host[0].energy;
      stats->energy_last = host[executed - 1].energy;
      float md;
      unsigned bits = host[executed - 1].max_delta;
      memcpy(&md, &bits, sizeof(md));
      stats->max_delta_last = md;
    }
    stats->device_ms = ms;
  }
  if (diverged)
    return kf_fail(KF_ERR_DIVERGED, "deformation field diverged (non-finite psi inside the band)");
  return KF_OK;
}

extern "C" int kf_psi_solve(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
                            int iterations, kf_solver solver, kf_solve_stats *stats,
                            void *stream) {
  if (stats) memset(stats, 0, sizeof(*stats));
  int launched = 0;
  int rc = solve_launch(live, canonical, psi, p, iterations, solver, kf_stream(stream), &launched);
  if (rc || !launched) return rc;
  return solve_finish(psi, stats, false);
}

extern "C" int kf_psi_solve_async(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
                                  int iterations, kf_solver solver, void *stream) {
  KF_REQUIRE(p, "params is NULL");
  KF_REQUIRE(!(p->early_exit && solver != KF_SOLVER_FUSED && solver != KF_SOLVER_PERVOXEL),
             "kf_psi_solve_async with early_exit needs KF_SOLVER_FUSED or _PERVOXEL (the other solvers "
             "alternate two buffers, and which one holds psi depends on the iterations run)");
  int launched = 0;
  int rc = solve_launch(live, canonical, psi, p, iterations, solver, kf_stream(stream), &launched);
  if (rc || !launched) return rc;
  // every iteration runs (no early exit): psi ends in buffer iterations % 2
  if (solver != KF_SOLVER_FUSED && solver != KF_SOLVER_PERVOXEL && (iterations & 1))
    for (int k = 0; k < 3; ++k) {
      void *t = psi->p[k];
      psi->p[k] = psi->q[k];
      psi->q[k] = t;
    }
  psi->pending = 2;  // 2: launched by kf_psi_solve_async
  return KF_OK;
}

extern "C" int kf_psi_solve_history(kf_field psi, int32_t max_iterations, double *energy, double *max_delta,
                                    int64_t *active, int32_t *count) {
  KF_REQUIRE(psi && count, "NULL argument");
  KF_REQUIRE(max_iterations >= 0, "max_iterations must be >= 0");
  *count = 0;
  KF_REQUIRE(psi->stats_host && psi->last_iterations > 0, "no solve has run on this field");
  KF_REQUIRE(psi->pending == 0, "the last solve on this field has not been waited for (kf_psi_solve_wait)");
  KF_REQUIRE(psi->last_solver != KF_SOLVER_PERVOXEL,
             "the per-voxel schedule keeps no per-iteration statistics");
  int n = 0;
  for (int k = 0; k < psi->last_iterations && n < max_iterations; ++k) {
    const IterStats &h = psi->stats_host[k];
    if (h.skipped) break;
    float md;
    memcpy(&md, &h.max_delta, sizeof(md));
    if (energy) energy[n] = h.energy;
    if (max_delta) max_delta[n] = md;
    if (active) active[n] = h.active;
    ++n;
    if (h.diverged) break;
  }
  *count = n;
  return KF_OK;
}

extern "C" int kf_psi_solve_wait(kf_field psi, kf_solve_stats *stats) {
  KF_REQUIRE(psi, "NULL argument");
  if (stats) memset(stats, 0, sizeof(*stats));
  KF_REQUIRE(psi->pending == 2, "no kf_psi_solve_async pending on this field");
  int rc = solve_finish(psi, stats, true);
  if (rc == KF_OK && psi->last_solver != KF_SOLVER_FUSED && psi->last_solver != KF_SOLVER_PERVOXEL &&
      stats && stats->iterations_run != psi->last_iterations)
    return kf_fail(KF_ERR_INVALID, "an asynchronous solve stopped early; psi is in the other buffer");
  return rc;
}
