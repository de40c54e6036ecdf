// Canonical-state files (checkpoint and resume of a frame sequence) and the
// reader of the reference's SDF dump.
//
// The reference only writes (SDF::dumpToBinFile, SDF.cpp:432-446: phi as
// doubles, no weights; DisplacementField::dumpToBinFile,
// DisplacementField.cpp:349-366), so a sequence cannot be resumed from its
// files.  The state file written here holds what the frame pipeline needs
// to continue bit for bit: the canonical SDF's float32 values and int32
// weights, psi (float32 or float64 planes) and the frame counter, with the
// grid's geometry in a header:
//   char magic[8] = "KFSTATE2"; int32 version = 2; int32 dims[3];
//   double min3d[3]; double voxel; double unknown_clip; int32 frame;
//   int32 flags (1: psi present, 2: psi float64); int64 count;
//   float phi[count]; int32 weight[count]; psi x, y, z planes[count] (if any)
// little-endian, as the host writes it.  Large grids go through a fixed
// pinned staging buffer in chunks.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <string>

#include "kf_internal.h"

namespace {

constexpr char kMagic[8] = {'K', 'F', 'S', 'T', 'A', 'T', 'E', '2'};
constexpr int32_t kVersion = 2;
constexpr size_t kChunk = 32u << 20;  // staging bytes per copy

#pragma pack(push, 1)
struct StateHeader {
  char magic[8];
  int32_t version;
  int32_t dims[3];
  double min3d[3];
  double voxel;
  double unknown_clip;
  int32_t frame;
  int32_t flags;
  int64_t count;
};
#pragma pack(pop)

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

struct Pinned {
  void *p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// device -> file, `bytes` from dev through the staging buffer
int write_device(FILE *f, const void *dev, size_t bytes, void *stage, cudaStream_t s) {
  for (size_t off = 0; off < bytes; off += kChunk) {
    const size_t n = bytes - off < kChunk ? bytes - off : kChunk;
    KF_CHECK_CUDA(cudaMemcpyAsync(stage, (const char *)dev + off, n, cudaMemcpyDeviceToHost, s));
    KF_CHECK_CUDA(cudaStreamSynchronize(s));
    if (fwrite(stage, 1, n, f) != n) return kf_fail(KF_ERR_INVALID, "short write of the state file");
  }
  return KF_OK;
}

// file -> device
int read_device(FILE *f, void *dev, size_t bytes, void *stage, cudaStream_t s) {
  for (size_t off = 0; off < bytes; off += kChunk) {
    const size_t n = bytes - off < kChunk ? bytes - off : kChunk;
    KF_CHECK_CUDA(cudaStreamSynchronize(s));  // the staging buffer is free again
    if (fread(stage, 1, n, f) != n) return kf_fail(KF_ERR_INVALID, "the state file is truncated");
    KF_CHECK_CUDA(cudaMemcpyAsync((char *)dev + off, stage, n, cudaMemcpyHostToDevice, s));
  }
  KF_CHECK_CUDA(cudaStreamSynchronize(s));
  return KF_OK;
}

int read_header(FILE *f, const char *path, StateHeader *h) {
  if (fread(h, sizeof(*h), 1, f) != 1) return kf_fail(KF_ERR_INVALID, std::string("not a state file: ") + path);
  if (memcmp(h->magic, kMagic, 8) != 0 || h->version != kVersion)
    return kf_fail(KF_ERR_INVALID, std::string("not a version-2 state file: ") + path);
  if (h->dims[0] <= 0 || h->dims[1] <= 0 || h->dims[2] <= 0 ||
      h->count != (int64_t)h->dims[0] * h->dims[1] * h->dims[2])
    return kf_fail(KF_ERR_INVALID, std::string("corrupt state file header: ") + path);
  return KF_OK;
}

}  // namespace

extern "C" int kf_state_save(const char *path, kf_grid canonical, kf_field psi, int32_t frame, void *stream) {
  KF_REQUIRE(path && canonical, "NULL argument");
  if (psi)
    for (int k = 0; k < 3; ++k) KF_REQUIRE(psi->n[k] == canonical->n[k], "psi and the SDF differ in size");
  cudaStream_t s = kf_stream(stream);
  StateHeader h;
  memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  for (int k = 0; k < 3; ++k) {
    h.dims[k] = canonical->n[k];
    h.min3d[k] = canonical->min3d[k];
  }
  h.voxel = canonical->voxel;
  h.unknown_clip = canonical->unknown_clip;
  h.frame = frame;
  h.flags = psi ? (1 | (psi->prec == KF_F64 ? 2 : 0)) : 0;
  h.count = canonical->count;
  File f;
  f.f = fopen(path, "wb");
  if (!f.f) return kf_fail(KF_ERR_INVALID, std::string("cannot open for writing: ") + path);
  if (fwrite(&h, sizeof(h), 1, f.f) != 1) return kf_fail(KF_ERR_INVALID, "short write of the state file");
  Pinned stage;
  KF_CHECK_CUDA(cudaMallocHost(&stage.p, kChunk));
  int rc = write_device(f.f, canonical->phi, (size_t)h.count * sizeof(float), stage.p, s);
  if (!rc) rc = write_device(f.f, canonical->w, (size_t)h.count * sizeof(int32_t), stage.p, s);
  for (int k = 0; psi && !rc && k < 3; ++k)
    rc = write_device(f.f, psi->p[k], (size_t)h.count * kf_prec_size(psi->prec), stage.p, s);
  if (rc) return rc;
  if (fflush(f.f) != 0) return kf_fail(KF_ERR_INVALID, "short write of the state file");
  return KF_OK;
}

extern "C" int kf_state_info(const char *path, int dims[3], double *voxel, double min3d[3],
                             double *unknown_clip, int32_t *frame, int *psi_precision) {
  KF_REQUIRE(path, "NULL path");
  File f;
  f.f = fopen(path, "rb");
  if (!f.f) return kf_fail(KF_ERR_INVALID, std::string("cannot open: ") + path);
  StateHeader h;
  int rc = read_header(f.f, path, &h);
  if (rc) return rc;
  for (int k = 0; k < 3; ++k) {
    if (dims) dims[k] = h.dims[k];
    if (min3d) min3d[k] = h.min3d[k];
  }
  if (voxel) *voxel = h.voxel;
  if (unknown_clip) *unknown_clip = h.unknown_clip;
  if (frame) *frame = h.frame;
  if (psi_precision) *psi_precision = (h.flags & 1) ? ((h.flags & 2) ? KF_F64 : KF_F32) : -1;
  return KF_OK;
}

extern "C" int kf_state_load(const char *path, kf_grid canonical, kf_field psi, int32_t *frame, void *stream) {
  KF_REQUIRE(path && canonical, "NULL argument");
  cudaStream_t s = kf_stream(stream);
  File f;
  f.f = fopen(path, "rb");
  if (!f.f) return kf_fail(KF_ERR_INVALID, std::string("cannot open: ") + path);
  StateHeader h;
  int rc = read_header(f.f, path, &h);
  if (rc) return rc;
  for (int k = 0; k < 3; ++k)
    KF_REQUIRE(h.dims[k] == canonical->n[k], "the state file's grid differs in size from the SDF");
  KF_REQUIRE(h.voxel == canonical->voxel && h.min3d[0] == canonical->min3d[0] &&
                 h.min3d[1] == canonical->min3d[1] && h.min3d[2] == canonical->min3d[2],
             "the state file's grid differs in placement or voxel size from the SDF");
  const bool has_psi = (h.flags & 1) != 0;
  if (psi) {
    KF_REQUIRE(has_psi, "the state file holds no psi");
    for (int k = 0; k < 3; ++k) KF_REQUIRE(psi->n[k] == h.dims[k], "psi and the state file differ in size");
    KF_REQUIRE((psi->prec == KF_F64) == ((h.flags & 2) != 0), "psi and the state file differ in precision");
  }
  Pinned stage;
  KF_CHECK_CUDA(cudaMallocHost(&stage.p, kChunk));
  if (psi) kf_field_written(psi);
  rc = read_device(f.f, canonical->phi, (size_t)h.count * sizeof(float), stage.p, s);
  if (!rc) rc = read_device(f.f, canonical->w, (size_t)h.count * sizeof(int32_t), stage.p, s);
  for (int k = 0; psi && !rc && k < 3; ++k)
    rc = read_device(f.f, psi->p[k], (size_t)h.count * kf_prec_size(psi->prec), stage.p, s);
  if (rc) return rc;
  if (frame) *frame = h.frame;
  return KF_OK;
}

// The reference's SDF dump (SDF.cpp:432-446): int32 dims[3], double min[3],
// double voxel, double truncation (voxel units), double phi[N].
extern "C" int kf_grid_load_ref_bin(const char *path, const kf_params *p, double unknown_clip, kf_grid *out,
                                    double *truncation, void *stream) {
  KF_REQUIRE(path && p && out, "NULL argument");
  *out = nullptr;
  File f;
  f.f = fopen(path, "rb");
  if (!f.f) return kf_fail(KF_ERR_INVALID, std::string("cannot open: ") + path);
  int32_t dims[3];
  double min3d[3], voxel, trunc;
  if (fread(dims, sizeof(int32_t), 3, f.f) != 3 || fread(min3d, sizeof(double), 3, f.f) != 3 ||
      fread(&voxel, sizeof(double), 1, f.f) != 1 || fread(&trunc, sizeof(double), 1, f.f) != 1)
    return kf_fail(KF_ERR_INVALID, std::string("truncated SDF header: ") + path);
  KF_REQUIRE(dims[0] > 0 && dims[1] > 0 && dims[2] > 0 && voxel > 0.0, "corrupt SDF header");
  const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
  kf_grid g = nullptr;
  int dd[3] = {dims[0], dims[1], dims[2]};
  int rc = kf_grid_create(dd, voxel, min3d, unknown_clip, p, &g);
  if (rc) return rc;
  cudaStream_t s = kf_stream(stream);
  // values as float32; a voxel with a value other than the initial one
  // (MaxSurfaceVoxelDistance + epsilon, SDF.cpp:133) gets weight 1: the
  // file keeps no weights
  const float init = (float)(p->max_surface + p->epsilon);
  const size_t per = kChunk / 8;
  double *buf = nullptr;
  float *fphi = nullptr;
  int32_t *fw = nullptr;
  cudaError_t e = cudaMallocHost(&buf, per * sizeof(double));
  if (e == cudaSuccess) e = cudaMallocHost(&fphi, per * sizeof(float));
  if (e == cudaSuccess) e = cudaMallocHost(&fw, per * sizeof(int32_t));
  if (e != cudaSuccess) rc = kf_cuda_fail(e, "pinned staging of the SDF file");
  for (int64_t off = 0; !rc && off < n; off += (int64_t)per) {
    const size_t m = (size_t)(n - off < (int64_t)per ? n - off : (int64_t)per);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      rc = kf_cuda_fail(e, "kf_grid_load_ref_bin");
      break;
    }
    if (fread(buf, sizeof(double), m, f.f) != m) {
      rc = kf_fail(KF_ERR_INVALID, std::string("truncated SDF values: ") + path);
      break;
    }
    for (size_t k = 0; k < m; ++k) {
      fphi[k] = (float)buf[k];
      fw[k] = fphi[k] != init ? 1 : 0;
    }
    e = cudaMemcpyAsync(g->phi + off, fphi, m * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->w + off, fw, m * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = kf_cuda_fail(e, "kf_grid_load_ref_bin copy");
  }
  cudaStreamSynchronize(s);
  cudaFreeHost(buf);
  cudaFreeHost(fphi);
  cudaFreeHost(fw);
  if (rc) {
    kf_grid_destroy(g);
    return rc;
  }
  if (truncation) *truncation = trunc;
  *out = g;
  return KF_OK;
}
