// C entry points over the reference's own SDF / DisplacementField /
// KillingFusion classes, compiled unmodified from the reference sources into
// oracle/_ref/libkf_ref.so (recipe: oracle/Makefile, target `ref`).  Tests use
// it to pin the FP64 restatement (oracle/kf_oracle.c) against the reference
// itself and to generate golden fixtures.  TEST INFRASTRUCTURE ONLY.
//
// The reference keeps computeDisplacementField / computeEnergyGradient and the
// SDF storage private (KillingFusion.h:42-58, SDF.h:17-31); this translation
// unit alone re-declares the class keyword as struct so that it can reach
// them.  Layouts follow the oracle: phi double[N], weights int64[N], psi
// double[N][3], index z*nx*ny + y*nx + x.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include <Eigen/Eigen>
#include <opencv2/opencv.hpp>
#include <config.h>

#define class struct
#define private public
#define protected public
#include <KillingFusion.h>
#undef protected
#undef private
#undef class

namespace {

SDF make_sdf(const int n[3], double voxel, double unknown_clip,
             const double *min3 = nullptr) {
  Eigen::Vector3d mn(0.0, 0.0, 0.0);
  if (min3) mn = Eigen::Vector3d(min3[0], min3[1], min3[2]);
  Eigen::Vector3d mx(mn(0) + (n[0] - 0.5) * voxel, mn(1) + (n[1] - 0.5) * voxel,
                     mn(2) + (n[2] - 0.5) * voxel);
  SDF s(voxel, mn, mx, unknown_clip);
  // The grid must come out with exactly the requested size.
  if (s.m_gridSize(0) != n[0] || s.m_gridSize(1) != n[1] || s.m_gridSize(2) != n[2]) {
    std::cerr << "ref_harness: grid size mismatch " << s.m_gridSize.transpose() << "\n";
    std::abort();
  }
  return s;
}

int64_t count(const int n[3]) { return (int64_t)n[0] * n[1] * n[2]; }

void load_sdf(SDF &s, const double *phi, const int64_t *w, int64_t N) {
  for (int64_t i = 0; i < N; ++i) {
    s.m_voxelGridTSDF[i] = phi ? phi[i] : 0.0;
    s.m_voxelGridWeight[i] = w ? (long)w[i] : 0;
  }
}

void store_sdf(const SDF &s, double *phi, int64_t *w, int64_t N) {
  for (int64_t i = 0; i < N; ++i) {
    if (phi) phi[i] = s.m_voxelGridTSDF[i];
    if (w) w[i] = s.m_voxelGridWeight[i];
  }
}

DisplacementField make_psi(const int n[3], const double *psi) {
  DisplacementField f(Eigen::Vector3i(n[0], n[1], n[2]), VoxelSize);
  if (psi)
    for (int64_t i = 0; i < count(n); ++i)
      f.m_gridDisplacementValue[i] = Eigen::Vector3d(psi[3 * i], psi[3 * i + 1], psi[3 * i + 2]);
  return f;
}

KillingFusion &fusion() {
  static KillingFusion *kf = new KillingFusion(DatasetReader(""));
  return *kf;
}

}  // namespace

extern "C" {

int ref_grid_size(const double bound[3], double voxel, int out[3]) {
  SDF s(voxel, Eigen::Vector3d(0.0, 0.0, 0.0), Eigen::Vector3d(bound[0], bound[1], bound[2]), 1.0);
  for (int k = 0; k < 3; ++k) out[k] = s.m_gridSize(k);
  return 0;
}

void ref_phi_sample(const double *phi, const int n[3], const double *pts, int cnt, double *out) {
  SDF s = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(s, phi, nullptr, count(n));
  for (int i = 0; i < cnt; ++i)
    out[i] = s.getDistance(Eigen::Vector3d(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
}

void ref_weight_sample(const int64_t *w, const int n[3], const double *pts, int cnt, double *out) {
  SDF s = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(s, nullptr, w, count(n));
  for (int i = 0; i < cnt; ++i)
    out[i] = s.getWeight(Eigen::Vector3d(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
}

void ref_psi_sample(const double *psi, const int n[3], const double *pts, int cnt, double *out) {
  DisplacementField f = make_psi(n, psi);
  for (int i = 0; i < cnt; ++i) {
    Eigen::Vector3d v = f.getDisplacementAtf(Eigen::Vector3d(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
    for (int k = 0; k < 3; ++k) out[3 * i + k] = v(k);
  }
}

void ref_distance_gradient_at(const double *phi, const int n[3], const double *pts, int cnt, double *out) {
  SDF s = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(s, phi, nullptr, count(n));
  for (int i = 0; i < cnt; ++i) {
    Eigen::Vector3d g = s.computeDistanceGradient(Eigen::Vector3d(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
    for (int k = 0; k < 3; ++k) out[3 * i + k] = g(k);
  }
}

void ref_distance_hessian_at(const double *phi, const int n[3], const double *pts, int cnt, double *out) {
  SDF s = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(s, phi, nullptr, count(n));
  for (int i = 0; i < cnt; ++i) {
    Eigen::Matrix3d H = s.computeDistanceHessian(Eigen::Vector3d(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) out[9 * i + 3 * r + c] = H(r, c);
  }
}

// Per-voxel quantities of the psi update at a list of voxels (xyz triples).
// what: 0 energy gradient, 1 distance gradient, 2 hessian (9), 3 Killing
// gradient, 4 warped value, 5 band test.
void ref_voxel_query(int what, const double *live, const double *can, const double *psi,
                     const int n[3], const int *xyz, int cnt, double *out) {
  SDF src = make_sdf(n, VoxelSize, UnknownClipDistance);
  SDF dst = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(src, live, nullptr, count(n));
  if (can) load_sdf(dst, can, nullptr, count(n));
  DisplacementField f = make_psi(n, psi);
  KillingFusion &kf = fusion();
  for (int i = 0; i < cnt; ++i) {
    Eigen::Vector3i v(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    if (what == 0) {
      Eigen::Vector3d g = kf.computeEnergyGradient(&src, &dst, &f, v);
      for (int k = 0; k < 3; ++k) out[3 * i + k] = g(k);
    } else if (what == 1) {
      Eigen::Vector3d g = src.computeDistanceGradient(v, &f);
      for (int k = 0; k < 3; ++k) out[3 * i + k] = g(k);
    } else if (what == 2) {
      Eigen::Matrix3d H = src.computeDistanceHessian(v, &f);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[9 * i + 3 * r + c] = H(r, c);
    } else if (what == 3) {
      Eigen::Vector3d g = f.computeKillingEnergyGradient2(v);
      for (int k = 0; k < 3; ++k) out[3 * i + k] = g(k);
    } else if (what == 4) {
      out[i] = src.getDistance(v, &f);
    } else {
      double s = src.getDistance(v, &f);
      out[i] = (s > MaxSurfaceVoxelDistance - epsilon || s < -UnknownClipDistance) ? 0.0 : 1.0;
    }
  }
}

// KillingFusion::computeDisplacementField with KILLING_MAX_ITERATIONS
// iterations of the Jacobi schedule.  Returns 0, or -1 on divergence.
int ref_solve(const double *live, const double *can, double *psi, const int n[3]) {
  SDF src = make_sdf(n, VoxelSize, UnknownClipDistance);
  SDF dst = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(src, live, nullptr, count(n));
  load_sdf(dst, can, nullptr, count(n));
  DisplacementField f = make_psi(n, psi);
  try {
    fusion().computeDisplacementField(&src, &dst, &f);
  } catch (int) {
    return -1;
  }
  for (int64_t i = 0; i < count(n); ++i)
    for (int k = 0; k < 3; ++k) psi[3 * i + k] = f.m_gridDisplacementValue[i](k);
  return 0;
}

void ref_jacobian(const double *psi, const int n[3], double x, double y, double z, double out[9]) {
  DisplacementField f = make_psi(n, psi);
  Eigen::Matrix3d J = f.computeJacobian(x, y, z);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[3 * r + c] = J(r, c);
}

double ref_killing_energy(const double *psi, const int n[3], double x, double y, double z) {
  DisplacementField f = make_psi(n, psi);
  return f.computeKillingEnergy(x, y, z);
}

void ref_killing_energy_gradient_fd(const double *psi, const int n[3], int x, int y, int z, double out[3]) {
  DisplacementField f = make_psi(n, psi);
  Eigen::Vector3d g = f.computeKillingEnergyGradient(Eigen::Vector3i(x, y, z));
  for (int k = 0; k < 3; ++k) out[k] = g(k);
}

// SDF::integrateDepthFrame on a grid with the given origin; c2w and K are
// row-major, depth row-major [height][width] in metres.
void ref_integrate(double *phi, int64_t *w, const int n[3], double voxel, const double min3[3],
                   double unknown_clip, const double *depth, int width, int height,
                   const double c2w[16], const double K[9], double min_depth, double max_depth) {
  SDF s = make_sdf(n, voxel, unknown_clip, min3);
  load_sdf(s, phi, w, count(n));
  Eigen::Matrix4d P;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) P(r, c) = c2w[4 * r + c];
  Eigen::Matrix3d KK;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) KK(r, c) = K[3 * r + c];
  cv::Mat img(height, width, const_cast<double *>(depth));
  s.integrateDepthFrame(img, P, KK, min_depth, max_depth);
  store_sdf(s, phi, w, count(n));
}

void ref_update(double *phi, int64_t *w, const double *psi, const int n[3]) {
  SDF s = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(s, phi, w, count(n));
  DisplacementField f = make_psi(n, psi);
  s.update(&f);
  store_sdf(s, phi, w, count(n));
}

void ref_fuse(double *phi1, int64_t *w1, const double *phi2, const int64_t *w2, const int n[3]) {
  SDF a = make_sdf(n, VoxelSize, UnknownClipDistance);
  SDF b = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(a, phi1, w1, count(n));
  load_sdf(b, phi2, w2, count(n));
  a.fuse(&b);
  store_sdf(a, phi1, w1, count(n));
}

void ref_fuse_psi(double *phi1, int64_t *w1, const double *phi2, const int64_t *w2,
                  const double *psi, const int n[3]) {
  SDF a = make_sdf(n, VoxelSize, UnknownClipDistance);
  SDF b = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(a, phi1, w1, count(n));
  load_sdf(b, phi2, w2, count(n));
  DisplacementField f = make_psi(n, psi);
  a.fuse(&b, &f);
  store_sdf(a, phi1, w1, count(n));
}

// SDF::getMesh: 9 doubles per triangle (vertices as stored by
// SimpleMesh::AddVertex); returns the triangle count, writes at most cap.
int64_t ref_mesh(const double *phi, const int n[3], double *verts, int64_t cap) {
  SDF s = make_sdf(n, VoxelSize, UnknownClipDistance);
  load_sdf(s, phi, nullptr, count(n));
  SimpleMesh *m = s.getMesh();
  std::vector<Vertex> &V = m->GetVertices();
  std::vector<Triangle> &T = m->GetTriangles();
  int64_t nt = (int64_t)T.size();
  for (int64_t t = 0; t < nt && t < cap; ++t) {
    unsigned idx[3] = {T[t].idx0, T[t].idx1, T[t].idx2};
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) verts[9 * t + 3 * j + k] = V[idx[j]](k);
  }
  delete m;
  return nt;
}

// SDF::getDataEnergyTestSample (SDF.cpp:64-115): the two-sphere fixture of
// processTest.  n receives the grid size; arrays must hold 1000 entries.
void ref_two_spheres(double voxel, double unknown_clip, int n[3], double *phi0, int64_t *w0,
                     double *phi1, int64_t *w1) {
  std::vector<SDF> s = SDF::getDataEnergyTestSample(voxel, unknown_clip);
  for (int k = 0; k < 3; ++k) n[k] = s[0].m_gridSize(k);
  store_sdf(s[0], phi0, w0, count(n));
  store_sdf(s[1], phi1, w1, count(n));
}

}  // extern "C"
