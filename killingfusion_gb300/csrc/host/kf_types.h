// Small value types standing in for the Eigen types of the reference's class
// API (Eigen::Vector3d/3i, Matrix3d/4d), and the run-time configuration that
// replaces the reference's compile-time config.h globals.
#pragma once

#include <cmath>
#include <cstdint>
#include <ostream>

#include "killingfusion.h"

namespace kf {

template <typename T>
struct Vec3 {
  T v[3] = {T(0), T(0), T(0)};
  Vec3() = default;
  Vec3(T a, T b, T c) : v{a, b, c} {}
  T &operator()(int i) { return v[i]; }
  T operator()(int i) const { return v[i]; }
  T &operator[](int i) { return v[i]; }
  T operator[](int i) const { return v[i]; }
  T x() const { return v[0]; }
  T y() const { return v[1]; }
  T z() const { return v[2]; }
  T *data() { return v; }
  const T *data() const { return v; }
  Vec3 operator+(const Vec3 &o) const { return Vec3(v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]); }
  Vec3 operator-(const Vec3 &o) const { return Vec3(v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]); }
  Vec3 operator*(T s) const { return Vec3(v[0] * s, v[1] * s, v[2] * s); }
  Vec3 operator/(T s) const { return Vec3(v[0] / s, v[1] / s, v[2] / s); }
  bool operator==(const Vec3 &o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
  T dot(const Vec3 &o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
  T norm() const { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
  T prod() const { return v[0] * v[1] * v[2]; }
};
typedef Vec3<double> Vec3d;
typedef Vec3<int> Vec3i;

template <typename T>
inline std::ostream &operator<<(std::ostream &os, const Vec3<T> &a) {
  return os << a.v[0] << " " << a.v[1] << " " << a.v[2];
}

// Row-major N x N matrix.
template <int N>
struct Mat {
  double m[N * N] = {};
  static Mat Identity() {
    Mat r;
    for (int i = 0; i < N; ++i) r.m[i * N + i] = 1.0;
    return r;
  }
  static Mat Zero() { return Mat(); }
  double &operator()(int r, int c) { return m[r * N + c]; }
  double operator()(int r, int c) const { return m[r * N + c]; }
  const double *data() const { return m; }
  bool isZero(double prec) const {
    for (int i = 0; i < N * N; ++i)
      if (std::fabs(m[i]) > prec) return false;
    return true;
  }
};
typedef Mat<3> Mat3d;
typedef Mat<4> Mat4d;

// The reference's configuration globals (config.h:11-74, values in
// config.cpp:4-57), settable at run time.
struct Config {
  double VoxelSize = 0.012;
  double UnknownClipDistance = 0.012 * 4;
  double MaxSurfaceVoxelDistance = 0.012 * 4;
  bool EnergyTypeUsed[3] = {true, true, true};  // data, level set, Killing
  bool UseZeroDisplacementFieldForNextFrame = true;
  // the trust-region step of the Jacobi schedule, data term alone
  // (config.cpp:27, KillingFusion.cpp:288-314)
  bool UseTrustStrategy = false;
  int KILLING_MAX_ITERATIONS = 1024;
  double deltaSize = 0.05;
  double alpha = 0.025;
  double threshold = 0.000001;
  double omegaKilling = 0.04;
  double gammaKilling = 0;
  double omegaLevelSet = 0.1;
  double epsilon = 0.00001;
  // solver of computeDisplacementField (the reference's Jacobi schedule in
  // one of its GPU forms, or its per-voxel schedule)
  kf_solver solver = KF_SOLVER_FUSED;
  // the dataset of the reference's directory layout (config.cpp:10-19):
  // 0 Duck, 1 Snoopy
  int datasetType = 1;
  const char *imageDir[2] = {"Duck/", "Snoopy/"};
  int numImageFiles[2] = {447, 630};
  const char *intrinsicParamsFile = "intrinsics_kinect1.txt";
  double datasetDepthMinMaxValues[2][2] = {{0.0497470, 1.2}, {0.0495164, 1.2}};

  kf_params params() const {
    kf_params p;
    kf_params_reference(&p);
    p.voxel_size = VoxelSize;
    p.unknown_clip = UnknownClipDistance;
    p.max_surface = MaxSurfaceVoxelDistance;
    p.epsilon = epsilon;
    p.delta_size = deltaSize;
    p.alpha = alpha;
    p.omega_k = omegaKilling;
    p.gamma_k = gammaKilling;
    p.omega_s = omegaLevelSet;
    p.threshold = threshold;
    p.use_data = EnergyTypeUsed[0];
    p.use_levelset = EnergyTypeUsed[1];
    p.use_killing = EnergyTypeUsed[2];
    p.use_trust = UseTrustStrategy;
    return p;
  }
};

// The process-wide configuration the classes read.
Config &config();

// Throws std::runtime_error with kf_last_error() when status != KF_OK.
void check(int status, const char *what);

}  // namespace kf
