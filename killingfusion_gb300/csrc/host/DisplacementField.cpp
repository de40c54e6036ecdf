#include "DisplacementField.h"

#include <cmath>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <vector>

using kf::Vec3d;
using kf::Vec3i;

DisplacementField::DisplacementField(Vec3i gridSize, double voxelSize, kf_precision precision)
    : m_voxelSize(voxelSize), m_gridSize(gridSize), m_precision(precision) {
  int dims[3] = {gridSize(0), gridSize(1), gridSize(2)};
  kf::check(kf_field_create(dims, precision, &m_field), "kf_field_create");
}

DisplacementField::DisplacementField(DisplacementField &&o) noexcept
    : m_field(o.m_field), m_voxelSize(o.m_voxelSize), m_gridSize(o.m_gridSize),
      m_precision(o.m_precision) {
  o.m_field = nullptr;
}

DisplacementField::~DisplacementField() { kf_field_destroy(m_field); }

Vec3d DisplacementField::getDisplacementAt(const Vec3i &i) const {
  int32_t xyz[3] = {i(0), i(1), i(2)};
  double out[3];
  kf::check(kf_field_get_voxels(m_field, xyz, 1, out, nullptr), "kf_field_get_voxels");
  return Vec3d(out[0], out[1], out[2]);
}

Vec3d DisplacementField::getDisplacementAt(int x, int y, int z) const {
  return getDisplacementAt(Vec3i(x, y, z));
}

Vec3d DisplacementField::sample(const Vec3d &p) const {
  double out[3];
  kf::check(kf_field_sample(m_field, p.data(), 1, out, nullptr), "kf_field_sample");
  return Vec3d(out[0], out[1], out[2]);
}

Vec3d DisplacementField::getDisplacementAtf(const Vec3d &p) const { return sample(p); }

Vec3d DisplacementField::getDisplacementAtf(double x, double y, double z) const {
  return sample(Vec3d(x, y, z));
}

void DisplacementField::update(const Vec3i &i, const Vec3d &delta) {
  int32_t xyz[3] = {i(0), i(1), i(2)};
  kf::check(kf_field_add_voxels(m_field, xyz, 1, delta.data(), nullptr), "kf_field_add_voxels");
}

DisplacementField &DisplacementField::operator+(const DisplacementField &other) {
  kf::check(kf_field_add(m_field, other.m_field, nullptr), "kf_field_add");
  return *this;
}

void DisplacementField::initializeAllVoxels(Vec3d d) {
  kf::check(kf_field_fill(m_field, d.data(), nullptr), "kf_field_fill");
}

kf::Mat3d DisplacementField::computeJacobian(double x, double y, double z) const {
  const double h = kf::config().deltaSize;
  double pts[18];
  for (int k = 0; k < 3; ++k) {
    double *a = pts + 6 * k, *b = a + 3;
    a[0] = x + (k == 0) * h; a[1] = y + (k == 1) * h; a[2] = z + (k == 2) * h;
    b[0] = x - (k == 0) * h; b[1] = y - (k == 1) * h; b[2] = z - (k == 2) * h;
  }
  double s[18];
  kf::check(kf_field_sample(m_field, pts, 6, s, nullptr), "kf_field_sample");
  kf::Mat3d J;
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < 3; ++r) J(r, k) = s[6 * k + r] - s[6 * k + 3 + r];
  const double den = 2 * h;
  for (int i = 0; i < 9; ++i) J.m[i] = J.m[i] / den;
  return J;
}

double DisplacementField::computeKillingEnergy(double x, double y, double z) const {
  kf::Mat3d J = computeJacobian(x, y, z);
  for (int i = 0; i < 9; ++i)
    if (!std::isfinite(J.m[i])) {
      std::cout << "Jacobian is infinite\n";
      return 0.0;
    }
  // column-major flattening of J and J^T, as the reference maps them
  double jv[9], jt[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) {
      jv[3 * c + r] = J(r, c);
      jt[3 * c + r] = J(c, r);
    }
  double d1 = jv[0] * jv[0], d2 = jt[0] * jv[0];
  for (int i = 1; i < 9; ++i) {
    d1 = d1 + jv[i] * jv[i];
    d2 = d2 + jt[i] * jv[i];
  }
  return d1 + kf::config().gammaKilling * d2;
}

Vec3d DisplacementField::computeKillingEnergyGradient(const Vec3i &s) const {
  const double h = kf::config().deltaSize;
  for (int k = 0; k < 3; ++k)
    if ((double)s(k) < 2 * h || (double)s(k) >= ((double)m_gridSize(k) - 2 * h)) return Vec3d();
  Vec3d g;
  for (int k = 0; k < 3; ++k)
    g(k) = computeKillingEnergy(s(0) + (k == 0) * h, s(1) + (k == 1) * h, s(2) + (k == 2) * h) -
           computeKillingEnergy(s(0) - (k == 0) * h, s(1) - (k == 1) * h, s(2) - (k == 2) * h);
  const double den = 2 * h;
  return Vec3d(g(0) / den, g(1) / den, g(2) / den);
}

Vec3d DisplacementField::computeKillingEnergyGradient2(const Vec3i &s) const {
  static const int off[19][3] = {{0, 0, 0},  {2, 0, 0},  {-2, 0, 0}, {0, 2, 0},   {0, -2, 0},
                                 {0, 0, 2},  {0, 0, -2}, {1, 0, 1},  {-1, 0, 1},  {0, 1, 1},
                                 {0, -1, 1}, {1, 1, 0},  {-1, 1, 0}, {-1, 0, -1}, {1, 0, -1},
                                 {0, -1, -1}, {0, 1, -1}, {-1, -1, 0}, {1, -1, 0}};
  const kf::Config &c = kf::config();
  const double h = c.deltaSize;
  double pts[57], d[57];
  for (int i = 0; i < 19; ++i)
    for (int k = 0; k < 3; ++k) pts[3 * i + k] = (double)s(k) + h * (double)off[i][k];
  kf::check(kf_field_sample(m_field, pts, 19, d, nullptr), "kf_field_sample");
  auto D = [&](int i, int k) { return d[3 * i + k]; };
  double xx[3], yy[3], zz[3], xy[3], xz[3], yz[3];
  for (int k = 0; k < 3; ++k) {
    xx[k] = (D(1, k) - 2 * D(0, k) + D(2, k));
    yy[k] = (D(3, k) - 2 * D(0, k) + D(4, k));
    zz[k] = (D(5, k) - 2 * D(0, k) + D(6, k));
    xz[k] = (D(7, k) + D(13, k) - D(14, k) - D(8, k));
    yz[k] = (D(9, k) + D(15, k) - D(16, k) - D(10, k));
    xy[k] = (D(11, k) + D(17, k) - D(18, k) - D(12, k));
  }
  double div[3] = {xx[0] + xy[1] + xz[2], xy[0] + yy[1] + yz[2], xz[0] + yz[1] + zz[2]};
  double gk = -2 * c.gammaKilling, kg[3];
  for (int k = 0; k < 3; ++k) kg[k] = -2.0 * (xx[k] + yy[k] + zz[k]) + gk * div[k];
  const double den = (4 * h * h), clamp = 0.1;
  double n = std::sqrt(kg[0] * kg[0] + kg[1] * kg[1] + kg[2] * kg[2]);
  if (n > clamp)
    for (int k = 0; k < 3; ++k) kg[k] = (kg[k] / n) * clamp;
  return Vec3d(kg[0] / den, kg[1] / den, kg[2] / den);
}

void DisplacementField::dumpToBinFile(std::string path) const {
  const int64_t n = (int64_t)m_gridSize(0) * m_gridSize(1) * m_gridSize(2);
  std::vector<double> xyz(3 * n);
  if (m_precision == KF_F64) {
    kf::check(kf_field_download(m_field, xyz.data(), nullptr), "kf_field_download");
  } else {
    std::vector<float> f32(3 * n);
    kf::check(kf_field_download(m_field, f32.data(), nullptr), "kf_field_download");
    for (int64_t i = 0; i < 3 * n; ++i) xyz[i] = (double)f32[i];
  }
  std::cout << "============================================================================\n";
  std::cout << "Saving Displacement voxel grid values at " << path << "\n";
  std::ofstream out(path, std::ios::binary | std::ios::out);
  out.write((const char *)m_gridSize.data(), 3 * sizeof(int));
  out.write((const char *)&m_voxelSize, sizeof(double));
  double mn = 1000, mx = -1000;
  for (int64_t i = 0; i < n; ++i) {
    out.write((const char *)&xyz[3 * i], 3 * sizeof(double));
    double nr = std::sqrt(xyz[3 * i] * xyz[3 * i] + xyz[3 * i + 1] * xyz[3 * i + 1] +
                          xyz[3 * i + 2] * xyz[3 * i + 2]);
    mn = std::min(mn, nr);
    mx = std::max(mx, nr);
  }
  std::cout << "minDisp is " << mn << " and maxDisp is " << mx << std::endl;
  std::cout << "============================================================================\n";
}

DisplacementField DisplacementField::loadFromBinFile(const std::string &path, kf_precision precision) {
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) throw std::runtime_error("cannot open " + path);
  int dims[3];
  double voxel;
  in.read((char *)dims, sizeof(dims));
  in.read((char *)&voxel, sizeof(double));
  const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
  std::vector<double> xyz(3 * n);
  in.read((char *)xyz.data(), 3 * n * sizeof(double));
  if (!in) throw std::runtime_error("short displacement file " + path);
  DisplacementField f(Vec3i(dims[0], dims[1], dims[2]), voxel, precision);
  if (precision == KF_F64) {
    kf::check(kf_field_upload(f.m_field, xyz.data(), nullptr), "kf_field_upload");
  } else {
    std::vector<float> f32(3 * n);
    for (int64_t i = 0; i < 3 * n; ++i) f32[i] = (float)xyz[i];
    kf::check(kf_field_upload(f.m_field, f32.data(), nullptr), "kf_field_upload");
  }
  return f;
}

// DisplacementField::testJacobian (DisplacementField.cpp:142-169)
void DisplacementField::testJacobian() {
  DisplacementField t(Vec3i(8, 8, 8), 0.5);
  for (int x = 0; x < 5; ++x)
    for (int y = 0; y < 5; ++y)
      for (int z = 0; z < 5; ++z) t.update(Vec3i(x, y, z), Vec3d(x + y + z, x + z, y + z));
  const kf::Mat3d J = t.computeJacobian(2, 2, 2);
  std::cout << "numericalJacobian at 2,2,2 is \n";
  for (int r = 0; r < 3; ++r) std::cout << J(r, 0) << " " << J(r, 1) << " " << J(r, 2) << "\n";
  std::cout << "analyticalJacobian at 2,2,2 is \n"
            << "1, 1, 1\n"
            << "1, 0, 1\n"
            << "0, 1, 1" << std::endl;
}

// DisplacementField::testKillingEnergy (DisplacementField.cpp:214-272)
void DisplacementField::testKillingEnergy() {
  const double eps = kf::config().epsilon, gamma = kf::config().gammaKilling;
  DisplacementField t(Vec3i(8, 8, 8), 0.5);
  for (int x = 0; x < 8; ++x)
    for (int y = 0; y < 8; ++y)
      for (int z = 0; z < 8; ++z) t.update(Vec3i(x, y, z), Vec3d(x + y + z, x + z, y));
  for (int x = 0; x < 7; ++x)
    for (int y = 1; y < 7; ++y)
      for (int z = 1; z < 7; ++z) {
        const kf::Mat3d J = t.computeJacobian(x, y, z);
        double avkf = 0.0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) avkf += J(i, j) * J(i, j) + gamma * J(i, j) * J(j, i);
        if (!(std::fabs(avkf - t.computeKillingEnergy(x, y, z)) < eps))
          throw std::runtime_error("Whoops! Check DisplacementField::testKillingEnergy");
      }
  t.initializeAllVoxels(Vec3d(0, 0, 0));
  for (int x = 0; x < 8; ++x)
    for (int y = 0; y < 8; ++y)
      for (int z = 0; z < 8; ++z) t.update(Vec3i(x, y, z), Vec3d((double)x * x, 0, 0));
  int mismatches = 0, checked = 0;
  for (int x = 1; x < 7; ++x)
    for (int y = 1; y < 7; ++y)
      for (int z = 1; z < 7; ++z) {
        const Vec3d g1 = t.computeKillingEnergyGradient(Vec3i(x, y, z));
        const Vec3d g2 = t.computeKillingEnergyGradient2(Vec3i(x, y, z));
        ++checked;
        if (!(std::fabs(g1(0) - g2(0)) < eps && std::fabs(g1(1) - g2(1)) < eps && std::fabs(g1(2) - g2(2)) < eps))
          ++mismatches;
      }
  std::cout << "Killing energy gradient forms differ at " << mismatches << " of " << checked
            << " voxels (finite differences against the clamped form, as in the reference)" << std::endl;
}
