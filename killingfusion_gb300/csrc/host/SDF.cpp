#include "SDF.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

using kf::Mat3d;
using kf::Vec3d;
using kf::Vec3i;

namespace kf {
Config &config() {
  static Config c;
  return c;
}

void check(int status, const char *what) {
  if (status != KF_OK) throw std::runtime_error(std::string(what) + ": " + kf_last_error());
}
}  // namespace kf

std::string &SDF::outputDir() {
  static std::string dir = "./";
  return dir;
}

static kf_params params_now() { return kf::config().params(); }

void SDF::allocate() {
  int dims[3] = {m_gridSize(0), m_gridSize(1), m_gridSize(2)};
  double mn[3] = {m_min3dLoc(0), m_min3dLoc(1), m_min3dLoc(2)};
  kf_params p = params_now();
  kf::check(kf_grid_create(dims, m_voxelSize, mn, m_unknownClipDistance, &p, &m_grid), "kf_grid_create");
}

SDF::SDF(double voxelSize, Vec3d min3dLoc, Vec3d max3dLoc, double unknownClipDistance)
    : m_min3dLoc(min3dLoc), m_max3dLoc(max3dLoc), m_voxelSize(voxelSize),
      m_unknownClipDistance(unknownClipDistance) {
  // SDF::computeVoxelGridSize (SDF.cpp:117-124): the cast may drop one cell
  Vec3d bound = max3dLoc - min3dLoc;
  for (int k = 0; k < 3; ++k) m_gridSize(k) = (int)(bound(k) / voxelSize) + 1;
  allocate();
}

SDF::SDF(const SDF &copy)
    : m_gridSize(copy.m_gridSize), m_min3dLoc(copy.m_min3dLoc), m_max3dLoc(copy.m_max3dLoc),
      m_voxelSize(copy.m_voxelSize), m_unknownClipDistance(copy.m_unknownClipDistance) {
  allocate();
}

SDF::SDF(SDF &&o) noexcept
    : m_grid(o.m_grid), m_gridSize(o.m_gridSize), m_min3dLoc(o.m_min3dLoc), m_max3dLoc(o.m_max3dLoc),
      m_voxelSize(o.m_voxelSize), m_unknownClipDistance(o.m_unknownClipDistance) {
  o.m_grid = nullptr;
}

SDF::~SDF() { kf_grid_destroy(m_grid); }

SDF::SDF(kf_grid grid, double unknownClipDistance) : m_grid(grid), m_unknownClipDistance(unknownClipDistance) {
  int dims[3];
  double mn[3];
  kf::check(kf_grid_info(grid, dims, &m_voxelSize, mn, nullptr), "kf_grid_info");
  for (int k = 0; k < 3; ++k) {
    m_gridSize(k) = dims[k];
    m_min3dLoc(k) = mn[k];
    m_max3dLoc(k) = mn[k] + ((double)dims[k] - 0.5) * m_voxelSize;
  }
}

SDF *SDF::loadFromBinFile(const std::string &path, double unknownClipDistance) {
  kf_params p = params_now();
  kf_grid g = nullptr;
  kf::check(kf_grid_load_ref_bin(path.c_str(), &p, unknownClipDistance, &g, nullptr, nullptr),
            "kf_grid_load_ref_bin");
  return new SDF(g, unknownClipDistance);
}

std::vector<SDF> SDF::getDataEnergyTestSample(double voxelSize, double unknownClipDistance) {
  Vec3d mn(0, 0, 0), mx(voxelSize * 9, voxelSize * 9, voxelSize * 9);
  SDF can(voxelSize, mn, mx, unknownClipDistance), next(voxelSize, mn, mx, unknownClipDistance);
  const Vec3i n = can.m_gridSize;
  const Vec3d c0((double)(n(0) / 2) + 0.5, (double)(n(1) / 2) + 0.5, (double)(n(2) / 2) + -0.5);
  const Vec3d c1((double)(n(0) / 2) + 0.5, (double)(n(1) / 2) + 0.5, (double)(n(2) / 2) + 0.5);
  std::cout << "Center for First Sphere is " << c0 << std::endl;
  std::cout << "Center for Second Sphere is " << c1 << std::endl;
  const double radius = 3 * can.m_voxelSize;
  const int64_t N = (int64_t)n(0) * n(1) * n(2);
  std::vector<float> p0(N), p1(N);
  std::vector<int32_t> w0(N), w1(N);
  kf::check(kf_grid_download(can.m_grid, p0.data(), nullptr, nullptr), "kf_grid_download");
  p1 = p0;
  for (int z = 0; z < n(2); ++z)
    for (int y = 0; y < n(1); ++y)
      for (int x = 0; x < n(0); ++x) {
        Vec3d loc(x + 0.5, y + 0.5, z + 0.5);
        int64_t i = (int64_t)z * n(0) * n(1) + (int64_t)y * n(0) + x;
        double d0 = (c0 - loc).norm() * voxelSize - radius;
        double d1 = (c1 - loc).norm() * voxelSize - radius;
        if (d0 >= -unknownClipDistance) {
          p0[i] = (float)d0;
          w0[i] = 1;
        } else {
          w0[i] = 0;
        }
        if (d1 >= -unknownClipDistance) {
          p1[i] = (float)d1;
          w1[i] = 1;
        } else {
          w1[i] = 0;
        }
      }
  kf::check(kf_grid_upload(can.m_grid, p0.data(), w0.data(), nullptr), "kf_grid_upload");
  kf::check(kf_grid_upload(next.m_grid, p1.data(), w1.data(), nullptr), "kf_grid_upload");
  std::vector<SDF> out;
  out.push_back(std::move(can));
  out.push_back(std::move(next));
  return out;
}

void SDF::integrateDepthFrame(const kf::DepthImage &depth, const kf::Mat4d &c2w, const Mat3d &K,
                              double minDepth, double maxDepth) {
  if (depth.is_raw())
    kf::check(kf_integrate_depth_u16(m_grid, depth.raw.data(), depth.cols, depth.rows, depth.scale, c2w.data(),
                                     K.data(), minDepth, maxDepth, nullptr),
              "kf_integrate_depth_u16");
  else
    kf::check(kf_integrate_depth(m_grid, depth.ptr(), depth.cols, depth.rows, c2w.data(), K.data(), minDepth,
                                 maxDepth, nullptr),
              "kf_integrate_depth");
}

bool SDF::indexInGridBounds(int x, int y, int z) const {
  return x >= 0 && x < m_gridSize(0) && y >= 0 && y < m_gridSize(1) && z >= 0 && z < m_gridSize(2);
}

double SDF::getDistanceAtIndex(const Vec3i &i) const {
  int32_t xyz[3] = {i(0), i(1), i(2)};
  double phi;
  kf_params p = params_now();
  kf::check(kf_grid_get_voxels(m_grid, &p, xyz, 1, &phi, nullptr, nullptr), "kf_grid_get_voxels");
  return phi;
}

long SDF::getWeightAtIndex(const Vec3i &i) const {
  int32_t xyz[3] = {i(0), i(1), i(2)};
  int64_t w;
  kf_params p = params_now();
  kf::check(kf_grid_get_voxels(m_grid, &p, xyz, 1, nullptr, &w, nullptr), "kf_grid_get_voxels");
  return (long)w;
}

std::vector<double> SDF::sampleDistances(const std::vector<double> &pts) const {
  std::vector<double> out(pts.size() / 3);
  kf_params p = params_now();
  kf::check(kf_grid_sample(m_grid, &p, pts.data(), (int)out.size(), out.data(), nullptr, nullptr),
            "kf_grid_sample");
  return out;
}

// (p + psi~(p)) + 0.5 for each point: the location SDF::getDistancef samples
// (SDF.cpp:577-582).
std::vector<double> SDF::warpedPoints(const std::vector<double> &pts, const DisplacementField *psi) const {
  std::vector<double> d(pts.size()), out(pts.size());
  kf::check(kf_field_sample(psi->handle(), pts.data(), (int)(pts.size() / 3), d.data(), nullptr),
            "kf_field_sample");
  for (size_t i = 0; i < pts.size(); ++i) out[i] = (pts[i] + d[i]) + 0.5;
  return out;
}

double SDF::getDistance(const Vec3d &p) const {
  return sampleDistances({p(0), p(1), p(2)})[0];
}

double SDF::getDistance(const Vec3i &i, const DisplacementField *psi) const {
  Vec3d d = psi->getDisplacementAt(i);
  return getDistance(Vec3d(((double)i(0) + d(0)) + 0.5, ((double)i(1) + d(1)) + 0.5,
                           ((double)i(2) + d(2)) + 0.5));
}

double SDF::getDistancef(const Vec3d &p, const DisplacementField *psi) const {
  return sampleDistances(warpedPoints({p(0), p(1), p(2)}, psi))[0];
}

double SDF::getWeight(const Vec3d &p) const {
  double w;
  kf_params pr = params_now();
  kf::check(kf_grid_sample(m_grid, &pr, p.data(), 1, nullptr, &w, nullptr), "kf_grid_sample");
  return w;
}

double SDF::getWeight(const Vec3i &i, const DisplacementField *psi) const {
  Vec3d d = psi->getDisplacementAt(i);
  return getWeight(Vec3d(((double)i(0) + d(0)) + 0.5, ((double)i(1) + d(1)) + 0.5,
                         ((double)i(2) + d(2)) + 0.5));
}

// SDF::computeDistanceGradient(gridLocation) (SDF.cpp:657-679)
Vec3d SDF::computeDistanceGradient(const Vec3d &p) const {
  for (int k = 0; k < 3; ++k)
    if (p(k) < 0.0 || p(k) >= (double)m_gridSize(k)) return Vec3d();
  std::vector<double> pts;
  for (int k = 0; k < 3; ++k)
    for (int s = 0; s < 2; ++s)
      for (int j = 0; j < 3; ++j) pts.push_back(p(j) + (s ? -1.0 : 1.0) * (j == k ? 1.0 : 0.0));
  std::vector<double> f = sampleDistances(pts);
  return Vec3d((f[0] - f[1]) / 2, (f[2] - f[3]) / 2, (f[4] - f[5]) / 2);
}

// SDF::computeDistanceGradient(spatialIndex, psi) (SDF.cpp:726-744)
Vec3d SDF::computeDistanceGradient(const Vec3i &i, const DisplacementField *psi) const {
  const double h = kf::config().deltaSize;
  const Vec3d g((double)i(0) + 0.5, (double)i(1) + 0.5, (double)i(2) + 0.5);
  std::vector<double> pts;
  for (int k = 0; k < 3; ++k)
    for (int s = 0; s < 2; ++s)
      for (int j = 0; j < 3; ++j) {
        double d = h * (double)(j == k);
        pts.push_back(s ? g(j) - d : g(j) + d);
      }
  std::vector<double> f = sampleDistances(warpedPoints(pts, psi));
  const double den = (2 * h);
  return Vec3d((f[0] - f[1]) / den, (f[2] - f[3]) / den, (f[4] - f[5]) / den);
}

// The self-tests' grid: voxel 0.5 over [0, 8]^3 (17^3 voxels) holding
// f = x + y - z in the SDF values (weights too when `weights`).
static SDF linear_test_sdf(bool weights) {
  SDF t(0.5, Vec3d(0, 0, 0), Vec3d(8, 8, 8), kf::config().UnknownClipDistance);
  const Vec3i n = t.getGridSize();
  std::vector<float> phi((size_t)n(0) * n(1) * n(2));
  std::vector<int32_t> w(phi.size(), 0);
  for (int z = 0; z < n(2); ++z)
    for (int y = 0; y < n(1); ++y)
      for (int x = 0; x < n(0); ++x) {
        const size_t i = ((size_t)z * n(1) + y) * n(0) + x;
        phi[i] = (float)(x + y - z);
        if (weights) w[i] = x + y - z;
      }
  kf::check(kf_grid_upload(t.handle(), phi.data(), w.data(), nullptr), "kf_grid_upload");
  return t;
}

static void self_check(bool ok, const char *what) {
  if (!ok) throw std::runtime_error(what);
}

void SDF::testGetDistance() {
  const SDF t = linear_test_sdf(false);
  const Vec3i n = t.getGridSize();
  const double eps = kf::config().epsilon;
  std::vector<double> pts, want;
  for (int z = 2; z < n(2) - 2; ++z)
    for (int y = 2; y < n(1) - 2; ++y)
      for (int x = 2; x < n(0) - 2; ++x)
        for (int i = 0; i < 10; ++i) {
          const double delta = i / 10.0;
          want.push_back(x + delta + y - delta - z + delta);
          pts.insert(pts.end(), {x + 0.5 + delta, y + 0.5 - delta, z + 0.5 - delta});
        }
  const std::vector<double> got = t.sampleDistances(pts);
  for (size_t k = 0; k < want.size(); ++k)
    self_check(std::fabs(want[k] - got[k]) < eps, "Whoops, check testGetDistance");
}

void SDF::testGetWeight() {
  const SDF t = linear_test_sdf(true);
  const Vec3i n = t.getGridSize();
  const double eps = kf::config().epsilon;
  std::vector<double> pts, want;
  for (int z = 2; z < n(2) - 2; ++z)
    for (int y = 2; y < n(1) - 2; ++y)
      for (int x = 2; x < n(0) - 2; ++x)
        for (int i = 0; i < 10; ++i) {
          const double delta = i / 10.0f;  // float division, as the reference writes it
          want.push_back(x + delta + y - delta - z + delta);
          pts.insert(pts.end(), {x + 0.5 + delta, y + 0.5 - delta, z + 0.5 - delta});
        }
  std::vector<double> got(want.size());
  kf_params pr = params_now();
  kf::check(kf_grid_sample(t.handle(), &pr, pts.data(), (int)want.size(), nullptr, got.data(), nullptr),
            "kf_grid_sample");
  for (size_t k = 0; k < want.size(); ++k)
    self_check(std::fabs(want[k] - got[k]) < eps, "Whoops, check testGetWeights");
}

void SDF::testComputeDistanceGradient() {
  const SDF t = linear_test_sdf(false);
  const Vec3i n = t.getGridSize();
  const double eps = kf::config().epsilon;
  for (int z = 2; z < n(2) - 2; ++z)
    for (int y = 2; y < n(1) - 2; ++y)
      for (int x = 2; x < n(0) - 2; ++x)
        for (int i = 0; i < 10; ++i) {
          const double delta = i / 10.0f;
          const Vec3d g = t.computeDistanceGradient(Vec3d(x + 0.5 + delta, y + 0.5 - delta, z + 0.5 - delta));
          self_check(std::fabs(g(0) - 1) < eps && std::fabs(g(1) - 1) < eps && std::fabs(g(2) + 1) < eps,
                     "Whoops, check SDF::testComputeDistanceGradient");
        }
}

void SDF::testComputeDistanceHessian() {
  const SDF t = linear_test_sdf(false);
  const Vec3i n = t.getGridSize();
  const double voxel = 0.5;
  for (int z = 2; z < n(2) - 2; ++z)
    for (int y = 2; y < n(1) - 2; ++y)
      for (int x = 2; x < n(0) - 2; ++x)
        for (int i = 0; i < 10; ++i) {
          const double delta = i * voxel / 10.0f;
          const Mat3d H = t.computeDistanceHessian(Vec3d(x + 0.5 + delta, y + 0.5 - delta, z + 0.5 - delta));
          self_check(H.isZero(1e-4), "Whoops, check SDF::testComputeDistanceGradient");
        }
}

static const int kHess[19][3] = {{0, 0, 0},  {2, 0, 0},  {-2, 0, 0}, {0, 2, 0},   {0, -2, 0},
                                 {0, 0, 2},  {0, 0, -2}, {1, 0, 1},  {-1, 0, 1},  {0, 1, 1},
                                 {0, -1, 1}, {1, 1, 0},  {-1, 1, 0}, {-1, 0, -1}, {1, 0, -1},
                                 {0, -1, -1}, {0, 1, -1}, {-1, -1, 0}, {1, -1, 0}};

static Mat3d assemble_hessian(const std::vector<double> &f, double h) {
  Mat3d H;
  double fxx = (f[1] - 2 * f[0] + f[2]);
  double fyy = (f[3] - 2 * f[0] + f[4]);
  double fzz = (f[5] - 2 * f[0] + f[6]);
  double fxz = (f[7] + f[13] - f[14] - f[8]);
  double fyz = (f[9] + f[15] - f[16] - f[10]);
  double fxy = (f[11] + f[17] - f[18] - f[12]);
  H(0, 0) = fxx; H(1, 1) = fyy; H(2, 2) = fzz;
  H(0, 1) = H(1, 0) = fxy;
  H(0, 2) = H(2, 0) = fxz;
  H(1, 2) = H(2, 1) = fyz;
  const double den = (4 * h * h);
  for (int k = 0; k < 9; ++k) H.m[k] = H.m[k] / den;
  return H;
}

// SDF::computeDistanceHessian(gridLocation) (SDF.cpp:746-795)
Mat3d SDF::computeDistanceHessian(const Vec3d &p) const {
  for (int k = 0; k < 3; ++k) {
    double t = p(k) - 0.5;
    if (t < 0.0 || t >= (double)m_gridSize(k)) return Mat3d::Zero();
  }
  const double h = kf::config().deltaSize;
  std::vector<double> pts;
  for (int s = 0; s < 19; ++s)
    for (int k = 0; k < 3; ++k) pts.push_back(p(k) + h * (double)kHess[s][k]);
  return assemble_hessian(sampleDistances(pts), h);
}

// SDF::computeDistanceHessian(spatialIndex, psi) (SDF.cpp:842-886)
Mat3d SDF::computeDistanceHessian(const Vec3i &i, const DisplacementField *psi) const {
  const double h = kf::config().deltaSize;
  std::vector<double> pts;
  for (int s = 0; s < 19; ++s)
    for (int k = 0; k < 3; ++k) pts.push_back(((double)i(k) + 0.5) + h * (double)kHess[s][k]);
  return assemble_hessian(sampleDistances(warpedPoints(pts, psi)), h);
}

void SDF::fuse(const SDF *other) { kf::check(kf_fuse(m_grid, other->m_grid, nullptr), "kf_fuse"); }

void SDF::fuse(const SDF *other, const DisplacementField *psi) {
  kf_params p = params_now();
  kf::check(kf_fuse_warped(m_grid, other->m_grid, psi->handle(), &p, nullptr), "kf_fuse_warped");
}

void SDF::update(const DisplacementField *psi) {
  kf_params p = params_now();
  kf::check(kf_warp(m_grid, psi->handle(), &p, nullptr), "kf_warp");
}

SimpleMesh *SDF::getMesh() const {
  kf_params p = params_now();
  int64_t n = 0;
  kf::check(kf_mesh_host(m_grid, &p, nullptr, 0, &n, nullptr), "kf_mesh_host");
  std::vector<float> v((size_t)std::max<int64_t>(n, 1) * 9);
  if (n > 0) kf::check(kf_mesh_host(m_grid, &p, v.data(), n, &n, nullptr), "kf_mesh_host");
  SimpleMesh *mesh = new SimpleMesh();
  mesh->AppendSoup(v.data(), n);
  return mesh;
}

SimpleMesh *SDF::getMesh(const DisplacementField &psi) const {
  SDF deformed(m_voxelSize, m_min3dLoc, m_max3dLoc, m_unknownClipDistance);
  deformed.fuse(this, &psi);
  return deformed.getMesh();
}

static std::string mesh_name(const std::string &prefix, int counter) {
  std::ostringstream s;
  s << SDF::outputDir() << prefix << std::setw(3) << std::setfill('0') << counter << ".off";
  return s.str();
}

void SDF::save_mesh(std::string prefix, int counter) const {
  std::string path = mesh_name(prefix, counter);
  SimpleMesh *mesh = getMesh();
  if (!mesh->WriteMesh(path)) std::cout << "ERROR: unable to write output file at" << path << "!" << std::endl;
  delete mesh;
}

void SDF::save_mesh(std::string prefix, int counter, const DisplacementField &psi) const {
  SDF deformed(m_voxelSize, m_min3dLoc, m_max3dLoc, m_unknownClipDistance);
  deformed.fuse(this, &psi);
  deformed.save_mesh(prefix, counter);
}

void SDF::dumpToBinFile(std::string path, double trunc, double) const {
  const int64_t N = (int64_t)m_gridSize(0) * m_gridSize(1) * m_gridSize(2);
  std::vector<float> phi(N);
  kf::check(kf_grid_download(m_grid, phi.data(), nullptr, nullptr), "kf_grid_download");
  std::cout << "============================================================================\n";
  std::cout << "Saving TSDF voxel grid values at " << path << "\n";
  std::ofstream out(path, std::ios::binary | std::ios::out);
  out.write((const char *)m_gridSize.data(), 3 * sizeof(int));
  out.write((const char *)m_min3dLoc.data(), 3 * sizeof(double));
  out.write((const char *)&m_voxelSize, sizeof(double));
  out.write((const char *)&trunc, sizeof(double));
  std::vector<double> d(phi.begin(), phi.end());
  out.write((const char *)d.data(), N * sizeof(double));
  out.close();
  double mn = d[0], mx = d[0];
  for (int64_t i = 0; i < N; ++i) {
    if (d[i] < mn)
      mn = d[i];
    else if (d[i] > mx)
      mx = d[i];
  }
  std::cout << "Minimum SDF value is " << mn << " and max value is " << mx << "\n";
  std::cout << "TSDF voxel grid values saved at " << path << "\n";
  std::cout << "============================================================================\n";
}
