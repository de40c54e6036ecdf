#include "KillingFusion.h"

#include <chrono>
#include <cstdio>
#include <iostream>
#include <stdexcept>

using kf::Mat3d;
using kf::Vec3d;

namespace {
struct Timer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  void reset() { t0 = std::chrono::steady_clock::now(); }
  double elapsed() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

// The 3x3 inverse by cofactors: inv(i,j) = cof(j,i) / det, det expanded
// along column 0.
Mat3d inverse3(const Mat3d &m) {
  auto cof = [&](int i, int j) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    return m(i1, j1) * m(i2, j2) - m(i1, j2) * m(i2, j1);
  };
  const double det = cof(0, 0) * m(0, 0) + cof(1, 0) * m(1, 0) + cof(2, 0) * m(2, 0);
  const double inv_det = 1.0 / det;
  Mat3d r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r(i, j) = cof(j, i) * inv_det;
  return r;
}
}  // namespace

KillingFusion::KillingFusion(DatasetReader reader) : m_datasetReader(std::move(reader)) {
  std::pair<Vec3d, Vec3d> b =
      computeBounds(m_datasetReader.getDepthIntrinsicMatrix(), m_datasetReader.getDepthWidth(),
                    m_datasetReader.getDepthHeight(), m_datasetReader.getMinimumDepthThreshold(),
                    m_datasetReader.getMaximumDepthThreshold());
  const kf::Config &c = kf::config();
  m_canonicalSdf = new SDF(c.VoxelSize, b.first, b.second, c.UnknownClipDistance);
  std::cout << m_canonicalSdf->getGridSize() << std::endl;
  m_startFrame = 1;
  m_endFrame = 50;
  m_stride = 1;
  m_currFrameIndex = m_startFrame;
}

KillingFusion::~KillingFusion() {
  delete m_canonicalSdf;
  delete m_prev2CanDisplacementField;
}

void KillingFusion::saveState(const std::string &path) const {
  kf::check(kf_state_save(path.c_str(), m_canonicalSdf->handle(),
                          m_prev2CanDisplacementField ? m_prev2CanDisplacementField->handle() : nullptr,
                          m_currFrameIndex, nullptr),
            "kf_state_save");
}

void KillingFusion::loadState(const std::string &path) {
  int dims[3];
  int prec = -1;
  int32_t frame = 0;
  kf::check(kf_state_info(path.c_str(), dims, nullptr, nullptr, nullptr, &frame, &prec), "kf_state_info");
  const kf::Vec3i n = m_canonicalSdf->getGridSize();
  if (dims[0] != n(0) || dims[1] != n(1) || dims[2] != n(2))
    throw std::runtime_error("KillingFusion::loadState: the state file's grid differs from this sequence's");
  DisplacementField *psi = nullptr;
  if (prec >= 0) psi = new DisplacementField(n, kf::config().VoxelSize, (kf_precision)prec);
  int rc = kf_state_load(path.c_str(), m_canonicalSdf->handle(), psi ? psi->handle() : nullptr, &frame, nullptr);
  if (rc) {
    delete psi;
    kf::check(rc, "kf_state_load");
  }
  delete m_prev2CanDisplacementField;
  m_prev2CanDisplacementField = psi;
  m_currFrameIndex = frame;
}

void KillingFusion::setFrameRange(int start, int end, int stride) {
  if (stride < 1 || end < start) throw std::invalid_argument("KillingFusion::setFrameRange");
  m_startFrame = start;
  m_endFrame = end;
  m_stride = stride;
  m_currFrameIndex = start;
}

// KillingFusion::computeBounds (KillingFusion.cpp:478-519): the eight
// frustum corners K^-1 (u, v, 1) scaled by the near/far depth, z replaced by
// the depth itself.
std::pair<Vec3d, Vec3d> KillingFusion::computeBounds(const Mat3d &K, int w, int h, double minDepth,
                                                     double maxDepth) {
  const double cu[8] = {0, 0, (double)(w - 1), (double)(w - 1), 0, 0, (double)(w - 1), (double)(w - 1)};
  const double cv[8] = {0, (double)(h - 1), (double)(h - 1), 0, 0, (double)(h - 1), (double)(h - 1), 0};
  const Mat3d Ki = inverse3(K);
  Vec3d lo, hi;
  for (int j = 0; j < 8; ++j) {
    const double d = j < 4 ? minDepth : maxDepth;
    Vec3d p;
    for (int r = 0; r < 2; ++r) p(r) = (Ki(r, 0) * cu[j] + Ki(r, 1) * cv[j] + Ki(r, 2) * 1.0) * d;
    p(2) = d;
    for (int k = 0; k < 3; ++k) {
      if (j == 0 || p(k) < lo(k)) lo(k) = p(k);
      if (j == 0 || p(k) > hi(k)) hi(k) = p(k);
    }
  }
  return std::make_pair(lo, hi);
}

// KillingFusion::computeSDF (KillingFusion.cpp:211-232): a frustum-bounded
// SDF with the frame integrated at pose = identity.
SDF *KillingFusion::computeSDF(int frameIndex) {
  const kf::Config &c = kf::config();
  const double minD = m_datasetReader.getMinimumDepthThreshold();
  const double maxD = m_datasetReader.getMaximumDepthThreshold();
  std::pair<Vec3d, Vec3d> b = computeBounds(m_datasetReader.getDepthIntrinsicMatrix(),
                                            m_datasetReader.getDepthWidth(),
                                            m_datasetReader.getDepthHeight(), minD, maxD);
  SDF *sdf = new SDF(c.VoxelSize, b.first, b.second, c.UnknownClipDistance);
  std::vector<kf::DepthImage> images = m_datasetReader.getImages(frameIndex);
  sdf->integrateDepthFrame(images.at(1), kf::Mat4d::Identity(), m_datasetReader.getDepthIntrinsicMatrix(),
                           minD, maxD);
  return sdf;
}

// A zero psi; float64 when the exact solver is configured (it replays the
// reference's float64 arithmetic).
DisplacementField *KillingFusion::createZeroDisplacementField(const SDF &sdf) {
  const kf::Config &c = kf::config();
  return new DisplacementField(sdf.getGridSize(), c.VoxelSize,
                               c.solver == KF_SOLVER_EXACT ? KF_F64 : KF_F32);
}

// KillingFusion::computeDisplacementField, Jacobi schedule
// (KillingFusion.cpp:248-352): KILLING_MAX_ITERATIONS sweeps in one
// kf_psi_solve.  Divergence throws -1 like the reference (:331).
void KillingFusion::computeDisplacementField(const SDF *src, const SDF *dest, DisplacementField *psi) {
  const kf::Config &c = kf::config();
  kf_params p = c.params();
  int rc = kf_psi_solve(src->handle(), dest->handle(), psi->handle(), &p, c.KILLING_MAX_ITERATIONS,
                        c.solver, &m_lastStats, nullptr);
  if (rc == KF_ERR_DIVERGED) {
    std::cout << "Error: deformation field has diverged: " << kf_last_error() << std::endl;
    throw -1;
  }
  kf::check(rc, "kf_psi_solve");
}

std::vector<SimpleMesh *> KillingFusion::processNextFrame() {
  const kf::Config &c = kf::config();
  SimpleMesh *live = nullptr, *registered = nullptr;
  if (m_currFrameIndex == m_startFrame) {
    delete m_canonicalSdf;
    m_canonicalSdf = nullptr;
    m_canonicalSdf = computeSDF(m_startFrame);
    delete m_prev2CanDisplacementField;
    m_prev2CanDisplacementField = nullptr;
    m_prev2CanDisplacementField = createZeroDisplacementField(*m_canonicalSdf);
    live = m_canonicalSdf->getMesh();
    registered = m_canonicalSdf->getMesh(*m_prev2CanDisplacementField);
    m_currFrameIndex += m_stride;
  } else if (m_currFrameIndex < m_endFrame) {
    Timer total, timer;
    std::cout << "Frame  Compute SDF    KillingOptimize    Fuse SDF    Total Time\n";
    SDF *curr = computeSDF(m_currFrameIndex);
    const double sdfTime = timer.elapsed();
    DisplacementField *psi;
    if (c.UseZeroDisplacementFieldForNextFrame) {
      delete m_prev2CanDisplacementField;
      m_prev2CanDisplacementField = nullptr;
      psi = createZeroDisplacementField(*curr);
    } else {
      psi = m_prev2CanDisplacementField;
    }
    m_prev2CanDisplacementField = psi;
    timer.reset();
    if (c.EnergyTypeUsed[0] || c.EnergyTypeUsed[1] || c.EnergyTypeUsed[2]) {
      try {
        computeDisplacementField(curr, m_canonicalSdf, psi);
      } catch (...) {
        delete curr;
        throw;
      }
    }
    const double killingTime = timer.elapsed();
    timer.reset();
    // SDF::update(psi) then canonical->fuse(curr) (KillingFusion.cpp:158-159)
    // in one pass; curr is left warped for the registered mesh.
    live = curr->getMesh();
    kf_params p = c.params();
    int rc = kf_warp_fuse(m_canonicalSdf->handle(), curr->handle(), psi->handle(), &p, nullptr);
    if (rc == KF_OK) registered = curr->getMesh();
    const double fuseTime = timer.elapsed();
    delete curr;
    kf::check(rc, "kf_warp_fuse");
    std::printf("%03d\t%0.6fs\t%0.6fs\t%0.6fs\t%0.6fs\n", m_currFrameIndex, sdfTime, killingTime, fuseTime,
                total.elapsed());
    m_currFrameIndex += m_stride;
  }
  std::vector<SimpleMesh *> meshes;
  meshes.push_back(live);
  meshes.push_back(registered);
  meshes.push_back(m_canonicalSdf->getMesh());
  return meshes;
}

// KillingFusion::process (KillingFusion.cpp:41-107): frames 4..99 (clamped
// to the dataset), psi carried over, fuse along psi.
void KillingFusion::process() {
  const int startFrame = 4;
  const int endFrame = std::min(100, m_datasetReader.getNumImageFiles());
  if (endFrame <= startFrame) throw std::runtime_error("KillingFusion::process: dataset too short");
  SDF *prev = computeSDF(startFrame);
  DisplacementField *psi = createZeroDisplacementField(*prev);
  m_canonicalSdf->fuse(prev);
  const char *names[4] = {"InputFrameSDF", "RegisteredFrameSDF", "CanonicalSDF", "LiveCanonicalSdf"};
  for (int k = 0; k < 4; ++k) prev->save_mesh(names[k], startFrame);
  Timer total, timer;
  std::cout << "Frame  Compute SDF    KillingOptimize    Fuse SDF\n";
  for (int i = startFrame + 1; i < endFrame; ++i) {
    timer.reset();
    SDF *curr = computeSDF(i);
    const double sdfTime = timer.elapsed();
    curr->save_mesh(names[0], i);
    timer.reset();
    try {
      computeDisplacementField(curr, m_canonicalSdf, psi);
    } catch (...) {
      delete curr;
      delete prev;
      delete psi;
      throw;
    }
    const double killingTime = timer.elapsed();
    curr->save_mesh(names[1], i, *psi);
    timer.reset();
    m_canonicalSdf->fuse(curr, psi);
    const double fuseTime = timer.elapsed();
    m_canonicalSdf->save_mesh(names[2], i);
    delete prev;
    prev = curr;
    std::printf("%03d\t%0.6fs\t%0.6fs\t%0.6fs\n", i, sdfTime, killingTime, fuseTime);
  }
  std::cout << "Total time spent " << total.elapsed() << std::endl;
  delete prev;
  delete psi;
  m_canonicalSdf->dumpToBinFile(SDF::outputDir() + "FinalCanonicalModel.bin", kf::config().UnknownClipDistance,
                                1.0);
}

void KillingFusion::processTest(int testType) {
  const kf::Config &c = kf::config();
  std::vector<SDF> s = SDF::getDataEnergyTestSample(c.VoxelSize, c.UnknownClipDistance);
  DisplacementField *psi = createZeroDisplacementField(s[1]);
  const std::string dir = SDF::outputDir();
  const double trunc = c.UnknownClipDistance;
  try {
    if (testType == 1) {
      s[0].dumpToBinFile(dir + "testType-1-outputSphere0.bin", trunc, 1.0);
      s[1].dumpToBinFile(dir + "testType-1-outputSphere1.bin", trunc, 1.0);
      s[0].fuse(&s[0]);
      s[0].dumpToBinFile(dir + "testType-1-outputSphere0MergedTo0.bin", trunc, 1.0);
    } else if (testType == 2) {
      s[0].dumpToBinFile(dir + "testType-1-outputSphere0.bin", trunc, 1.0);
      s[1].dumpToBinFile(dir + "testType-1-outputSphere1.bin", trunc, 1.0);
      s[0].fuse(&s[1]);
      s[0].dumpToBinFile(dir + "testType-1-outputSphere1MergedTo0.bin", trunc, 1.0);
    } else {
      computeDisplacementField(&s[1], &s[0], psi);
      s[0].fuse(&s[1], psi);
      SDF srcCopy(s[1]);
      srcCopy.fuse(&s[1], psi);
      srcCopy.dumpToBinFile(dir + "testType-2-outputSphere1Deformed.bin", trunc, 1.0);
      s[0].dumpToBinFile(dir + "testType-2-outputSphere1MergedTo0UsingKilling.bin", trunc, 1.0);
    }
  } catch (...) {
    delete psi;
    throw;
  }
  delete psi;
}
