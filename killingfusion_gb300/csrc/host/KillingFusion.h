// The frame driver with the reference's interface (KillingFusion.h:13-100).
// SDFs and psi live on the device; computeDisplacementField is one
// kf_psi_solve call (the reference's Jacobi schedule, KillingFusion.cpp:248-352)
// and warp + fuse is one kf_warp_fuse pass.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "DatasetReader.h"
#include "DisplacementField.h"
#include "SDF.h"
#include "SimpleMesh.h"

class KillingFusion {
 public:
  KillingFusion() = delete;
  explicit KillingFusion(DatasetReader datasetReader);
  ~KillingFusion();
  KillingFusion(const KillingFusion &) = delete;
  KillingFusion &operator=(const KillingFusion &) = delete;

  // Fuses every frame, carrying psi from frame to frame and saving the four
  // mesh series (KillingFusion.cpp:41-107).
  void process();

  // Fuses one frame into the canonical SDF and returns {live, registered,
  // canonical} meshes (owned by the caller; the first two are NULL once the
  // end frame is reached) (KillingFusion.cpp:109-175).
  std::vector<SimpleMesh *> processNextFrame();

  // The two-sphere tests (KillingFusion.cpp:177-209): 1 fuses sphere 0 into
  // itself, 2 fuses sphere 1 into sphere 0, 3 registers sphere 1 onto sphere 0
  // and fuses it along psi.
  void processTest(int testType);

  int getCurrentFrameIndex() const { return m_currFrameIndex; }
  int getEndFrameIndex() const { return m_endFrame; }
  DisplacementField *getCurrentFrameDisplacementField() { return m_prev2CanDisplacementField; }

  // Frame range of processNextFrame; the reference fixes 1, 50, 1
  // (KillingFusion.cpp:25-28).
  void setFrameRange(int start, int end, int stride = 1);
  const SDF *getCanonicalSdf() const { return m_canonicalSdf; }
  // Statistics of the last computeDisplacementField.
  const kf_solve_stats &lastSolveStats() const { return m_lastStats; }

  // Checkpoint (no counterpart in the reference, whose dumps keep no weights
  // and have no reader): the canonical SDF with its weights, psi and the
  // current frame index go to a state file (kf_state_save).
  void saveState(const std::string &path) const;
  // Resume from a state file of saveState, written by a KillingFusion over a
  // dataset of the same geometry: the next processNextFrame continues the
  // sequence where the saved object stood, with the same results.
  void loadState(const std::string &path);

  // The frustum bounds of a w x h camera between minDepth and maxDepth in
  // world space with pose = identity (KillingFusion.cpp:478-519).
  static std::pair<kf::Vec3d, kf::Vec3d> computeBounds(const kf::Mat3d &K, int w, int h,
                                                       double minDepth, double maxDepth);

 private:
  SDF *computeSDF(int frameIndex);
  DisplacementField *createZeroDisplacementField(const SDF &sdf);
  void computeDisplacementField(const SDF *src, const SDF *dest, DisplacementField *srcToDest);

  int m_startFrame, m_endFrame, m_currFrameIndex, m_stride;
  DisplacementField *m_prev2CanDisplacementField = nullptr;
  DatasetReader m_datasetReader;
  SDF *m_canonicalSdf = nullptr;
  kf_solve_stats m_lastStats = {};
};
