// Depth-sequence reader with the reference's interface (DatasetReader.h:14-44).
// It reads two directory layouts.
//
// The reference's own (DatasetReader.cpp:15-66, config.cpp:10-19), used when
// the root holds no meta.txt:
//   <root>/intrinsics_kinect1.txt            9 numbers, row-major 3x3 K
//   <root>/<Duck/|Snoopy/>depth_%06d.png      16-bit depth, millimetres
//   <root>/<Duck/|Snoopy/>omask_%06d.png      8-bit object mask
// The dataset is kf::config().datasetType; frame count and depth range are the
// reference's cached values; frames are 640x480.  A frame is its depth where
// the mask is non-zero and 0 elsewhere, kept as 16-bit values with scale
// 1/1000 (the reference converts to double metres, DatasetReader.cpp:131-132).
//
// A raw layout for synthetic sequences, used when <root>/meta.txt exists:
//   intrinsics.txt      9 numbers, row-major 3x3 K
//   meta.txt            "width height numFrames minDepth maxDepth"
//   depth_%06d.f32      float32 metres, row-major [height][width], 0 = invalid
// killingfusion_gb300.synth.write_dataset writes it.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "SDF.h"
#include "kf_types.h"

class DatasetReader {
 public:
  DatasetReader() = delete;
  explicit DatasetReader(const std::string &datasetRootDir);

  // {color (empty: colour is not read), masked depth} for frameIndex, as
  // DatasetReader::getImages returns (DatasetReader.cpp:49-66).
  std::vector<kf::DepthImage> getImages(int frameIndex) const;

  int getNumImageFiles() const { return m_numImageFiles; }
  int getDepthHeight() const { return m_depthHeight; }
  int getDepthWidth() const { return m_depthWidth; }
  kf::Mat3d getDepthIntrinsicMatrix() const { return m_depthIntrinsicMatrix; }
  double getMinimumDepthThreshold() const { return m_minMaxDepth.first; }
  double getMaximumDepthThreshold() const { return m_minMaxDepth.second; }
  // true when reading the reference's PNG layout
  bool referenceLayout() const { return m_reference; }

 private:
  std::string m_root, m_imageDir;
  bool m_reference = false;
  kf::Mat3d m_depthIntrinsicMatrix;
  int m_numImageFiles = 0;
  int m_depthHeight = 0, m_depthWidth = 0;
  std::pair<double, double> m_minMaxDepth;
};
