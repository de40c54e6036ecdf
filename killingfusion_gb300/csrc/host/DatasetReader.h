// Depth-sequence reader with the reference's interface (DatasetReader.h:14-44).
// A dataset directory holds
//   intrinsics.txt      9 numbers, row-major 3x3 K (the reference's
//                       intrinsics file, read the same way, DatasetReader.cpp:36-47)
//   meta.txt            "width height numFrames minDepth maxDepth"
//   depth_%06d.f32      float32 metres, row-major [height][width], 0 = invalid
//                       (the masked depth the reference derives from its PNGs,
//                       DatasetReader.cpp:49-66)
// killingfusion_gb300.synth.write_dataset writes this layout.
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

 private:
  std::string m_root;
  kf::Mat3d m_depthIntrinsicMatrix;
  int m_numImageFiles = 0;
  int m_depthHeight = 0, m_depthWidth = 0;
  std::pair<double, double> m_minMaxDepth;
};
