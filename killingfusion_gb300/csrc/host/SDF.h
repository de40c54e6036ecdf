// The TSDF grid with the reference's interface (SDF.h:16-200), stored on the
// device as a kf_grid.  Whole-grid methods (integrateDepthFrame, fuse,
// update, getMesh) are single C ABI calls; the point accessors are device
// queries with the reference's sampling rules, one round trip per call.
#pragma once

#include <string>
#include <vector>

#include "DisplacementField.h"
#include "SimpleMesh.h"
#include "kf_types.h"

namespace kf {
// A depth image, standing in for the cv::Mat the reference integrates
// (SDF.cpp:137-177): float32 metres in `data`, or -- as the reference's PNG
// frames arrive -- 16-bit values in `raw` that are (double)v * scale metres
// (DatasetReader.cpp:131-132).  Row-major.
struct DepthImage {
  int rows = 0, cols = 0;
  std::vector<float> data;
  std::vector<uint16_t> raw;
  double scale = 0.0;
  const float *ptr() const { return data.data(); }
  bool is_raw() const { return !raw.empty(); }
};
}  // namespace kf

class SDF {
 public:
  // SDF::SDF (SDF.cpp:14-30): grid size int(bound / voxel) + 1 per axis,
  // phi = MaxSurfaceVoxelDistance + epsilon, weights 0.
  SDF(double voxelSize, kf::Vec3d min3dLoc, kf::Vec3d max3dLoc, double unknownClipDistance);
  // A new SDF of the same geometry; values are not copied (SDF.cpp:32-43).
  SDF(const SDF &copy);
  SDF(SDF &&other) noexcept;
  SDF &operator=(const SDF &) = delete;
  ~SDF();

  // The two-sphere fixture of KillingFusion::processTest (SDF.cpp:64-115).
  static std::vector<SDF> getDataEnergyTestSample(double voxelSize, double unknownClipDistance);

  // The reference's self-tests (SDF.cpp:526-568, 606-648, 681-724, 797-840)
  // on a 17^3 grid of voxel 0.5 holding f = x + y - z, through this class's
  // queries.  Where the reference asserts, these throw std::runtime_error
  // with the reference's message.
  static void testGetDistance();
  static void testGetWeight();
  static void testComputeDistanceGradient();
  static void testComputeDistanceHessian();

  void integrateDepthFrame(const kf::DepthImage &depthFrame, const kf::Mat4d &depthFrameC2WPose,
                           const kf::Mat3d &depthIntrinsicMatrix, double minDepth, double maxDepth);

  bool indexInGridBounds(int x, int y, int z) const;
  bool indexInGridBounds(const kf::Vec3i &i) const { return indexInGridBounds(i(0), i(1), i(2)); }
  double getDistanceAtIndex(const kf::Vec3i &i) const;
  double getDistanceAtIndex(int x, int y, int z) const { return getDistanceAtIndex(kf::Vec3i(x, y, z)); }
  long getWeightAtIndex(const kf::Vec3i &i) const;
  long getWeightAtIndex(int x, int y, int z) const { return getWeightAtIndex(kf::Vec3i(x, y, z)); }

  double getDistance(const kf::Vec3d &gridLocation) const;
  double getDistance(const kf::Vec3i &spatialIndex, const DisplacementField *psi) const;
  double getDistancef(const kf::Vec3d &gridLocation, const DisplacementField *psi) const;
  double getWeight(const kf::Vec3d &gridLocation) const;
  double getWeight(const kf::Vec3i &spatialIndex, const DisplacementField *psi) const;

  kf::Vec3d computeDistanceGradient(const kf::Vec3d &gridLocation) const;
  kf::Vec3d computeDistanceGradient(const kf::Vec3i &spatialIndex, const DisplacementField *psi) const;
  kf::Mat3d computeDistanceHessian(const kf::Vec3d &gridLocation) const;
  kf::Mat3d computeDistanceHessian(const kf::Vec3i &spatialIndex, const DisplacementField *psi) const;

  void fuse(const SDF *otherSdf);
  void fuse(const SDF *otherSdf, const DisplacementField *otherDisplacementField);
  void update(const DisplacementField *displacementField);

  SimpleMesh *getMesh() const;
  SimpleMesh *getMesh(const DisplacementField &displacementField) const;
  // <prefix><counter, 3 digits>.off (SDF.cpp:380-394, 423-430)
  void save_mesh(std::string meshNamePrefix, int fileCounter) const;
  void save_mesh(std::string meshNamePrefix, int fileCounter,
                 const DisplacementField &displacementField) const;

  // int32 dims[3], double min[3], double voxel, double truncation, double[N]
  // phi (SDF.cpp:432-460).
  void dumpToBinFile(std::string outputFilePath, double truncationDistanceInVoxelSizeUnit,
                     double minimumWeightThreshold) const;
  // Reads a file in dumpToBinFile's layout (no counterpart in the reference,
  // which only writes it): the grid's dims, placement and voxel size come
  // from the file, values are stored as float32.  The file keeps no
  // weights: a voxel whose value is not the initial MaxSurfaceVoxelDistance
  // + epsilon gets weight 1, the others 0.  getMax3dLoc() is the min corner
  // plus (dims - 1/2) voxels, a bound that gives the file's dims back.
  static SDF *loadFromBinFile(const std::string &path, double unknownClipDistance);

  kf::Vec3d getMin3dLoc() const { return m_min3dLoc; }
  kf::Vec3d getMax3dLoc() const { return m_max3dLoc; }
  kf::Vec3i getGridSize() const { return m_gridSize; }
  double getVoxelSize() const { return m_voxelSize; }
  kf_grid handle() const { return m_grid; }

  // Output directory of save_mesh (the reference's OUTPUT_DIR).
  static std::string &outputDir();

 private:
  void allocate();
  SDF(kf_grid grid, double unknownClipDistance);  // adopts a grid made by the C ABI
  std::vector<double> sampleDistances(const std::vector<double> &pts) const;
  std::vector<double> warpedPoints(const std::vector<double> &pts, const DisplacementField *psi) const;
  kf_grid m_grid = nullptr;
  kf::Vec3i m_gridSize;
  kf::Vec3d m_min3dLoc, m_max3dLoc;
  double m_voxelSize;
  double m_unknownClipDistance;
};
