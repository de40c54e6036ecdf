// Stand-in for the reference's DatasetReader (DatasetReader.h:14-44), whose
// real implementation loads PNG frames through OpenCV.  It describes a 1x1
// camera at depth [1,1] so that KillingFusion's constructor allocates a
// one-voxel canonical grid; the oracle harness supplies every SDF itself.
// TEST INFRASTRUCTURE ONLY.
#include <DatasetReader.h>

DatasetReader::DatasetReader(const std::string DatasetRootDir)
    : m_imageDir(DatasetRootDir), m_numImageFiles(0), m_depthHeight(1), m_depthWidth(1),
      m_minMaxDepth(1.0, 1.0) {
  m_depthIntrinsicMatrix = Eigen::Matrix3d::Identity();
}
std::vector<cv::Mat> DatasetReader::getImages(int) { return std::vector<cv::Mat>(3, cv::Mat(1, 1)); }
int DatasetReader::getNumImageFiles() const { return m_numImageFiles; }
int DatasetReader::getDepthHeight() { return m_depthHeight; }
int DatasetReader::getDepthWidth() { return m_depthWidth; }
Eigen::Matrix3d DatasetReader::getDepthIntrinsicMatrix() { return m_depthIntrinsicMatrix; }
std::vector<double> DatasetReader::LoadMatrixFromFile(std::string, int) { return {}; }
cv::Mat DatasetReader::readDepthImage(std::string) { return cv::Mat(1, 1); }
void DatasetReader::analyzeMinMaxDepthValues(const DEFORMABLE_DATASET) {}
