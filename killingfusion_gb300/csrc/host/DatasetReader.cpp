#include "DatasetReader.h"

#include <cstdio>
#include <iomanip>
#include <sstream>
#include <stdexcept>

static std::string join(const std::string &root, const std::string &name) {
  if (root.empty() || root.back() == '/') return root + name;
  return root + "/" + name;
}

DatasetReader::DatasetReader(const std::string &root) : m_root(root) {
  std::string kpath = join(root, "intrinsics.txt");
  FILE *fp = std::fopen(kpath.c_str(), "r");
  if (!fp) throw std::runtime_error("DatasetReader: cannot open " + kpath);
  for (int i = 0; i < 9; ++i) {
    double v = 0;
    if (std::fscanf(fp, "%lf", &v) != 1) {
      std::fclose(fp);
      throw std::runtime_error("DatasetReader: short intrinsics file " + kpath);
    }
    m_depthIntrinsicMatrix.m[i] = v;
  }
  std::fclose(fp);
  std::string mpath = join(root, "meta.txt");
  fp = std::fopen(mpath.c_str(), "r");
  if (!fp) throw std::runtime_error("DatasetReader: cannot open " + mpath);
  double lo = 0, hi = 0;
  int ok = std::fscanf(fp, "%d %d %d %lf %lf", &m_depthWidth, &m_depthHeight, &m_numImageFiles, &lo, &hi);
  std::fclose(fp);
  if (ok != 5 || m_depthWidth <= 0 || m_depthHeight <= 0 || m_numImageFiles < 0)
    throw std::runtime_error("DatasetReader: bad meta file " + mpath);
  m_minMaxDepth = std::make_pair(lo, hi);
}

std::vector<kf::DepthImage> DatasetReader::getImages(int frameIndex) const {
  std::ostringstream name;
  name << "depth_" << std::setw(6) << std::setfill('0') << frameIndex << ".f32";
  std::string path = join(m_root, name.str());
  kf::DepthImage depth;
  depth.rows = m_depthHeight;
  depth.cols = m_depthWidth;
  depth.data.resize((size_t)m_depthHeight * m_depthWidth);
  FILE *fp = std::fopen(path.c_str(), "rb");
  if (!fp) throw std::runtime_error("Error: depth image file not read! " + path);
  size_t got = std::fread(depth.data.data(), sizeof(float), depth.data.size(), fp);
  std::fclose(fp);
  if (got != depth.data.size()) throw std::runtime_error("DatasetReader: short depth file " + path);
  std::vector<kf::DepthImage> out(2);
  out[1] = std::move(depth);
  return out;
}
