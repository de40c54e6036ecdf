#include "DatasetReader.h"

#include <cstdio>
#include <iomanip>
#include <sstream>
#include <stdexcept>

#include "png.h"

static std::string join(const std::string &root, const std::string &name) {
  if (root.empty() || root.back() == '/') return root + name;
  return root + "/" + name;
}

static bool exists(const std::string &path) {
  FILE *fp = std::fopen(path.c_str(), "rb");
  if (!fp) return false;
  std::fclose(fp);
  return true;
}

// DatasetReader::LoadMatrixFromFile (DatasetReader.cpp:36-47): 9 numbers.
static kf::Mat3d load_intrinsics(const std::string &path) {
  FILE *fp = std::fopen(path.c_str(), "r");
  if (!fp) throw std::runtime_error("DatasetReader: cannot open " + path);
  kf::Mat3d K;
  for (int i = 0; i < 9; ++i) {
    double v = 0;
    if (std::fscanf(fp, "%lf", &v) != 1) {
      std::fclose(fp);
      throw std::runtime_error("DatasetReader: short intrinsics file " + path);
    }
    K.m[i] = v;
  }
  std::fclose(fp);
  return K;
}

static std::string frame_name(const char *prefix, int frameIndex, const char *ext) {
  std::ostringstream name;
  name << prefix << std::setw(6) << std::setfill('0') << frameIndex << ext;
  return name.str();
}

DatasetReader::DatasetReader(const std::string &root) : m_root(root) {
  const std::string meta = join(root, "meta.txt");
  if (exists(meta)) {
    m_depthIntrinsicMatrix = load_intrinsics(join(root, "intrinsics.txt"));
    FILE *fp = std::fopen(meta.c_str(), "r");
    double lo = 0, hi = 0;
    int ok = std::fscanf(fp, "%d %d %d %lf %lf", &m_depthWidth, &m_depthHeight, &m_numImageFiles, &lo, &hi);
    std::fclose(fp);
    if (ok != 5 || m_depthWidth <= 0 || m_depthHeight <= 0 || m_numImageFiles < 0)
      throw std::runtime_error("DatasetReader: bad meta file " + meta);
    m_minMaxDepth = std::make_pair(lo, hi);
    return;
  }
  // the reference's layout (DatasetReader.cpp:15-26, analyzeMinMaxDepthValues :68-80)
  const kf::Config &c = kf::config();
  const int t = c.datasetType;
  if (t < 0 || t > 1) throw std::runtime_error("DatasetReader: datasetType must be 0 (Duck) or 1 (Snoopy)");
  m_reference = true;
  m_imageDir = join(root, c.imageDir[t]);
  m_numImageFiles = c.numImageFiles[t];
  m_depthIntrinsicMatrix = load_intrinsics(join(root, c.intrinsicParamsFile));
  m_depthHeight = 480;
  m_depthWidth = 640;
  m_minMaxDepth = std::make_pair(c.datasetDepthMinMaxValues[t][0], c.datasetDepthMinMaxValues[t][1]);
}

std::vector<kf::DepthImage> DatasetReader::getImages(int frameIndex) const {
  std::vector<kf::DepthImage> out(2);
  kf::DepthImage &depth = out[1];
  depth.rows = m_depthHeight;
  depth.cols = m_depthWidth;
  if (m_reference) {
    // depth.copyTo(masked, mask) into a fresh matrix: zero where the mask is
    // zero (DatasetReader.cpp:59-64)
    const std::string dpath = m_imageDir + frame_name("depth_", frameIndex, ".png");
    const std::string mpath = m_imageDir + frame_name("omask_", frameIndex, ".png");
    if (!exists(dpath)) throw std::runtime_error("Error: depth image file not read! " + dpath);
    const kf::png::Image d = kf::png::read(dpath);
    const kf::png::Image m = kf::png::read(mpath);
    if (d.channels != 1) throw std::runtime_error("DatasetReader: depth image is not single-channel: " + dpath);
    if (d.width != m.width || d.height != m.height)
      throw std::runtime_error("DatasetReader: depth and mask sizes differ at frame " + std::to_string(frameIndex));
    depth.rows = d.height;
    depth.cols = d.width;
    depth.scale = 1.0 / 1000;
    depth.raw.resize((size_t)d.width * d.height);
    for (size_t i = 0; i < depth.raw.size(); ++i) {
      // IMREAD_GRAYSCALE of a colour mask: BT.601 luma in 14-bit fixed point
      unsigned g;
      if (m.channels >= 3) {
        const uint16_t *px = &m.samples[i * m.channels];
        g = (px[0] * 4899u + px[1] * 9617u + px[2] * 1868u + (1u << 13)) >> 14;
      } else {
        g = m.samples[i * m.channels];
      }
      depth.raw[i] = g ? d.samples[i] : 0;
    }
    return out;
  }
  const std::string path = join(m_root, frame_name("depth_", frameIndex, ".f32"));
  depth.data.resize((size_t)m_depthHeight * m_depthWidth);
  FILE *fp = std::fopen(path.c_str(), "rb");
  if (!fp) throw std::runtime_error("Error: depth image file not read! " + path);
  size_t got = std::fread(depth.data.data(), sizeof(float), depth.data.size(), fp);
  std::fclose(fp);
  if (got != depth.data.size()) throw std::runtime_error("DatasetReader: short depth file " + path);
  return out;
}
