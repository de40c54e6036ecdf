// Minimal stand-in for the single OpenCV type the reference's hot-path files
// touch: cv::Mat used as a row-major double depth image (SDF.cpp:137-177).
// Written for this project so that those files compile unmodified into the
// oracle reference build (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
#ifndef KF_SHIM_OPENCV
#define KF_SHIM_OPENCV

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace cv {
class Mat {
 public:
  int rows = 0, cols = 0;
  Mat() {}
  Mat(int r, int c) : rows(r), cols(c), buf_(std::make_shared<std::vector<double>>((size_t)r * c)) {}
  // Wraps caller memory without copying (the harness owns it).
  Mat(int r, int c, double *p) : rows(r), cols(c), ext_(p) {}
  template <typename T>
  T &at(int r, int c) {
    return reinterpret_cast<T *>(base())[(size_t)r * cols + c];
  }
  template <typename T>
  const T &at(int r, int c) const {
    return reinterpret_cast<const T *>(base())[(size_t)r * cols + c];
  }

 private:
  double *base() const { return ext_ ? ext_ : buf_->data(); }
  std::shared_ptr<std::vector<double>> buf_;
  double *ext_ = nullptr;
};
}  // namespace cv

#endif
