// Minimal stand-in for the parts of OpenCV that painty's hot-path headers name, written for
// this repository so painty/image/Mat.hxx and the renderer headers compile unmodified in the
// oracle build (OpenCV is not installed here).
//
// cv::Mat_<T> shares its buffer on copy, as OpenCV's does. New buffers are zero-filled and
// carry one extra zero row of slack: painty's FootprintBrush reads one row past its padded
// footprint when the pickup map is one cell wider (FootprintBrush.hxx:352, 396), and the
// padding value 0 is what that read is meant to see.
//
// cv::resize is the footprint scaler of FootprintBrush::setRadius. OpenCV's Lanczos-4 kernel
// is replaced by a bilinear resample (pixel-centre aligned, BORDER_REFLECT) implemented by
// the harness with painty's own painty::Interpolate.
//
// TextureBrushDictionary.cxx adds cv::normalize (NORM_MINMAX: OpenCV's documented
// dst = src * scale + shift with scale = (b - a) / (max - min), 0 when max - min is at most
// DBL_EPSILON, computed in double and rounded to the destination type), cv::flip about the
// x axis and Mat_::convertTo, and the standard headers OpenCV's own headers bring in.
#pragma once
#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#define CV_MAKETYPE(depth, cn) ((depth) + (((cn)-1) << 3))
#define CV_32FC1 CV_MAKETYPE(5, 1)

namespace cv {
enum BorderTypes { BORDER_CONSTANT = 0, BORDER_REPLICATE = 1, BORDER_REFLECT = 2 };
enum InterpolationFlags { INTER_NEAREST = 0, INTER_LINEAR = 1, INTER_LANCZOS4 = 4 };
enum NormTypes { NORM_MINMAX = 32 };

template <typename T>
class DataDepth {
 public:
  enum { value = 0, fmt = 0 };
};

template <typename T>
class DataType {
 public:
  typedef T value_type;
  typedef T channel_type;
  enum { generic_type = 0, depth = 0, channels = 1, fmt = 0, type = 0 };
};

struct Size {
  int width = 0, height = 0;
  Size() = default;
  Size(int w, int h) : width(w), height(h) {}
};

// BORDER_REFLECT ("fedcba|abcdefgh|hgfedcb"), the only mode painty uses
inline int borderInterpolate(int p, int len, int /*borderType*/) {
  if (len == 1) return 0;
  while (p < 0 || p >= len) p = p < 0 ? -p - 1 : len - 1 - (p - len);
  return p;
}

template <typename T>
class Mat_ {
 public:
  int rows = 0, cols = 0;
  unsigned char* data = nullptr;  // the first element, as OpenCV's Mat::data
  Mat_() = default;
  Mat_(int r, int c) : rows(r), cols(c), buf_(std::make_shared<std::vector<T>>(
                                              static_cast<size_t>(r + 1) * c + 1, T())) {
    data = reinterpret_cast<unsigned char*>(buf_->data());
  }
  explicit Mat_(Size s) : Mat_(s.height, s.width) {}
  size_t total() const { return static_cast<size_t>(rows) * cols; }
  Size size() const { return Size(cols, rows); }
  T& operator()(int r, int c) { return (*buf_)[static_cast<size_t>(r) * cols + c]; }
  const T& operator()(int r, int c) const { return (*buf_)[static_cast<size_t>(r) * cols + c]; }
  T& operator()(int i) { return (*buf_)[static_cast<size_t>(i)]; }
  const T& operator()(int i) const { return (*buf_)[static_cast<size_t>(i)]; }
  T* begin() { return buf_ ? buf_->data() : nullptr; }
  T* end() { return buf_ ? buf_->data() + total() : nullptr; }
  const T* begin() const { return buf_ ? buf_->data() : nullptr; }
  const T* end() const { return buf_ ? buf_->data() + total() : nullptr; }
  Mat_ clone() const {
    Mat_ r(rows, cols);
    if (buf_) *r.buf_ = *buf_;
    return r;
  }
  bool empty() const { return total() == 0; }
  // dst = src * alpha + beta in double, rounded to U (a plain conversion when alpha is 1 and
  // beta 0)
  template <typename U>
  void convertTo(Mat_<U>& dst, int /*rtype*/, double alpha = 1.0, double beta = 0.0) const {
    Mat_<U> out(rows, cols);
    for (size_t i = 0; i < total(); i++) {
      const double v = static_cast<double>((*buf_)[i]);
      out(static_cast<int>(i)) =
        static_cast<U>(alpha == 1.0 && beta == 0.0 ? v : v * alpha + beta);
    }
    dst = out;
  }

 private:
  std::shared_ptr<std::vector<T>> buf_;
};

template <typename S, typename D>
void normalize(const Mat_<S>& src, Mat_<D>& dst, double a, double b, int /*norm_type*/) {
  double smin = 0.0, smax = 0.0;
  for (size_t i = 0; i < src.total(); i++) {
    const double v = static_cast<double>(src(static_cast<int>(i)));
    if (i == 0 || v < smin) smin = v;
    if (i == 0 || v > smax) smax = v;
  }
  const double dmin = std::min(a, b), dmax = std::max(a, b);
  const double scale = (dmax - dmin) * (smax - smin > DBL_EPSILON ? 1.0 / (smax - smin) : 0.0);
  const double shift = dmin - smin * scale;
  src.convertTo(dst, 0, scale, shift);  // into a new buffer: src may be dst
}

// flip_code 0: about the x axis (row order reversed)
template <typename T>
void flip(const Mat_<T>& src, Mat_<T>& dst, int /*flip_code*/) {
  Mat_<T> out(src.rows, src.cols);
  for (int r = 0; r < src.rows; r++)
    for (int c = 0; c < src.cols; c++) out(r, c) = src(src.rows - 1 - r, c);
  dst = out;
}

// Implemented by the harness with painty::Interpolate (see the file comment).
void shim_resize_bilinear(const Mat_<double>& src, Mat_<double>& dst, int rows, int cols);

inline void resize(const Mat_<double>& src, Mat_<double>& dst, Size dsize, double, double,
                   int) {
  shim_resize_bilinear(src, dst, dsize.height, dsize.width);
}
}  // namespace cv
