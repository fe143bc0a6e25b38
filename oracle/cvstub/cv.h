// cv.h -- TEST INFRASTRUCTURE ONLY.  A minimal stand-in, written for this
// project, for the few OpenCV 2 pieces that the reference's UCM sources
// (src/contours2ucm.cpp, src/watershed.cpp, src/ucm_mean_pb.cpp,
// src/MATLAB_functions.cpp, src/mex_contour_sides.cpp) use, so that those
// files compile where they lie and serve as the oracle of the OWT-UCM stage.
// OpenCV itself is absent from this machine.
//
// Semantics kept from OpenCV's documented behaviour:
//   * a Mat shares its buffer on copy and assignment (clone() copies);
//   * row-major storage, at<T>(i, j) and the single-index at<T>(i) of a
//     continuous matrix;
//   * convertTo(dst, type, alpha, beta): saturate_cast<dst type>(v*alpha+beta),
//     rounding to nearest with ties to even (cvRound);
//   * minMaxLoc over all elements; Mat - scalar; Mat * Mat (matrix product
//     of two CV_64F matrices).
// Anything else the sources mention but the UCM path never calls aborts.
#ifndef GPB_CVSTUB_CV_H
#define GPB_CVSTUB_CV_H
#include <assert.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <memory>
#include <string>
#include <vector>

#define CV_8U 0
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_8UC1 CV_8U
#define CV_32SC1 CV_32S
#define CV_64FC1 CV_64F
#define CV_8UC3 16

namespace cv {

using std::string;  // OpenCV 2 brings these into namespace cv
using std::vector;
typedef unsigned char uchar;

struct Size {
  int width, height;
  Size() : width(0), height(0) {}
  Size(int w, int h) : width(w), height(h) {}
};

struct Scalar {
  double v;
  Scalar(double x = 0) : v(x) {}
};

inline void cvstub_unsupported(const char* what) {
  fprintf(stderr, "cvstub: %s is not part of the UCM path\n", what);
  abort();
}

inline size_t cvstub_elem(int type) {
  switch (type) {
    case CV_8U: return 1;
    case CV_32S: case CV_32F: return 4;
    case CV_64F: return 8;
    default: cvstub_unsupported("this element type"); return 0;
  }
}

class Mat {
 public:
  int rows, cols;
  uchar* data;

  Mat() : rows(0), cols(0), data(0), type_(CV_64F) {}
  Mat(int r, int c, int t) { alloc(r, c, t); }
  Mat(Size s, int t) { alloc(s.height, s.width, t); }
  Mat(int r, int c, int t, char* ext) { alloc(r, c, t); memcpy(data, ext, bytes()); }

  static Mat zeros(int r, int c, int t) { return Mat(r, c, t); }
  static Mat zeros(Size s, int t) { return Mat(s, t); }

  int type() const { return type_; }
  Size size() const { return Size(cols, rows); }
  bool empty() const { return rows == 0 || cols == 0; }
  size_t total() const { return (size_t)rows * cols; }
  void release() { buf_.reset(); data = 0; rows = cols = 0; }

  Mat clone() const {
    Mat m(rows, cols, type_);
    if (bytes()) memcpy(m.data, data, bytes());
    return m;
  }

  template <typename T> T& at(int i, int j) { return ((T*)data)[(size_t)i * cols + j]; }
  template <typename T> const T& at(int i, int j) const { return ((const T*)data)[(size_t)i * cols + j]; }
  template <typename T> T& at(int i) { return ((T*)data)[i]; }
  template <typename T> const T& at(int i) const { return ((const T*)data)[i]; }

  double get(size_t k) const {
    switch (type_) {
      case CV_8U: return data[k];
      case CV_32S: return ((const int*)data)[k];
      case CV_32F: return ((const float*)data)[k];
      default: return ((const double*)data)[k];
    }
  }
  void put(size_t k, double v) {  // saturate_cast with round-half-even
    switch (type_) {
      case CV_8U: {
        if (v != v) { data[k] = 0; break; }  // cvRound(NaN) saturates to 0
        double r = nearbyint(v);
        data[k] = (uchar)(r < 0 ? 0 : (r > 255 ? 255 : r));
        break;
      }
      case CV_32S: {
        double r = nearbyint(v);
        ((int*)data)[k] = (int)(r < -2147483648.0 ? -2147483648.0 : (r > 2147483647.0 ? 2147483647.0 : r));
        break;
      }
      case CV_32F: ((float*)data)[k] = (float)v; break;
      default: ((double*)data)[k] = v;
    }
  }

  void convertTo(Mat& dst, int t, double alpha = 1.0, double beta = 0.0) const {
    Mat out(rows, cols, t);
    for (size_t k = 0; k < total(); k++) out.put(k, get(k) * alpha + beta);
    dst = out;
  }

  // present in the compiled sources, never called on the UCM path
  Mat colRange(int, int) const { cvstub_unsupported("colRange"); return Mat(); }
  Mat rowRange(int, int) const { cvstub_unsupported("rowRange"); return Mat(); }
  Mat col(int) const { cvstub_unsupported("col"); return Mat(); }
  Mat reshape(int, int) const { cvstub_unsupported("reshape"); return Mat(); }
  void copyTo(Mat) const { cvstub_unsupported("copyTo"); }
  void create(int, int, int) { cvstub_unsupported("create"); }
  void setTo(Scalar, const Mat&) { cvstub_unsupported("setTo"); }

 private:
  int type_;
  std::shared_ptr<std::vector<uchar> > buf_;
  size_t bytes() const { return total() * cvstub_elem(type_); }
  // zero-filled guard bands of three rows on either side: reads a little
  // outside the matrix (CleanWatersheds near the border) see zeros
  void alloc(int r, int c, int t) {
    rows = r; cols = c; type_ = t;
    const size_t guard = (3 * (size_t)(c > 0 ? c : 1) + 8) * cvstub_elem(t);
    buf_.reset(new std::vector<uchar>((size_t)r * c * cvstub_elem(t) + 2 * guard, 0));
    data = buf_->data() + guard;
  }
};

inline Mat operator-(const Mat& a, double s) {
  Mat m(a.rows, a.cols, a.type());
  for (size_t k = 0; k < a.total(); k++) m.put(k, a.get(k) - s);
  return m;
}

inline Mat operator*(const Mat& a, const Mat& b) {
  if (a.type() != CV_64F || b.type() != CV_64F || a.cols != b.rows) cvstub_unsupported("this matrix product");
  Mat m(a.rows, b.cols, CV_64F);
  for (int i = 0; i < a.rows; i++)
    for (int j = 0; j < b.cols; j++) {
      double s = 0;
      for (int k = 0; k < a.cols; k++) s += a.at<double>(i, k) * b.at<double>(k, j);
      m.at<double>(i, j) = s;
    }
  return m;
}

inline void minMaxLoc(const Mat& a, double* mn, double* mx) {
  double lo = 0, hi = 0;
  for (size_t k = 0; k < a.total(); k++) {
    const double v = a.get(k);
    if (k == 0 || v < lo) lo = v;
    if (k == 0 || v > hi) hi = v;
  }
  if (mn) *mn = lo;
  if (mx) *mx = hi;
}

inline void merge(const Mat*, size_t, Mat&) { cvstub_unsupported("merge"); }
inline void repeat(const Mat&, int, int, Mat&) { cvstub_unsupported("repeat"); }
inline bool imwrite(const std::string&, const Mat&) { cvstub_unsupported("imwrite"); return false; }

}  // namespace cv
#endif
