// ucm_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// extern "C" entry points, written for this project, around the reference's
// own OWT-UCM sources compiled where they lie (src/contours2ucm.cpp,
// src/watershed.cpp, src/ucm_mean_pb.cpp, src/MATLAB_functions.cpp,
// src/fit_contour.cpp, src/mex_contour_sides.cpp, on top of lib_image's
// contour_set) against the OpenCV stand-in in oracle/cvstub.  Used only in
// this container to pin the oracle restatement and to write golden
// fixtures; never part of the product.
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "math/matrices/matrix.hh"

#include "head.h"

using math::matrices::matrix;

// Definitions the compiled sources reference from files that are not
// compiled here (src/utilities.cpp, src/mex_pb_parts_final_selected.cpp).
void OpenCVFileWriter(const cv::Mat&, std::string, std::string) {}
matrix<> ToMatrix(const cv::Mat& a) {  // row-major copy, as mex_pb_parts_final_selected.cpp:40-53
  matrix<> m((unsigned long)a.rows, (unsigned long)a.cols);
  for (int r = 0; r < a.rows; r++)
    for (int c = 0; c < a.cols; c++) m((unsigned long)r, (unsigned long)c) = a.at<double>(r, c);
  return m;
}

// Functions of src/contours2ucm.cpp that head.h does not declare.
superContour4COutput SuperContour4C(cv::Mat& pb);
cv::Mat CleanWatersheds(cv::Mat& wsClean);
cv::Mat NormalizeOutput(cv::Mat pb);
cv::Mat CreateFinestPartition(std::string pieceFilePat, std::vector<cv::Mat>& pbOriented);

namespace {
cv::Mat from_rows(const double* p, int r, int c) {
  cv::Mat m(r, c, CV_64F);
  memcpy(m.data, p, sizeof(double) * (size_t)r * c);
  return m;
}
std::vector<cv::Mat> planes(const double* p, int H, int W, int n) {
  std::vector<cv::Mat> v;
  for (int o = 0; o < n; o++) v.push_back(from_rows(p + (size_t)o * H * W, H, W));
  return v;
}
void to_rows(const cv::Mat& m, double* out) {
  for (int i = 0; i < m.rows; i++)
    for (int j = 0; j < m.cols; j++) out[(size_t)i * m.cols + j] = m.at<double>(i, j);
}
}  // namespace

extern "C" {

// Contours2Ucm (src/contours2ucm.cpp:405-490) on 8 row-major H x W planes;
// out holds (2H+1) x (2W+1) values when double_size, else (H+1) x (W+1).
int ref_ucm_contours2ucm(const double* orient, int H, int W, int double_size, double* out) {
  std::vector<cv::Mat> pb = planes(orient, H, W, 8);
  cv::Mat u = Contours2Ucm("", pb, double_size ? "doubleSize" : "imageSize");
  to_rows(u, out);
  return u.rows * 65536 + u.cols;
}

// watershed_yupeng (src/watershed.cpp:28-108), 8-connected, on a u8 image
int ref_ucm_watershed(const uint8_t* a, int H, int W, int32_t* out) {
  cv::Mat A(H, W, CV_8U);
  memcpy(A.data, a, (size_t)H * W);
  cv::Mat L = watershed_yupeng(A, 8);
  memcpy(out, L.data, sizeof(int32_t) * (size_t)H * W);
  return 0;
}

// CreateFinestPartition (src/contours2ucm.cpp:251-403): ws_wt, H x W
int ref_ucm_finest_partition(const double* orient, int H, int W, double* wswt) {
  std::vector<cv::Mat> pb = planes(orient, H, W, 8);
  to_rows(CreateFinestPartition("", pb), wswt);
  return 0;
}

// fit_contour (src/fit_contour.cpp) on a 0/1 image.  Returns the number of
// edges, or -1 when a capacity is too small.  vert: n_vert x 2 (row, col);
// edges: n_edges x 2 vertex ids; compl: completion flags; off: n_edges + 1
// offsets into xy, which holds (row, col) pairs of each edge's interior.
int ref_ucm_fit_contour(const double* bw, int H, int W, int cap_v, int cap_e, int cap_xy, int32_t* n_vert,
                        int32_t* vert, int32_t* edges, int32_t* compl_, int32_t* off, int32_t* xy) {
  cv::Mat m = from_rows(bw, H, W);
  FitContourOutput c = fit_contour(m);
  const int nv = c.vertices.rows, ne = (int)c.edge_x_coords.size();
  if (nv > cap_v || ne > cap_e) return -1;
  *n_vert = nv;
  for (int v = 0; v < nv; v++) {
    vert[2 * v] = c.vertices.at<int>(v, 0);
    vert[2 * v + 1] = c.vertices.at<int>(v, 1);
  }
  int k = 0;
  for (int e = 0; e < ne; e++) {
    edges[2 * e] = c.edges.at<int>(e, 0);
    edges[2 * e + 1] = c.edges.at<int>(e, 1);
    compl_[e] = c.is_completion.at<int>(e, 0);
    off[e] = k;
    const int n = c.edge_x_coords[e].rows;
    if (k + n > cap_xy) return -1;
    for (int p = 0; p < n; p++, k++) {
      xy[2 * k] = c.edge_x_coords[e].at<int>(p, 0);
      xy[2 * k + 1] = c.edge_y_coords[e].at<int>(p, 0);
    }
  }
  off[ne] = k;
  return ne;
}

// The middle of Contours2Ucm (src/contours2ucm.cpp:418-458): SuperContour4C,
// CleanWatersheds, bwlabel and the padded ws_wt2.  wswt2: (2H+1) x (2W+1);
// labels: H x W (from 0).
int ref_ucm_super_clean(const double* wswt, int H, int W, double* wswt2, int32_t* labels) {
  cv::Mat w = from_rows(wswt, H, W);
  superContour4COutput s = SuperContour4C(w);
  cv::Mat t = s.pb2.clone();
  t = CleanWatersheds(t);
  const int rows = t.rows, cols = t.cols;
  cv::Mat flag = cv::Mat::zeros(rows, cols, CV_32S);
  for (int i = 0; i < rows; i++)
    for (int j = 0; j < cols; j++)
      if (t.at<double>(i, j) == 0) flag.at<int>(i, j) = 1;
  cv::Mat l2 = bwlabel(flag, 8);
  for (int i = 0; i < rows / 2; i++)
    for (int j = 0; j < cols / 2; j++) labels[(size_t)i * (cols / 2) + j] = l2.at<int>(2 * i + 1, 2 * j + 1) - 1;
  for (int i = 0; i < rows + 1; i++)
    for (int j = 0; j < cols + 1; j++)
      wswt2[(size_t)i * (cols + 1) + j] = t.at<double>(i == rows ? rows - 1 : i, j == cols ? cols - 1 : j);
  return 0;
}

// UcmMeanPb (src/ucm_mean_pb.cpp:402-449): ucm, (2H+1) x (2W+1)
int ref_ucm_mean_pb(const double* wswt2, const int32_t* labels, int H, int W, double* ucm) {
  cv::Mat w = from_rows(wswt2, 2 * H + 1, 2 * W + 1);
  cv::Mat l(H, W, CV_32S);
  memcpy(l.data, labels, sizeof(int32_t) * (size_t)H * W);
  to_rows(UcmMeanPb(w, l), ucm);
  return 0;
}

// NormalizeOutput (src/contours2ucm.cpp:191-249)
int ref_ucm_normalize(const double* in, int rows, int cols, double* out) {
  to_rows(NormalizeOutput(from_rows(in, rows, cols)), out);
  return 0;
}

// bwlabel (bwlabelManu, src/MATLAB_functions.cpp:164-223) of a 0/1 image
int ref_ucm_bwlabel(const int32_t* bw, int H, int W, int32_t* out) {
  cv::Mat b(H, W, CV_32S);
  memcpy(b.data, bw, sizeof(int32_t) * (size_t)H * W);
  cv::Mat l = bwlabel(b, 8);
  memcpy(out, l.data, sizeof(int32_t) * (size_t)H * W);
  return 0;
}

}  // extern "C"
