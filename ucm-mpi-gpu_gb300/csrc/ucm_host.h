// ucm_host.h -- host stages of the oriented watershed transform and the
// ultrametric contour map (ucm_host.cpp).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <functional>
#include <vector>

namespace gpb {
namespace ucm {

struct FitResult {
  std::vector<int32_t> vx, vy;    // vertex (row, column)
  std::vector<int32_t> es, ee;    // edge start / end vertex
  std::vector<int32_t> off, px;   // edge e's interior pixels (row * W + column) are px[off[e] .. off[e+1])
};

uint32_t components8(const uint8_t* bw, int H, int W, std::vector<uint32_t>& lab);
// runs f(0..n-1), possibly on several threads
using ParFor = std::function<void(int, const std::function<void(int)>&)>;
bool fit_contours(const uint8_t* bw, int H, int W, FitResult& out, const ParFor* par = nullptr);
int edge_orientation(int x1, int y1, int x2, int y2);
// UcmMeanPb: the (2H+1) x (2W+1) map before calibration
void mean_pb_merge(const double* lb, const int32_t* part, int H, int W, double* ucm);
// the same on float strengths, calibrated (NormalizeOutput): the doubled
// grid, or with half Contours2Ucm's (H+1) x (W+1) output; with par the
// setup and the output run on the pool (the merge itself is sequential)
void mean_pb_ucm(const float* lb, const int32_t* part, int H, int W, bool half, double* out,
                 const ParFor* par = nullptr);
void normalize(double* u, size_t n);
// the pixels painted along the edges with their orientation bins, edge by
// edge: interior pixels, then the two end points
void paint_list(const FitResult& f, int W, std::vector<int32_t>& pix, std::vector<uint8_t>& ori,
                const ParFor* par = nullptr);

}  // namespace ucm
}  // namespace gpb
