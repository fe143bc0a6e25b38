// tables.cpp -- host-built constant tables of libgpb.
//
// Every table is computed here, on the host, from the reference's formulas;
// the kernels only read them.  Citations are to the reference's files.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gpb_internal.h"

namespace gpb {

static const double kRefPi = 3.1415926535;  // include/UCM_CONSTANTS.h:4

// ---------------------------------------------------------------- slices
// Half-disc slice of the label at offset (drow, dcol) from the centre:
// orientation_slice_map (globalPb/src/math/libraries/lib_image.cc:3052-3081)
// at the window position the convolution in compute_hist_gradient_2D
// (lib_image.cc:3120-3235) pairs with that label, i.e. the point
// (-drow-0.5, -dcol-0.5), evaluated in double: the compiled reference gives
// this map at every offset within radius 20, the exact diagonals included.
int slice_of(int drow, int dcol) {
  const double x = -(double)drow - 0.5, y = -(double)dcol - 0.5;
  int idx = (int)floor((atan2(y, x) + M_PI) / M_PI * 8.0);
  if (idx > 15) idx = 15;
  return idx;
}

// --------------------------------------------------------------- oeFilter
// Oriented first derivative of a Gaussian, sigma 1, support 3, as Berkeley's
// oeFilter computes it (the algorithm src/oeFilter.cpp:21-196 ports): 70x70
// sub-samples binned by their unrotated position, the separable function
// looked up on a finer grid at the rotated position, zero mean, unit L1 norm.
void oe_filter(double theta, double* out) {
  const double sigma = 1.0;
  const int hsz = 3, sz = 7, rate = 10, frate = 10, samples = sz * rate;
  const double r = floor(sz / 2.0) + 0.5 * (1 - 1.0 / rate);
  std::vector<double> dom(samples);
  for (int i = 0; i < samples; i++) dom[i] = -r + (2 * r) * i / (samples - 1);
  const double R = r * sqrt(2.0) * 1.01;
  int fs = (int)ceil(R * rate * frate);
  fs = fs + (fs + 1) % 2;
  std::vector<double> fx(fs), fy(fs);
  for (int i = 0; i < fs; i++) {
    const double t = -R + (2 * R) * i / (fs - 1);
    fx[i] = exp(-t * t / (2 * sigma * sigma));
    fy[i] = exp(-t * t / (2 * sigma * sigma)) * (-t / (sigma * sigma));
  }
  const double gap = 2 * R / (fs - 1);
  double acc[49] = {0};
  const double st = sin(theta), ct = cos(theta);
  for (int i = 0; i < samples; i++)
    for (int j = 0; j < samples; j++) {
      const double sx = dom[j], sy = dom[i];
      const int mx = (int)round(sx), my = (int)round(sy);
      const int memb = (mx + hsz + 1) + (my + hsz) * sz;
      if (memb < 1 || memb > sz * sz) continue;
      const double su = sx * st + sy * ct, sv = sx * ct - sy * st;
      const int xi = (int)round(su / gap) + fs / 2;
      const int yi = (int)round(sv / gap) + fs / 2;
      const int li = memb - 1;
      acc[(li % sz) * sz + li / sz] += fx[xi] * fy[yi];
    }
  double mean = 0;
  for (int i = 0; i < 49; i++) mean += acc[i];
  mean /= 49;
  double s = 0;
  for (int i = 0; i < 49; i++) {
    acc[i] -= mean;
    s += fabs(acc[i]);
  }
  for (int i = 0; i < 49; i++) out[i] = s > 0 ? acc[i] / s : acc[i];
}

// ------------------------------------------------------------------ IC
// The reference's intervening-contour walk (buildW/src/ic.cc:86-545) and the
// scanline lookup of computeAffinities2 (buildW/src/affinity.cc:58-156),
// evaluated once per clipping configuration on a symbolic lattice whose
// "values" are sets of mPb pixels (a 121-bit mask over the 11x11 box) and
// whose max is set union.  The result, per configuration and stencil offset,
// is the set of pixels whose mPb the reference max-accumulates.
namespace {
struct Mask {
  uint64_t lo = 0, hi = 0;
  void set(int b) { if (b < 64) lo |= 1ull << b; else hi |= 1ull << (b - 64); }
  void merge(const Mask& o) { lo |= o.lo; hi |= o.hi; }
};
struct SymPt {
  int x, y;
  Mask m;
};
struct SymLattice {
  int width, height, x0, y0;
  // H(x,y) = mPb[y-1][x], V(x,y) = mPb[y][x-1] (src/buildW.cpp:55-116)
  Mask pix(int x, int y) const {
    Mask m;
    m.set((y - y0 + kStencilR) * 11 + (x - x0 + kStencilR));
    return m;
  }
  Mask H(int x, int y) const { return y > 0 ? pix(x, y - 1) : Mask(); }
  Mask V(int x, int y) const { return x > 0 ? pix(x - 1, y) : Mask(); }
};

void sym_walk(const SymLattice& L, int x0, int y0, int x1, int y1, int x2, int y2, int x3, int y3,
              int wr, std::vector<int>& scanCount, std::vector<SymPt>& scan) {
  const long long dx1 = x1 - x0, dy1 = y1 - y0, dx2 = x2 - x0, dy2 = y2 - y0, dx3 = x3 - x0,
                  dy3 = y3 - y0;
  const long long dot11 = dx1 * dx1 + dy1 * dy1, dot22 = dx2 * dx2 + dy2 * dy2,
                  dot33 = dx3 * dx3 + dy3 * dy3;
  const int dx = x2 - x0, dy = y2 - y0, adx = abs(dx), ady = abs(dy);
  int oct = -1;
  if (dx > 0 && dy >= 0) oct = (adx > ady) ? 0 : 1;
  else if (dx <= 0 && dy > 0) oct = (adx < ady) ? 2 : 3;
  else if (dy <= 0 && dx < 0) oct = (adx > ady) ? 4 : 5;
  else if (dx >= 0 && dy < 0) oct = (adx < ady) ? 6 : 7;
  int t = (oct == 0 || oct == 3 || oct == 4 || oct == 7) ? -adx : -ady;
  Mask maxpb;
  int xi = x0, yi = y0, ox = xi, oy = yi;
  std::vector<SymPt> pts;
  while (xi != x2 || yi != y2) {
    switch (oct) {
      case 0: xi++; t += (ady << 1); if (t > 0) { yi++; t -= (adx << 1); } break;
      case 1: yi++; t += (adx << 1); if (t > 0) { xi++; t -= (ady << 1); } break;
      case 2: yi++; t += (adx << 1); if (t > 0) { xi--; t -= (ady << 1); } break;
      case 3: xi--; t += (ady << 1); if (t > 0) { yi++; t -= (adx << 1); } break;
      case 4: xi--; t += (ady << 1); if (t > 0) { yi--; t -= (adx << 1); } break;
      case 5: yi--; t += (adx << 1); if (t > 0) { xi--; t -= (ady << 1); } break;
      case 6: yi--; t += (adx << 1); if (t > 0) { xi++; t -= (ady << 1); } break;
      case 7: xi++; t += (ady << 1); if (t > 0) { yi--; t -= (adx << 1); } break;
    }
    const long long dxi = xi - x0, dyi = yi - y0;
    const long long dotii = dxi * dxi + dyi * dyi, doti1 = dxi * dx1 + dyi * dy1,
                    doti2 = dxi * dx2 + dyi * dy2, doti3 = dxi * dx3 + dyi * dy3;
    const bool good = (doti2 * doti2 == dotii * dot22) ||
                      (dot11 * doti2 * doti2 > dot22 * doti1 * doti1 &&
                       dot33 * doti2 * doti2 >= dot22 * doti3 * doti3);
    Mask in;
    if (ox == xi) {
      if (yi > oy) in = L.H(xi, yi);
      else if (yi < oy) in = L.H(ox, oy);
    } else if (oy == yi) {
      if (xi > ox) in = L.V(xi, yi);
      else if (xi < ox) in = L.V(ox, oy);
    } else if (xi > ox && yi > oy) {
      in.merge(L.H(ox, yi)); in.merge(L.H(xi, yi)); in.merge(L.V(xi, oy)); in.merge(L.V(xi, yi));
    } else if (xi > ox && yi < oy) {
      in.merge(L.H(ox, oy)); in.merge(L.H(xi, oy)); in.merge(L.V(xi, oy)); in.merge(L.V(xi, yi));
    } else if (xi < ox && yi > oy) {
      in.merge(L.H(ox, yi)); in.merge(L.H(xi, yi)); in.merge(L.V(ox, oy)); in.merge(L.V(ox, yi));
    } else if (xi < ox && yi < oy) {
      in.merge(L.H(ox, oy)); in.merge(L.H(xi, oy)); in.merge(L.V(ox, oy)); in.merge(L.V(ox, yi));
    }
    maxpb.merge(in);
    ox = xi;
    oy = yi;
    if (!good) continue;
    // mPb <= 1 after the clip, so the "maxpb > thresh(1.0)" stop never fires
    SymPt p;
    p.x = xi;
    p.y = yi;
    p.m = maxpb;
    pts.push_back(p);
  }
  const int wd = 2 * wr + 1;
  auto put = [&](const SymPt& p) {
    const int yind = p.y - y0 + wr;
    scan[yind * wd + scanCount[yind]++] = p;
  };
  if (oct == 0 || oct == 1 || oct == 6 || oct == 7) {
    for (size_t i = 0; i < pts.size(); i++) put(pts[i]);
  } else {
    for (int i = (int)pts.size() - 1; i >= 0; i--) put(pts[i]);
  }
}

std::vector<SymPt> sym_intervening(const SymLattice& L, int x0, int y0, int wr) {
  const int width = L.width, height = L.height, wd = 2 * wr + 1;
  std::vector<int> cnt(wd, 0);
  std::vector<SymPt> scan(wd * wd);
  const int rxa = std::max(0, x0 - wr), rya = std::max(0, y0 - wr);
  const int rxb = std::min(x0 + wr, width - 1), ryb = std::min(y0 + wr, height - 1);
  auto W = [&](int a, int b, int c, int d, int e, int f) { sym_walk(L, x0, y0, a, b, c, d, e, f, wr, cnt, scan); };
  auto P = [&](int x, int y) {
    SymPt p;
    p.x = x;
    p.y = y;
    const int yind = y - y0 + wr;
    scan[yind * wd + cnt[yind]++] = p;  // sim 1: no pixel crossed
  };
  if (x0 > rxa) {
    if ((y0 > 0) && (y0 < ryb)) W(rxa, y0 - 1, rxa, y0, rxa, y0 + 1);
    for (int y = y0 - 1; y > rya; y--) W(rxa, y - 1, rxa, y, rxa, y + 1);
  }
  if (x0 > rxa + 1 || y0 > rya + 1 || ((x0 > rxa) && (y0 > rya))) W(rxa, rya + 1, rxa, rya, rxa + 1, rya);
  if (((x0 == rxa) && (y0 == rya + 1)) || ((x0 == rxa + 1) && (y0 == rya))) P(rxa, rya);
  if (y0 > rya)
    for (int x = rxa + 1; x < rxb; x++) W(x - 1, rya, x, rya, x + 1, rya);
  if ((y0 > rya + 1) || (x0 < rxb - 1) || ((y0 > rya) && (x0 < rxb))) W(rxb - 1, rya, rxb, rya, rxb, rya + 1);
  if (((x0 == rxb - 1) && (y0 == rya)) || ((x0 == rxb) && (y0 == rya + 1))) P(rxb, rya);
  if (x0 < rxb)
    for (int y = rya + 1; y < y0; y++) W(rxb, y - 1, rxb, y, rxb, y + 1);
  if (x0 > rxa)
    for (int y = y0 + 1; y < ryb; y++) W(rxa, y - 1, rxa, y, rxa, y + 1);
  if ((x0 > rxa + 1) || (y0 < ryb - 1) || ((x0 > rxa) && (y0 < ryb))) W(rxa, ryb - 1, rxa, ryb, rxa + 1, ryb);
  if (((x0 == rxa) && (y0 == ryb - 1)) || ((x0 == rxa + 1) && (y0 == ryb))) P(rxa, ryb);
  if (y0 < ryb)
    for (int x = rxa + 1; x < rxb; x++) W(x - 1, ryb, x, ryb, x + 1, ryb);
  if ((y0 < ryb - 1) || (x0 < rxb - 1) || ((y0 < ryb) && (x0 < rxb))) W(rxb - 1, ryb, rxb, ryb, rxb, ryb - 1);
  if (((x0 == rxb - 1) && (y0 == ryb)) || ((x0 == rxb) && (y0 == ryb - 1))) P(rxb, ryb);
  if (x0 < rxb) {
    for (int y = ryb - 1; y > y0; y--) W(rxb, y - 1, rxb, y, rxb, y + 1);
    if ((y0 > 0) && (y0 < ryb)) W(rxb, y0 - 1, rxb, y0, rxb, y0 + 1);
  }
  std::vector<SymPt> adj;
  for (int y = 0; y < wd; y++)
    for (int i = 0; i < cnt[y]; i++) adj.push_back(scan[y * wd + i]);
  return adj;
}

void build_ic(HostTables& t) {
  t.ic.assign((size_t)kIcConfigs * kStencilN, IcPath());
  for (int cl = 0; cl < 6; cl++)
    for (int cr = 0; cr < 6; cr++)
      for (int ct = 0; ct < 6; ct++)
        for (int cb = 0; cb < 6; cb++) {
          const int cfg = ((cl * 6 + cr) * 6 + ct) * 6 + cb;
          SymLattice L;
          L.width = cl + cr + 1;
          L.height = ct + cb + 1;
          L.x0 = cl;
          L.y0 = ct;
          if (L.width < 2 || L.height < 2) continue;  // patches are >= 32 px
          const std::vector<SymPt> adj = sym_intervening(L, L.x0, L.y0, kStencilR);
          size_t idx = 0;
          for (int k = 0; k < kStencilN; k++) {
            IcPath& e = t.ic[(size_t)cfg * kStencilN + k];
            e.count = 0;
            const int u = t.sdy[k], v = t.sdx[k];
            const int yy = L.y0 + u, xx = L.x0 + v;
            if (xx < 0 || xx >= L.width || yy < 0 || yy >= L.height) continue;
            while (idx < adj.size() && adj[idx].y < yy) idx++;
            while (idx < adj.size() && adj[idx].x < xx) idx++;
            if (u == 0 && v == 0) continue;
            if (idx < adj.size() && adj[idx].x == xx && adj[idx].y == yy) {
              const Mask& m = adj[idx].m;
              int c = 0;
              for (int b = 0; b < 121; b++) {
                const bool on = b < 64 ? ((m.lo >> b) & 1) : ((m.hi >> (b - 64)) & 1);
                if (!on) continue;
                if (c < kIcMaxPath) {
                  e.dy[c] = (int8_t)(b / 11 - kStencilR);
                  e.dx[c] = (int8_t)(b % 11 - kStencilR);
                }
                c++;
              }
              e.count = (int8_t)std::min(c, kIcMaxPath);
              idx++;
            } else {
              e.count = -1;  // not found: icsim = 0
            }
          }
        }
}
}  // namespace

// ------------------------------------------------------------------ build
void build_tables(HostTables& t, int compat) {
  // stencil offsets in the scanline order of computeAffinities2 (u = dy, v = dx)
  int n = 0;
  for (int u = -kStencilR; u <= kStencilR; u++)
    for (int v = -kStencilR; v <= kStencilR; v++)
      if (u * u + v * v <= kStencilR * kStencilR) {
        t.sdy[n] = u;
        t.sdx[n] = v;
        n++;
      }
  // Schmid S filters (src/SPFeatures.cpp:117-183), FP32 as genTextonMap uses them
  static const int st[kNschmid][2] = {{2, 1}, {4, 1}, {4, 2}, {6, 1}, {6, 2}, {6, 3}, {8, 1},
                                      {8, 2}, {8, 3}, {10, 1}, {10, 2}, {10, 3}, {10, 4}};
  std::vector<double> F((size_t)kNschmid * 49 * 49);
  for (int f = 0; f < kNschmid; f++) {
    const int sg = st[f][0], ta = st[f][1];
    double fsum = 0, fabs_sum = 0;
    for (int i = 0; i < 49; i++)
      for (int j = 0; j < 49; j++) {
        const double x = j - 24, y = i - 24, r = sqrt(x * x + y * y);
        double v = cos(r * (kRefPi * ta / sg));
        v *= exp(-r * r / (2 * sg * sg));
        F[(size_t)f * 2401 + i * 49 + j] = v;
        fsum += v;
        fabs_sum += fabs(v);
      }
    const double mean = fsum / 2401, inv = 1.0 / fabs_sum;
    for (int k = 0; k < 2401; k++) F[(size_t)f * 2401 + k] = (F[(size_t)f * 2401 + k] - mean) * inv;
  }
  // rings (distinct a^2 + b^2, ascending) and symmetric groups (a <= b)
  int ring_id[2 * 24 * 24 + 1];
  for (int s = 0; s <= 2 * 24 * 24; s++) ring_id[s] = -1;
  for (int a = 0; a <= 24; a++)
    for (int b = 0; b <= 24; b++) ring_id[a * a + b * b] = 0;
  int nr = 0;
  for (int s = 0; s <= 2 * 24 * 24; s++)
    if (ring_id[s] == 0) ring_id[s] = nr++;
  t.n_rings = nr;
  t.k32_ring.assign((size_t)kNschmid * nr, 0.0);
  int g = 0;
  for (int a = 0; a <= 24; a++)
    for (int b = a; b <= 24; b++) {
      t.group_a[g] = a;
      t.group_b[g] = b;
      t.group_ring[g] = ring_id[a * a + b * b];
      for (int f = 0; f < kNschmid; f++) {
        const float k = (float)F[(size_t)f * 2401 + (24 + a) * 49 + (24 + b)];
        t.k32_group[f][g] = k;
        t.k32_ring[(size_t)f * nr + t.group_ring[g]] = (double)k;
      }
      g++;
    }
  // FP32 error bound of a response: sum of 325 products with |prod| <= 2040|k|,
  // accumulated in FP32 (Higham's gamma_n bound with n = 2*325, doubled)
  for (int f = 0; f < kNschmid; f++) {
    double s = 0;
    for (int q = 0; q < kSchmidGroups; q++) s += 2040.0 * fabs((double)t.k32_group[f][q]);
    t.err_bound[f] = (float)(2.0 * 650 * ldexp(1.0, -24) * s);
  }
  // colour: gamma 2.5 of u8/255 (lib_image.cc:123-140 after globalPb.cpp:20)
  for (int i = 0; i < 256; i++) t.gamma_lut[i] = pow(i * (1.0 / 255.0), 2.5);
  // bin smoothing kernels: lib_image::gaussian(0.1*25) and (0.05*25)
  // (mex_pb_parts_final_selected.cpp:95-97, lib_image.cc:1374-1441)
  auto gauss = [](double sigma, float* k) {
    const int sup = (int)ceil(3 * sigma), size = 2 * sup + 1;
    double tmp[64], s = 0;
    double x = -(double)sup;
    const double nt = -0.5 * (1.0 / (sigma * sigma));
    for (int i = 0; i < size; i++, x++) {
      tmp[i] = exp(x * x * nt);
      s += fabs(tmp[i]);
    }
    for (int i = 0; i < size; i++) k[i] = (float)(tmp[i] / s);
    return size;
  };
  t.nkbg = gauss(2.5, t.kbg);
  t.nkcg = gauss(1.25, t.kcg);
  // annulus offset lists, split over 32 lanes: lane = half*16 + slice
  static const int rad[kNannulus] = {3, 5, 10, 20};
  t.ann_dy.clear();
  t.ann_dx.clear();
  memset(t.slice_pixels, 0, sizeof(t.slice_pixels));
  for (int a = 0; a < kNannulus; a++) {
    const int r0 = a == 0 ? -1 : rad[a - 1], r1 = rad[a];
    std::vector<std::pair<int, int>> per_slice[16];
    for (int dy = -r1; dy <= r1; dy++)
      for (int dx = -r1; dx <= r1; dx++) {
        const int d2 = dy * dy + dx * dx;
        if (d2 > r1 * r1 || (r0 >= 0 && d2 <= r0 * r0)) continue;
        per_slice[slice_of(dy, dx)].push_back(std::make_pair(dy, dx));
      }
    for (int s = 0; s < 16; s++) {
      t.slice_pixels[a][s] = (a ? t.slice_pixels[a - 1][s] : 0) + (int)per_slice[s].size();
      for (int h = 0; h < 2; h++) {
        const int lane = h * 16 + s;
        t.ann_start[a][lane] = (int)t.ann_dy.size();
        int c = 0;
        for (size_t i = h; i < per_slice[s].size(); i += 2) {
          t.ann_dy.push_back((int16_t)per_slice[s][i].first);
          t.ann_dx.push_back((int16_t)per_slice[s][i].second);
          c++;
        }
        t.ann_count[a][lane] = c;
      }
    }
  }
  // weights (D10): CPU sets multiscalePb.cpp:19-26 and globalPb.cpp:31-36;
  // GPU sets combine.cu:16-21 and globalPb.cu:13
  static const float wm_cpu[12] = {0.0146f, 0.0145f, 0.0163f, 0.0210f, 0.0243f, 0.0287f,
                                   0.0166f, 0.0185f, 0.0204f, 0.0101f, 0.0111f, 0.0141f};
  static const float wg_cpu[13] = {0, 0, 0.0039f, 0.0050f, 0.0058f, 0.0069f, 0.0040f,
                                   0.0044f, 0.0049f, 0.0024f, 0.0027f, 0.0170f, 0.0074f};
  static const float wm_gpu[12] = {0.0123f, 0.0110f, 0.0117f, 0.0169f, 0.0176f, 0.0198f,
                                   0.0138f, 0.0138f, 0.0145f, 0.0144f, 0.0149f, 0.0158f};
  static const float wg_gpu[13] = {0, 0, 0.0028f, 0.0041f, 0.0042f, 0.0047f, 0.0033f,
                                   0.0033f, 0.0035f, 0.0035f, 0.0035f, 0.0188f, 0.0139f};
  const float* wm = compat ? wm_gpu : wm_cpu;
  const float* wgg = compat ? wg_gpu : wg_cpu;
  for (int k = 0; k < 12; k++) {
    t.w_mpb[k] = wm[k];
    t.w_g[k] = wgg[k];
  }
  t.w_spb = wgg[12];
  // oriented NMS (lib_image.cc:4083-4197) at orientations i*PI/8 with the
  // reference's truncated PI and tolerance PI/8: suppression direction,
  // interpolation weight and the orientation-difference cosines
  const long double PI_L = 3.141592653589793238462643383279502884L;
  const long double PI_2L = PI_L / 2, PI_4L = PI_L / 4;
  double oris[kNori];
  for (int i = 0; i < kNori; i++) oris[i] = (double)i * kRefPi / (double)kNori;
  const double o_tol = kRefPi / 8;
  for (int i = 0; i < kNori; i++) {
    double theta = (long double)oris[i] + PI_2L;
    theta = (long double)theta - floorl((long double)theta / PI_L) * PI_L;
    double d = 0;
    int nb[4][2];
    if (theta == 0) {
      int v[4][2] = {{-1, 0}, {-1, 0}, {1, 0}, {1, 0}};
      memcpy(nb, v, sizeof(v));
    } else if (theta < PI_4L) {
      d = tan(theta);
      int v[4][2] = {{-1, 0}, {-1, -1}, {1, 0}, {1, 1}};
      memcpy(nb, v, sizeof(v));
    } else if (theta < PI_2L) {
      d = tanl(PI_2L - theta);
      int v[4][2] = {{0, -1}, {-1, -1}, {0, 1}, {1, 1}};
      memcpy(nb, v, sizeof(v));
    } else if (theta == PI_2L) {
      int v[4][2] = {{0, -1}, {0, -1}, {0, 1}, {0, 1}};
      memcpy(nb, v, sizeof(v));
    } else if (theta < 3.0L * PI_4L) {
      d = tanl(theta - PI_2L);
      int v[4][2] = {{0, -1}, {1, -1}, {0, 1}, {-1, 1}};
      memcpy(nb, v, sizeof(v));
    } else {
      d = tanl(PI_L - theta);
      int v[4][2] = {{1, 0}, {1, -1}, {-1, 0}, {-1, 1}};
      memcpy(nb, v, sizeof(v));
    }
    memcpy(t.nms_nb[i], nb, sizeof(nb));
    t.nms_d[i] = (float)d;
    for (int j = 0; j < kNori; j++) {
      double o = oris[j] - oris[i];
      o = (long double)o - floorl((long double)o / (2 * PI_L)) * (2 * PI_L);
      if (o >= PI_L) o = 2 * PI_L - o;
      if (o >= PI_2L) o = PI_L - o;
      o = (o <= o_tol) ? 0 : (o - o_tol);
      t.nms_cos[i][j] = (float)cos(o);
    }
  }
  build_ic(t);
  // sPb: 8 oriented filters at theta = o*PI/8 into slot ch_per[o]
  // (src/spectralPb.cpp:291-322); with the Berkeley filter the slot that
  // aligns sPb_o with the orientation of the local cues is (4 - o) mod 8
  // (the reference's {3,2,1,0,7,6,5,4} belongs to its own filter port)
  static const int chp[8] = {4, 3, 2, 1, 0, 7, 6, 5};
  for (int o = 0; o < kNori; o++) {
    double f[49];
    oe_filter((kRefPi / 8) * (double)o, f);
    for (int i = 0; i < 49; i++) t.oe[o][i] = (float)f[i];
    t.ch_per[o] = chp[o];
  }
}

}  // namespace gpb
