// ucm_host.cpp -- the sequential stages of the oriented watershed transform
// and the ultrametric contour map (Contours2Ucm, src/contours2ucm.cpp:251-490)
// on the host: contour fitting of the watershed arcs and the greedy
// mean-boundary merge.  The data-parallel stages around them (orientation
// max, 8-bit quantisation, flooding, super-contour grid, labelling, edge
// painting) run on the GPU (k_ucm.cu).
//
// Contour fitting restates lib_image::connected_components and
// lib_image::contour_set (globalPb/src/math/libraries/lib_image.cc:4773-4910,
// 5320-5485 construction and tracing, 5685-5744 split_edge, 5953-6022
// subdivide_local, 6138-6326 subdivide_global) as called by MexContourSides
// (src/mex_contour_sides.cpp:120-225).  The completion edges of
// completion_cdt are never painted (contours2ucm.cpp:337,379) and are not
// built.  Intersections of the straight-line approximations are found by
// exact integer tests over a uniform grid of cells rather than by the
// reference's Bentley-Ottmann sweep (globalPb/src/math/geometry/
// seg_intersect.cc); the marking rules per intersection point are the
// reference's.
//
// The merge restates ComputeUcm (src/ucm_mean_pb.cpp:254-398): the same
// priority order (energy, region1, region2), the same pushes and the same
// running sums, so ties break exactly as there.  Boundary elements that
// became interior are dropped lazily instead of by a scan of the father's
// list, and the smaller of two element lists is moved into the larger; both
// leave every update of the map unchanged.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <deque>
#include <map>
#include <queue>
#include <utility>
#include <vector>

#include "../../include/gpb.h"
#include "ucm_host.h"

namespace gpb {
namespace ucm {

// ------------------------------------------------------------ components

// 8-connected components of the non-zero pixels of a row-major H x W map,
// numbered 1.. in the order of each component's first pixel in row-major
// order (lib_image.cc:4773-4910 visits elements in linear order and floods
// each new component).  Two raster passes: provisional labels, in order of
// their first pixel, with their equivalences in a union-find whose roots
// are the smallest labels; then each root, taken in label order, is
// numbered -- which is the order of the components' first pixels.
static uint32_t find_root(std::vector<uint32_t>& p, uint32_t a) {
  while (p[a] != a) {
    p[a] = p[p[a]];
    a = p[a];
  }
  return a;
}

uint32_t components8(const uint8_t* bw, int H, int W, std::vector<uint32_t>& lab) {
  const size_t N = (size_t)H * W;
  lab.assign(N, 0);
  std::vector<uint32_t> par(1, 0);  // provisional label 0 is the background
  auto unite = [&](uint32_t a, uint32_t b) {
    a = find_root(par, a);
    b = find_root(par, b);
    if (a == b) return;
    if (a < b) std::swap(a, b);
    par[a] = b;
  };
  for (int x = 0; x < H; x++) {
    const uint8_t* r = bw + (size_t)x * W;
    uint32_t* l = lab.data() + (size_t)x * W;
    const uint32_t* u = x > 0 ? l - W : nullptr;
    for (int y = 0; y < W; y++) {
      if (!r[y]) continue;
      uint32_t m = 0;  // the smallest labelled neighbour seen so far
      auto see = [&](uint32_t v) {
        if (!v) return;
        if (!m) m = v;
        else if (v != m) unite(m, v);
      };
      if (y > 0) see(l[y - 1]);
      if (u) {
        if (y > 0) see(u[y - 1]);
        see(u[y]);
        if (y + 1 < W) see(u[y + 1]);
      }
      if (!m) {
        m = (uint32_t)par.size();
        par.push_back(m);
      }
      l[y] = m;
    }
  }
  std::vector<uint32_t> fin(par.size(), 0);
  uint32_t n = 0;
  for (uint32_t v = 1; v < par.size(); v++) {
    const uint32_t r = find_root(par, v);
    fin[v] = r == v ? ++n : fin[r];  // a root is its component's first label
  }
  for (size_t i = 0; i < N; i++) lab[i] = fin[lab[i]];
  return n;
}

// ------------------------------------------------------------ contour set

namespace {

// Neighbour bits in the reference's naming, x = row and y = column:
// n = (x, y+1), s = (x, y-1), e = (x+1, y), w = (x-1, y), ne = (x+1, y+1),
// nw = (x-1, y+1), se = (x+1, y-1), sw = (x-1, y-1).
enum { BN = 1, BS = 2, BE = 4, BW = 8, BNE = 16, BNW = 32, BSE = 64, BSW = 128 };

// is_vertex_2D (lib_image.cc:4421-4478) restated as a predicate on the
// 8-bit neighbour mask; tabulated once.
bool vertex_rule(unsigned m) {
  const bool n = m & BN, s = m & BS, e = m & BE, w = m & BW;
  const bool ne = m & BNE, nw = m & BNW, se = m & BSE, sw = m & BSW;
  const int nadj = n + s + e + w, ndiag = ne + nw + se + sw, nn = nadj + ndiag;
  if (nn <= 1) return true;  // an end point
  if (nn == 2) return (n && (ne || nw)) || (s && (se || sw)) || (e && (ne || se)) || (w && (nw || sw));
  if (nn == 3 || nn == 4) {
    if ((nw && n && w) || (n && ne && e) || (w && sw && s) || (e && s && se)) return true;  // 2x2 block
    if ((nw && n && ne) || (sw && s && se) || (nw && w && sw) || (ne && e && se)) return nn == 3;
    if (nadj >= 3 || ndiag >= 3) return true;
    if ((n && se && sw) || (s && ne && nw) || (w && se && ne) || (e && nw && sw)) return true;
    if ((nw && s && e) || (ne && s && w) || (sw && n && e) || (se && n && w)) return true;
    return false;
  }
  return !(nadj == 2 && ((n && s) || (e && w)));  // not the middle of an H
}

struct VertexTable {
  bool v[256];
  VertexTable() {
    for (unsigned m = 0; m < 256; m++) v[m] = vertex_rule(m);
  }
};
const VertexTable kVertex;

struct Vert {
  int x, y;
  int degree;  // edges starting or ending here
};

struct Edge {
  int vs, ve;                // vertex ids
  std::vector<int32_t> px;   // interior pixels, packed x * W + y, in trace order
};

class Contours {
 public:
  Contours(const uint8_t* bw, int H, int W, const ParFor* par) : H_(H), W_(W), par_(par) { build(bw); }

  void subdivide_local();
  bool subdivide_global();  // false where the reference throws

  int H_, W_;
  const ParFor* par_;  // host pool for the crossing tests, or null
  std::vector<Vert> vert;
  std::vector<Edge> edge;

 private:
  std::vector<uint32_t> lab_;
  std::vector<uint8_t> is_v_, is_e_;
  std::vector<int32_t> assign_;

  uint32_t lab(int x, int y) const { return lab_[(size_t)x * W_ + y]; }
  void build(const uint8_t* bw);
  void trace(int v_id, int x, int y);
  int add_vertex(int x, int y) {
    const int id = (int)vert.size();
    vert.push_back({x, y, 0});
    const size_t i = (size_t)x * W_ + y;
    assign_[i] = id;
    is_v_[i] = 1;
    return id;
  }
  void add_edge(int vs, int ve, std::vector<int32_t>&& px) {
    edge.push_back({vs, ve, std::move(px)});
    vert[vs].degree++;
    vert[ve].degree++;
  }
  void split(int e_id, size_t p);
  double dist_seg(int32_t pix, int a, int b) const;
  size_t farthest(const Edge& e) const;
};

// Distance from a pixel to the segment between two vertices, in the
// operation order of point_2D::distance_to_segment (point_2D.cc:239-256).
double Contours::dist_seg(int32_t pix, int a, int b) const {
  const double px = pix / W_, py = pix % W_;
  const double ax = vert[a].x, ay = vert[a].y, bx = vert[b].x, by = vert[b].y;
  const double xa = bx - ax, ya = by - ay, xb = px - ax, yb = py - ay, xc = px - bx, yc = py - by;
  if ((xa * xc + ya * yc) >= 0) return sqrt(xc * xc + yc * yc);
  if ((-xa * xb - ya * yb) >= 0) return sqrt(xb * xb + yb * yb);
  return fabs(xa * yb - ya * xb) / sqrt(xa * xa + ya * ya);
}

// find_contour_point_farthest_from_segment (lib_image.cc:6110-6127)
size_t Contours::farthest(const Edge& e) const {
  size_t pos = 0;
  double best = 0;
  for (size_t n = 0; n < e.px.size(); n++) {
    const double d = dist_seg(e.px[n], e.vs, e.ve);
    if (d > best) {
      pos = n;
      best = d;
    }
  }
  return pos;
}

void Contours::build(const uint8_t* bw) {
  const size_t N = (size_t)H_ * W_;
  const uint32_t nl = components8(bw, H_, W_, lab_);
  is_v_.assign(N, 0);
  is_e_.assign(N, 0);
  assign_.assign(N, 0);
  std::vector<uint8_t> has_v(nl, 0);
  std::vector<int> last_x(nl, 0), last_y(nl, 0);
  for (int x = 0; x < H_; x++)
    for (int y = 0; y < W_; y++) {
      const uint32_t l = lab(x, y);
      if (!l) continue;
      unsigned m = 0;
      const bool hn = y + 1 < W_, hs = y > 0, he = x + 1 < H_, hw = x > 0;
      if (hn && lab(x, y + 1) == l) m |= BN;
      if (hs && lab(x, y - 1) == l) m |= BS;
      if (he && lab(x + 1, y) == l) m |= BE;
      if (hw && lab(x - 1, y) == l) m |= BW;
      if (hn && he && lab(x + 1, y + 1) == l) m |= BNE;
      if (hn && hw && lab(x - 1, y + 1) == l) m |= BNW;
      if (hs && he && lab(x + 1, y - 1) == l) m |= BSE;
      if (hs && hw && lab(x - 1, y - 1) == l) m |= BSW;
      if (kVertex.v[m]) {
        add_vertex(x, y);
        has_v[l - 1] = 1;
      }
      last_x[l - 1] = x;
      last_y[l - 1] = y;
    }
  for (uint32_t l = 0; l < nl; l++)  // a closed loop: its last pixel becomes a vertex
    if (!has_v[l]) add_vertex(last_x[l], last_y[l]);
  for (size_t v_id = 0; v_id < vert.size(); v_id++) {  // grows while tracing
    const int vx = vert[v_id].x, vy = vert[v_id].y;
    const uint32_t l = lab(vx, vy);
    int qx[8], qy[8], nq = 0;
    const int x0 = vx > 0 ? vx - 1 : vx + 1, y0 = vy > 0 ? vy - 1 : vy + 1;
    for (int x = x0; x <= vx + 1 && x < H_; x += 2)
      if (lab(x, vy) == l) qx[nq] = x, qy[nq++] = vy;
    for (int y = y0; y <= vy + 1 && y < W_; y += 2)
      if (lab(vx, y) == l) qx[nq] = vx, qy[nq++] = y;
    for (int x = x0; x <= vx + 1 && x < H_; x += 2)
      for (int y = y0; y <= vy + 1 && y < W_; y += 2)
        if (lab(x, y) == l && lab(vx, y) != l && lab(x, vy) != l) qx[nq] = x, qy[nq++] = y;
    for (int k = 0; k < nq; k++) {
      const size_t i = (size_t)qx[k] * W_ + qy[k];
      if (is_v_[i]) {
        if (assign_[i] > (int32_t)v_id) add_edge((int)v_id, assign_[i], {});
      } else if (!is_e_[i]) {
        trace((int)v_id, qx[k], qy[k]);
      }
    }
  }
  // drop vertices without edges (single-pixel islands) and renumber
  std::vector<int> remap(vert.size(), -1);
  std::vector<Vert> kept;
  for (size_t v = 0; v < vert.size(); v++) {
    if (vert[v].degree == 0) {
      is_v_[(size_t)vert[v].x * W_ + vert[v].y] = 0;
      continue;
    }
    remap[v] = (int)kept.size();
    kept.push_back(vert[v]);
  }
  vert.swap(kept);
  for (Edge& e : edge) {
    e.vs = remap[e.vs];
    e.ve = remap[e.ve];
  }
}

// trace_edge (lib_image.cc:5554-5680): follow unassigned pixels of the
// component, adjacent steps before diagonal ones and non-vertices before
// vertices, until a vertex or a dead end (which becomes a new vertex).
void Contours::trace(int v_id, int x, int y) {
  const size_t iv = (size_t)vert[v_id].x * W_ + vert[v_id].y;
  const uint32_t l = lab_[iv];
  const int e_id = (int)edge.size();
  std::vector<int32_t> px;
  is_e_[iv] = 1;
  bool new_vertex = false;
  for (;;) {
    const size_t i = (size_t)x * W_ + y;
    px.push_back((int32_t)i);
    is_e_[i] = 1;
    assign_[i] = e_id;
    const bool hn = y + 1 < W_, hs = y > 0, he = x + 1 < H_, hw = x > 0;
    auto av = [&](bool has, size_t j) { return has && lab_[j] == l && !is_e_[j]; };
    const size_t in = i + 1, is = i - 1, ie = i + W_, iw = i - W_;
    const bool an = av(hn, in), as = av(hs, is), ae = av(he, ie), aw = av(hw, iw);
    const bool ane = av(hn && he, ie + 1), anw = av(hn && hw, iw + 1), ase = av(hs && he, ie - 1),
               asw = av(hs && hw, iw - 1);
    if (an && !is_v_[in]) { y++; continue; }
    if (as && !is_v_[is]) { y--; continue; }
    if (ae && !is_v_[ie]) { x++; continue; }
    if (aw && !is_v_[iw]) { x--; continue; }
    if (an) { y++; break; }
    if (as) { y--; break; }
    if (ae) { x++; break; }
    if (aw) { x--; break; }
    if (ane && !is_v_[ie + 1]) { x++; y++; continue; }
    if (anw && !is_v_[iw + 1]) { x--; y++; continue; }
    if (ase && !is_v_[ie - 1]) { x++; y--; continue; }
    if (asw && !is_v_[iw - 1]) { x--; y--; continue; }
    if (ane) { x++; y++; break; }
    if (anw) { x--; y++; break; }
    if (ase) { x++; y--; break; }
    if (asw) { x--; y--; break; }
    new_vertex = true;
    is_e_[i] = 0;
    break;
  }
  is_e_[iv] = 0;
  const size_t iend = (size_t)x * W_ + y;
  if (new_vertex) {
    px.pop_back();
    add_vertex(x, y);
  }
  add_edge(v_id, assign_[iend], std::move(px));
}

// split_edge (lib_image.cc:5685-5744): a new vertex at interior point p;
// the edge keeps the points before it, a new edge (appended) those after.
void Contours::split(int e_id, size_t p) {
  const int32_t at = edge[e_id].px[p];
  const int v = (int)vert.size();
  vert.push_back({(int)(at / W_), (int)(at % W_), 2});
  is_v_[at] = 1;
  Edge tail;
  tail.vs = v;
  tail.ve = edge[e_id].ve;
  tail.px.assign(edge[e_id].px.begin() + p + 1, edge[e_id].px.end());
  edge[e_id].px.resize(p);
  edge[e_id].ve = v;
  edge.push_back(std::move(tail));
}

// subdivide_local (lib_image.cc:5953-6022) with its default arguments
// (lib_image.hh:1521-1527): split where a point deviates from the chord by
// more than max(0.05 x chord, 2 px), or where it is seen from either end
// at more than pi/2 from the chord, at the point farthest from the chord.
void Contours::subdivide_local() {
  const double max_angle = (double)1.5707963267948966192313216916397514L, max_dev = 0.05, tol = 2.0;
  std::deque<int> q;
  for (size_t e = 0; e < edge.size(); e++) q.push_back((int)e);
  while (!q.empty()) {
    const int e = q.front();
    q.pop_front();
    const double sx = vert[edge[e].vs].x, sy = vert[edge[e].vs].y;
    const double ex = vert[edge[e].ve].x, ey = vert[edge[e].ve].y;
    const double rx = ex - sx, ry = ey - sy;
    const double len = sqrt(rx * rx + ry * ry), max_dist = max_dev * len;
    size_t pos = 0;
    double best = 0;
    bool cut = false;
    const std::vector<int32_t>& P = edge[e].px;
    for (size_t n = 0; n < P.size(); n++) {
      const double d = dist_seg(P[n], edge[e].vs, edge[e].ve);
      if (d > best) {
        pos = n;
        best = d;
      }
      if (!cut) cut = (d > max_dist) && (d > tol);
      if (!cut) {
        const double px = P[n] / W_, py = P[n] % W_;
        const double ax = px - sx, ay = py - sy, bx = px - ex, by = py - ey;
        const double a0 = acos((ax * rx + ay * ry) / (sqrt(ax * ax + ay * ay) * len));
        const double a1 = acos((bx * -rx + by * -ry) / (sqrt(bx * bx + by * by) * len));
        cut = ((a0 > a1) ? a0 : a1) > max_angle;
      }
    }
    if (cut) {
      split(e, pos);
      q.push_back(e);
      q.push_back((int)edge.size() - 1);
    }
  }
}

// ------------------------------------------------------------ intersections

typedef long long i64;

int orient(i64 ax, i64 ay, i64 bx, i64 by, i64 cx, i64 cy) {  // sign of (b - a) x (c - a)
  const i64 v = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
  return (v > 0) - (v < 0);
}

// lexicographic (x, then y) order of point_2D::compare_to (point_2D.cc:186-190)
bool lex_less(i64 ax, i64 ay, i64 bx, i64 by) { return ax < bx || (ax == bx && ay < by); }

// The reference's quicksort (lang/array.hh:1676-1709), restated so that
// edges with equal keys end in the same order.
template <class Cmp>
void ref_quicksort(std::vector<int>& a, long lo, long hi, const Cmp& cmp) {
  if (lo >= hi) return;
  long pivot = (lo + hi) / 2, i = lo, j = hi;
  for (;;) {
    while (cmp(a[i], a[pivot]) < 0) i++;
    while (cmp(a[j], a[pivot]) > 0) j--;
    if (i < j) {
      std::swap(a[i], a[j]);
      if (pivot == i) pivot = j;
      else if (pivot == j) pivot = i;
      i++;
      j--;
    } else {
      break;
    }
  }
  ref_quicksort(a, lo, j, cmp);
  ref_quicksort(a, j + 1, hi, cmp);
}

}  // namespace

// subdivide_global (lib_image.cc:6138-6326)
bool Contours::subdivide_global() {
  // (1) edges joining the same two vertices: split the less straight one
  {
    auto key_cmp = [&](int a, int b) {
      const int a0 = std::min(edge[a].vs, edge[a].ve), a1 = std::max(edge[a].vs, edge[a].ve);
      const int b0 = std::min(edge[b].vs, edge[b].ve), b1 = std::max(edge[b].vs, edge[b].ve);
      if (a0 != b0) return a0 < b0 ? -1 : 1;
      return a1 < b1 ? -1 : (a1 > b1 ? 1 : 0);
    };
    std::vector<int> order(edge.size());
    for (size_t e = 0; e < edge.size(); e++) order[e] = (int)e;
    if (order.size() > 1) ref_quicksort(order, 0, (long)order.size() - 1, key_cmp);
    size_t prev = 0;
    for (size_t cur = 1; cur < order.size(); cur++) {
      const int ep = order[prev], ec = order[cur];
      if (key_cmp(ep, ec) != 0) {
        prev = cur;
        continue;
      }
      const int va = edge[ep].vs, vb = edge[ep].ve;  // the common end points, as edge ep has them
      const bool can_p = !edge[ep].px.empty(), can_c = !edge[ec].px.empty();
      bool split_prev = false;
      if (can_p && can_c) {
        double dp = 0, dc = 0;
        {
          size_t pos = 0;
          double best = 0;
          for (size_t n = 0; n < edge[ep].px.size(); n++) {
            const double d = dist_seg(edge[ep].px[n], va, vb);
            if (d > best) pos = n, best = d;
          }
          dp = dist_seg(edge[ep].px[pos], va, vb);
        }
        {
          size_t pos = 0;
          double best = 0;
          for (size_t n = 0; n < edge[ec].px.size(); n++) {
            const double d = dist_seg(edge[ec].px[n], va, vb);
            if (d > best) pos = n, best = d;
          }
          dc = dist_seg(edge[ec].px[pos], va, vb);
        }
        split_prev = dp > dc;
      } else if (can_p) {
        split_prev = true;
      } else if (!can_c) {
        return false;  // identical straight edges cannot be separated
      }
      const int e = split_prev ? ep : ec;
      size_t pos = 0;
      double best = 0;
      for (size_t n = 0; n < edge[e].px.size(); n++) {
        const double d = dist_seg(edge[e].px[n], va, vb);
        if (d > best) pos = n, best = d;
      }
      split(e, pos);
      if (split_prev) prev = cur;
    }
  }
  // (2) until no chord crosses another chord's interior
  for (int round = 0;; round++) {
    if (round > 100000) return false;
    const size_t ne = edge.size(), nv = vert.size();
    // cells of 8 x 8 pixels (CSR); a chord is listed in every cell its bounding box covers
    const int CS = 8, GX = (H_ + CS - 1) / CS, GY = (W_ + CS - 1) / CS;
    std::vector<int> cstart((size_t)GX * GY + 1, 0), cell_items;
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) {
        for (size_t c = 0; c < (size_t)GX * GY; c++) cstart[c + 1] += cstart[c];
        cell_items.resize(cstart.back());
      }
      for (size_t e = 0; e < ne; e++) {
        const Vert &a = vert[edge[e].vs], &b = vert[edge[e].ve];
        for (int cx = std::min(a.x, b.x) / CS; cx <= std::max(a.x, b.x) / CS; cx++)
          for (int cy = std::min(a.y, b.y) / CS; cy <= std::max(a.y, b.y) / CS; cy++) {
            const size_t c = (size_t)cx * GY + cy;
            if (pass == 0) cstart[c + 1]++;
            else cell_items[cstart[c]++] = (int)e;
          }
      }
      if (pass == 1)  // restore the starts
        for (size_t c = (size_t)GX * GY; c > 0; c--) cstart[c] = cstart[c - 1];
      if (pass == 1) cstart[0] = 0;
    }
    auto cell_begin = [&](size_t c) { return cell_items.data() + cstart[c]; };
    auto cell_end = [&](size_t c) { return cell_items.data() + cstart[c + 1]; };
    // the marks form a set, so slices of the vertices and of the cell rows
    // are scanned independently (on the host pool when one is given)
    const int nt = par_ ? 16 : 1;
    std::vector<std::vector<uint8_t>> marks(nt, std::vector<uint8_t>(ne, 0));
    std::vector<char> founds(nt, 0);
    auto scan = [&](int t) {
      std::vector<uint8_t>& mark = marks[t];
      char found = 0;
      // (a) a vertex inside a chord's interior: every such chord is split
      for (size_t v = nv * t / nt; v < nv * (t + 1) / nt; v++) {
        const i64 px = vert[v].x, py = vert[v].y;
        const size_t cv = (size_t)(px / CS) * GY + py / CS;
        for (const int* it = cell_begin(cv); it != cell_end(cv); ++it) {
          const int e = *it;
          const int a = edge[e].vs, b = edge[e].ve;
          if (a == (int)v || b == (int)v) continue;
          const i64 ax = vert[a].x, ay = vert[a].y, bx = vert[b].x, by = vert[b].y;
          if (orient(ax, ay, bx, by, px, py) != 0) continue;
          const bool lo_a = lex_less(ax, ay, bx, by);
          const i64 lx = lo_a ? ax : bx, ly = lo_a ? ay : by, ux = lo_a ? bx : ax, uy = lo_a ? by : ay;
          if (lex_less(lx, ly, px, py) && lex_less(px, py, ux, uy)) {
            mark[e] = 1;
            found = 1;
          }
        }
      }
      // (b) two chords crossing at a point that is no vertex: the one whose
      // contour comes nearer the other's chord is kept, the other split.
      // A pair is tested in the cell holding the corner of its boxes' overlap.
      for (int cx = GX * t / nt; cx < GX * (t + 1) / nt; cx++)
        for (int cy = 0; cy < GY; cy++) {
          const int* c = cell_begin((size_t)cx * GY + cy);
          const size_t csz = (size_t)(cell_end((size_t)cx * GY + cy) - c);
          for (size_t i = 0; i < csz; i++)
            for (size_t j = i + 1; j < csz; j++) {
              const int s = std::min(c[i], c[j]), tt = std::max(c[i], c[j]);
              const Vert &a0 = vert[edge[s].vs], &a1 = vert[edge[s].ve];
              const Vert &b0 = vert[edge[tt].vs], &b1 = vert[edge[tt].ve];
              const int lx = std::max(std::min(a0.x, a1.x), std::min(b0.x, b1.x));
              const int ly = std::max(std::min(a0.y, a1.y), std::min(b0.y, b1.y));
              const int hx = std::min(std::max(a0.x, a1.x), std::max(b0.x, b1.x));
              const int hy = std::min(std::max(a0.y, a1.y), std::max(b0.y, b1.y));
              if (lx > hx || ly > hy || lx / CS != cx || ly / CS != cy) continue;
              const i64 ax = a0.x, ay = a0.y, bx = a1.x, by = a1.y;
              const i64 qx = b0.x, qy = b0.y, dx = b1.x, dy = b1.y;
              const int o1 = orient(ax, ay, bx, by, qx, qy), o2 = orient(ax, ay, bx, by, dx, dy);
              const int o3 = orient(qx, qy, dx, dy, ax, ay), o4 = orient(qx, qy, dx, dy, bx, by);
              if (!(o1 * o2 < 0 && o3 * o4 < 0)) continue;  // no proper crossing
              // crossing point = a + (b - a) * num / den, exactly
              const i64 den = (bx - ax) * (dy - qy) - (by - ay) * (dx - qx);
              const i64 num = (qx - ax) * (dy - qy) - (qy - ay) * (dx - qx);
              const i64 X = ax * den + (bx - ax) * num, Y = ay * den + (by - ay) * num;
              if (X % den == 0 && Y % den == 0) {  // an integer crossing point: is it a vertex?
                const i64 xi = X / den, yi = Y / den;
                if (xi >= 0 && xi < H_ && yi >= 0 && yi < W_ && is_v_[(size_t)xi * W_ + yi]) continue;  // under (a)
              }
              found = 1;
              // order the two as the sweep does at the crossing: by the angle of
              // the part left of the sweep line (compute_sweep_line_angle)
              const double fx = (double)X / (double)den, fy = (double)Y / (double)den;
              auto ang = [&](int e) {
                const Vert &p = vert[edge[e].vs], &q = vert[edge[e].ve];
                const Vert& lo = lex_less(p.x, p.y, q.x, q.y) ? p : q;
                return atan2(fx - lo.x, fy - lo.y);
              };
              const double g0 = ang(s), g1 = ang(tt);
              int ea = s, eb = tt;
              if (g1 < g0) std::swap(ea, eb);
              if (edge[ea].px.empty()) {
                mark[eb] = 1;
                continue;
              }
              if (edge[eb].px.empty()) {
                mark[ea] = 1;
                continue;
              }
              auto closest = [&](int e, int other) {  // find_contour_point_closest_to_segment
                const int p = edge[other].vs, q = edge[other].ve;
                double best = dist_seg(edge[e].px[0], p, q);
                size_t pos = 0;
                for (size_t n = 1; n < edge[e].px.size(); n++) {
                  const double d = dist_seg(edge[e].px[n], p, q);
                  if (d < best) pos = n, best = d;
                }
                return dist_seg(edge[e].px[pos], p, q);
              };
              if (closest(ea, eb) < closest(eb, ea)) mark[eb] = 1;
              else mark[ea] = 1;
            }
        }
      founds[t] = found;
    };
    if (par_) (*par_)(nt, scan);
    else scan(0);
    bool found = false;
    std::vector<uint8_t>& mark = marks[0];
    for (int t = 0; t < nt; t++) {
      found = found || founds[t];
      if (t)
        for (size_t e = 0; e < ne; e++) mark[e] |= marks[t][e];
    }
    if (!found) break;
    for (size_t e = 0; e < ne; e++) {
      if (!mark[e]) continue;
      if (edge[e].px.empty()) return false;
      split((int)e, farthest(edge[e]));
    }
  }
  return true;
}

// Contour fitting of a 0/1 watershed-arc map (MexContourSides): vertices,
// the non-completion edges and their interior pixels.  Returns false where
// the reference's subdivision throws, in which case MexContourSides returns
// no contours and nothing is painted.
bool fit_contours(const uint8_t* bw, int H, int W, FitResult& out, const ParFor* par) {
  Contours c(bw, H, W, par);
  c.subdivide_local();
  const bool ok = c.subdivide_global();
  out.vx.clear();
  out.vy.clear();
  out.es.clear();
  out.ee.clear();
  out.off.assign(1, 0);
  out.px.clear();
  if (!ok) return false;
  for (const Vert& v : c.vert) {
    out.vx.push_back(v.x);
    out.vy.push_back(v.y);
  }
  for (const Edge& e : c.edge) {
    out.es.push_back(e.vs);
    out.ee.push_back(e.ve);
    out.px.insert(out.px.end(), e.px.begin(), e.px.end());
    out.off.push_back((int32_t)out.px.size());
  }
  return true;
}

// The orientation bin of an edge from its end points
// (contours2ucm.cpp:336-372): the chord's angle in float degrees, binned
// into 8 sectors of 22.5 degrees centred on 90, 67.5, ..., -67.5.
int edge_orientation(int x1, int y1, int x2, int y2) {
  float ang = (float)(M_PI / 2);
  if (y1 != y2) ang = (float)atan((x1 - x2) * 1.0 / (y1 - y2));
  const float deg = (float)(ang * 180 / M_PI);
  int o = 0;
  if (deg < -78.75 || deg >= 78.75) o = 1;
  else if (deg < 78.75 && deg >= 56.25) o = 2;
  else if (deg < 56.25 && deg >= 33.75) o = 3;
  else if (deg < 33.75 && deg >= 11.25) o = 4;
  else if (deg < 11.25 && deg >= -11.25) o = 5;
  else if (deg < -11.25 && deg >= -33.75) o = 6;
  else if (deg < -33.75 && deg >= -56.25) o = 7;
  else if (deg < -56.25 && deg >= -78.75) o = 8;
  return o - 1;
}

// ------------------------------------------------------------ mean-pb merge

namespace {

// One adjacent pair of regions, shared by both sides (the reference keeps a
// copy in each region's neighbour map; both copies are always updated together).
struct Pair {
  double energy = 0, total = 0, length = 0;
  double pushed = -1.0;      // energy and first region of the pair's last queue entry
  double raise = -INFINITY;  // pending raise of the boundary list
  int first = -1;
  int head = -1, tail = -1;  // the pair's boundary coordinates: a linked list of nodes
};

// open-addressing map from an unordered region pair to its Pair index
class PairTable {
 public:
  explicit PairTable(size_t expect) {
    size_t c = 16;
    while (c < 2 * expect) c <<= 1;
    key_.assign(c, kEmpty);
    val_.assign(c, -1);
  }
  // index of pair {a, b}, or -1; with create, a new pair is appended to `pairs`
  int find(int a, int b, std::vector<Pair>* pairs) {
    const uint64_t k = a < b ? ((uint64_t)(uint32_t)a << 32) | (uint32_t)b : ((uint64_t)(uint32_t)b << 32) | (uint32_t)a;
    size_t h = (size_t)((k * 0x9E3779B97F4A7C15ull) >> 20) & (key_.size() - 1);
    for (;; h = (h + 1) & (key_.size() - 1)) {
      if (key_[h] == k) return val_[h];
      if (key_[h] == kEmpty) break;
    }
    if (!pairs) return -1;
    key_[h] = k;
    val_[h] = (int)pairs->size();
    pairs->emplace_back();
    if (++used_ * 2 > key_.size()) grow();
    return (int)pairs->size() - 1;
  }

 private:
  static constexpr uint64_t kEmpty = ~0ull;
  std::vector<uint64_t> key_;
  std::vector<int> val_;
  size_t used_ = 0;
  void grow() {
    std::vector<uint64_t> k2(key_.size() * 2, kEmpty);
    std::vector<int> v2(key_.size() * 2, -1);
    for (size_t i = 0; i < key_.size(); i++) {
      if (key_[i] == kEmpty) continue;
      size_t h = (size_t)((key_[i] * 0x9E3779B97F4A7C15ull) >> 20) & (k2.size() - 1);
      while (k2[h] != kEmpty) h = (h + 1) & (k2.size() - 1);
      k2[h] = key_[i];
      v2[h] = val_[i];
    }
    key_.swap(k2);
    val_.swap(v2);
  }
};

struct Entry {
  double energy;
  int r1, r2;
  int pair;  // index of the pair {r1, r2}, fixed while both regions live
  bool operator>(const Entry& o) const {  // the reference's (energy, region1, region2) order
    if (energy != o.energy) return energy > o.energy;
    if (r1 != o.r1) return r1 > o.r1;
    return r2 > o.r2;
  }
};

}  // namespace

// ComputeUcm + CompleteContourMap (ucm_mean_pb.cpp:230-398) on the
// (2H+1) x (2W+1) grid, row-major here (the reference stores it
// column-major; the grid coordinates are the same).  lb: local boundary
// strengths; part: H x W region ids 0..n-1 (negative ids are skipped).
//
// The reference sums each pair's boundary strengths in column-major order
// of the coordinates; the grid is walked in that order here.
//
// The reference walks the son's whole boundary on every merge, raising the
// map to the merge's saliency.  Here each pair of regions keeps one linked
// list of its boundary coordinates: the son-father list takes the saliency
// when it closes, the son's other lists are joined to the father's in O(1).
// With saliencies that never decrease -- the reference stops
// being defined otherwise: it frees its arrays and carries on -- every
// coordinate ends at the saliency of the merge that joins its two sides,
// as there.
//
// After every merge the reference pushes (d, k, father) for each neighbour
// k of the father.  A push identical to the pair's last entry still in the
// queue changes nothing (the copy pops right after it and fails the energy
// or label check), so only pairs whose energy changed (the son's former
// neighbours) or whose last entry had the other order are pushed; the pop
// order, and so every merge, is the reference's.
template <class Real>
static void merge_impl(const Real* lb, const int32_t* part, int H, int W, double* ucm) {
  const int GW = 2 * W + 1, GH = 2 * H + 1;
  int n = 0;
  for (size_t p = 0; p < (size_t)H * W; p++) n = std::max(n, part[p] + 1);
  for (size_t i = 0; i < (size_t)GH * GW; i++) ucm[i] = 0.0;
  if (n <= 0) return;
  std::vector<int> up(n);  // union-find; a root is a live region, its id the father's
  for (int c = 0; c < n; c++) up[c] = c;
  std::vector<Pair> P;
  P.reserve((size_t)n * 8);
  PairTable T((size_t)n * 8);
  // each pair's boundary coordinates as a linked list of nodes (coordinate,
  // next); lists are joined in O(1) when their pairs join
  std::vector<int32_t> node_coord, node_next;
  node_coord.reserve((size_t)H * W);
  node_next.reserve((size_t)H * W);
  std::vector<std::vector<std::pair<int, int>>> nb(n), pending(n);  // (neighbour, pair index)
  // Boundary coordinates in the reference's column-major order, so that
  // each pair's sum runs in that order: grid column 2y holds the (odd, even)
  // coordinates between horizontal neighbours (x, y-1), (x, y); grid column
  // 2y+1 the (even, odd) ones between vertical neighbours (x-1, y), (x, y).
  // A transposed copy of the labels makes the walk sequential.
  std::vector<int32_t> tr((size_t)H * W);
  for (int x0 = 0; x0 < H; x0 += 32)
    for (int y0 = 0; y0 < W; y0 += 32)
      for (int x = x0; x < std::min(H, x0 + 32); x++)
        for (int y = y0; y < std::min(W, y0 + 32); y++) tr[(size_t)y * H + x] = part[(size_t)x * W + y];
  int last_a = -1, last_b = -1, last_p = -1;  // runs repeat a pair
  auto add = [&](int a, int b, int32_t coord) {
    if (a < 0 || b < 0 || a == b) return;
    int pi;
    if (a == last_a && b == last_b) {
      pi = last_p;
    } else {
      const size_t np = P.size();
      pi = T.find(a, b, &P);
      if (P.size() != np) {
        nb[a].push_back({b, pi});
        nb[b].push_back({a, pi});
      }
      last_a = a;
      last_b = b;
      last_p = pi;
    }
    Pair& pr = P[pi];
    const int32_t nd = (int32_t)node_coord.size();
    node_coord.push_back(coord);
    node_next.push_back(-1);
    if (pr.tail < 0) pr.head = nd;
    else node_next[pr.tail] = nd;
    pr.tail = nd;
    pr.total += (double)lb[coord];
    pr.length += 1.0;
  };
  for (int y = 0; y < W; y++) {
    const int32_t* cur = tr.data() + (size_t)y * H;
    if (y > 0) {
      const int32_t* left = cur - H;
      for (int x = 0; x < H; x++) add(left[x], cur[x], (2 * x + 1) * GW + 2 * y);
    }
    for (int x = 1; x < H; x++) add(cur[x - 1], cur[x], (2 * x) * GW + 2 * y + 1);
  }
  std::vector<int32_t>().swap(tr);
  // a 4-ary min-heap in the reference's (energy, region1, region2) order
  std::vector<Entry> heap;
  heap.reserve(P.size() * 2);
  auto before = [](const Entry& a, const Entry& b) { return b > a; };
  auto heap_push = [&](const Entry& e) {
    size_t i = heap.size();
    heap.push_back(e);
    while (i > 0) {
      const size_t par = (i - 1) / 4;
      if (!before(heap[i], heap[par])) break;
      std::swap(heap[i], heap[par]);
      i = par;
    }
  };
  auto heap_pop = [&]() {
    const Entry top = heap[0];
    heap[0] = heap.back();
    heap.pop_back();
    const size_t sz = heap.size();
    size_t i = 0;
    for (;;) {
      const size_t c0 = 4 * i + 1;
      if (c0 >= sz) break;
      size_t best = c0;
      const size_t ce = std::min(c0 + 4, sz);
      for (size_t c = c0 + 1; c < ce; c++)
        if (before(heap[c], heap[best])) best = c;
      if (!before(heap[best], heap[i])) break;
      std::swap(heap[i], heap[best]);
      i = best;
    }
    return top;
  };
  auto push = [&](int pi, double d, int a, int b) {  // entry (d, a, b); b is the region that pushes
    heap_push({d, a, b, pi});
    P[pi].pushed = d;
    P[pi].first = a;
    pending[a].push_back({b, pi});
  };
  for (int c = 0; c < n; c++)
    for (const auto& kp : nb[c])
      if (kp.first > c) {
        Pair& pr = P[kp.second];
        pr.energy = pr.total / pr.length;
        push(kp.second, pr.energy, c, kp.first);
      }
  auto flush = [&](Pair& pr, double extra) {
    const double r = std::max(pr.raise, extra);
    for (int32_t k = pr.head; k >= 0; k = node_next[k])
      if (ucm[node_coord[k]] < r) ucm[node_coord[k]] = r;
    pr.head = pr.tail = -1;
  };
  std::vector<std::pair<int, int>> touched;
  while (!heap.empty()) {
    const Entry m = heap_pop();
    if (up[m.r1] != m.r1 || up[m.r2] != m.r2) continue;
    const int ci = m.pair;  // both regions live, so the pair is the one pushed
    if (m.energy != P[ci].energy) continue;
    const double saliency = P[ci].total / P[ci].length;
    const int son = std::min(m.r1, m.r2), father = std::max(m.r1, m.r2);
    flush(P[ci], saliency);  // the son-father boundary becomes interior
    up[son] = father;
    // the son's live neighbours other than the father join the father's
    touched.clear();
    for (const auto& kp : nb[son]) {
      const int k = kp.first, si = kp.second;
      if (up[k] != k || k == father) continue;
      const size_t np = P.size();
      const int fi = T.find(father, k, &P);
      if (P.size() != np) {
        nb[father].push_back({k, fi});
        nb[k].push_back({father, fi});
      }
      Pair &s = P[si], &f = P[fi];
      f.total += s.total;
      f.length += s.length;
      // the son's side is raised to this saliency; with saliencies that
      // never decrease only the raise at closing shows, so lists join as
      // they are and keep the larger pending raise
      if (s.head >= 0) {
        if (f.head < 0) f.head = s.head;
        else node_next[f.tail] = s.head;
        f.tail = s.tail;
        f.raise = std::max(f.raise, std::max(s.raise, saliency));
        s.head = s.tail = -1;
      }
      touched.push_back({k, fi});
    }
    std::vector<std::pair<int, int>>().swap(nb[son]);
    std::vector<std::pair<int, int>>().swap(pending[son]);
    for (const auto& kp : pending[father]) touched.push_back(kp);
    std::vector<std::pair<int, int>>().swap(pending[father]);
    for (const auto& kp : touched) {
      const int k = kp.first;
      if (up[k] != k || k == father) continue;
      Pair& f = P[kp.second];
      const double d = f.total / f.length;
      f.energy = d;
      if (!(f.pushed == d && f.first == k)) push(kp.second, d, k, father);
    }
    if (nb[father].size() > 64) {  // drop merged-away neighbours now and then
      std::vector<std::pair<int, int>>& v = nb[father];
      size_t w = 0;
      for (size_t r = 0; r < v.size(); r++)
        if (up[v[r].first] == v[r].first) v[w++] = v[r];
      v.resize(w);
    }
  }
  for (Pair& pr : P)  // boundaries never closed (a split adjacency graph)
    if (pr.head >= 0) flush(pr, -INFINITY);
  // CompleteContourMap: every even-even grid point takes the largest of its
  // four neighbours (starting from 0)
  for (int x = 0; x < GH; x += 2)
    for (int y = 0; y < GW; y += 2) {
      double m = 0.0;
      if (x + 1 < GH && m < ucm[(size_t)(x + 1) * GW + y]) m = ucm[(size_t)(x + 1) * GW + y];
      if (y + 1 < GW && m < ucm[(size_t)x * GW + y + 1]) m = ucm[(size_t)x * GW + y + 1];
      if (x >= 1 && m < ucm[(size_t)(x - 1) * GW + y]) m = ucm[(size_t)(x - 1) * GW + y];
      if (y >= 1 && m < ucm[(size_t)x * GW + y - 1]) m = ucm[(size_t)x * GW + y - 1];
      ucm[(size_t)x * GW + y] = m;
    }
}

void mean_pb_merge(const double* lb, const int32_t* part, int H, int W, double* ucm) {
  merge_impl(lb, part, H, W, ucm);
}

// the same on float strengths (as the device grid holds them; widened exactly)
void mean_pb_merge(const float* lb, const int32_t* part, int H, int W, double* ucm) {
  merge_impl(lb, part, H, W, ucm);
}

// NormalizeOutput (contours2ucm.cpp:191-249): logistic calibration of the
// mean boundary strength, rescaled and clipped to [0, 1].
// Most of the grid is 0 and boundary runs repeat one value, so a value
// equal to the previous one reuses its result (the same arithmetic either way).
void normalize(double* u, size_t n) {
  auto f = [](double x) {
    const double z = 0.0 + 1.0 * -2.7487 + x * 11.1189;
    double v = 1.0 / (1.0 + exp(-z));
    v = (v - 0.0602) / (1.0 - 0.0602);
    return std::min(1.0, std::max(0.0, v));
  };
  const double f0 = f(0.0);
  double last_in = 0.0, last_out = f0;
  for (size_t i = 0; i < n; i++) {
    const double x = u[i];
    if (x == 0.0) {
      u[i] = f0;
    } else if (x == last_in) {
      u[i] = last_out;
    } else {
      last_in = x;
      last_out = f(x);
      u[i] = last_out;
    }
  }
}

}  // namespace ucm
}  // namespace gpb
