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
// priority order (energy, region1, region2), the same running sums in the
// same order, so ties break exactly as there.  Boundaries are kept as
// linked lists of segments joined in O(1), pushes that cannot change the
// pop order are left out, and queue entries of merged-away regions are
// dropped in bulk; none of this changes a merge or a value of the map.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <deque>
#include <functional>
#include <new>
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
  const uint8_t* bw_ = nullptr;  // the arcs (non-zero); 8-neighbours of an arc pixel that are
                                 // arcs are in its component
  std::vector<uint8_t> is_v_, is_e_;
  std::vector<int32_t> assign_;

  bool arc(int x, int y) const { return bw_[(size_t)x * W_ + y] != 0; }
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
  bw_ = bw;
  is_v_.assign(N, 0);
  is_e_.assign(N, 0);
  assign_.assign(N, 0);
  // One raster pass: the pattern vertices in row-major order, and the
  // 8-connected components as provisional labels (two rows at a time) whose
  // equivalences go to a union-find with the smallest label as root, as in
  // components8; per provisional label whether it holds a vertex and its
  // last pixel.
  std::vector<uint32_t> par(1, 0), rows(2 * (size_t)W_, 0);
  std::vector<uint8_t> pv(1, 0);
  std::vector<size_t> plast(1, 0);
  auto unite = [&](uint32_t a, uint32_t b) {
    a = find_root(par, a);
    b = find_root(par, b);
    if (a == b) return;
    if (a < b) std::swap(a, b);
    par[a] = b;
  };
  for (int x = 0; x < H_; x++) {
    const uint8_t* r = bw + (size_t)x * W_;
    const uint8_t* rn = x + 1 < H_ ? r + W_ : nullptr;  // the reference's e side
    const uint8_t* rp = x > 0 ? r - W_ : nullptr;       // w side
    uint32_t* l = rows.data() + (size_t)(x & 1) * W_;
    const uint32_t* u = x > 0 ? rows.data() + (size_t)((x + 1) & 1) * W_ : nullptr;
    for (int y = 0; y < W_; y++) {
      if (!r[y]) {
        l[y] = 0;
        continue;
      }
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
        if (y + 1 < W_) see(u[y + 1]);
      }
      if (!m) {
        m = (uint32_t)par.size();
        par.push_back(m);
        pv.push_back(0);
        plast.push_back(0);
      }
      l[y] = m;
      const bool hn = y + 1 < W_, hs = y > 0;
      unsigned k = 0;
      if (hn && r[y + 1]) k |= BN;
      if (hs && r[y - 1]) k |= BS;
      if (rn && rn[y]) k |= BE;
      if (rp && rp[y]) k |= BW;
      if (hn && rn && rn[y + 1]) k |= BNE;
      if (hn && rp && rp[y + 1]) k |= BNW;
      if (hs && rn && rn[y - 1]) k |= BSE;
      if (hs && rp && rp[y - 1]) k |= BSW;
      if (kVertex.v[k]) {
        add_vertex(x, y);
        pv[m] = 1;
      }
      plast[m] = (size_t)x * W_ + y;
    }
  }
  // each component (a root, in the order of the components' first pixels)
  // without a vertex is a closed loop: its last pixel becomes a vertex
  std::vector<uint8_t> rv(par.size(), 0);
  std::vector<size_t> rlast(par.size(), 0);
  for (uint32_t v = 1; v < par.size(); v++) {
    const uint32_t r = find_root(par, v);
    rv[r] |= pv[v];
    rlast[r] = std::max(rlast[r], plast[v]);
  }
  for (uint32_t v = 1; v < par.size(); v++)
    if (par[v] == v && !rv[v]) add_vertex((int)(rlast[v] / W_), (int)(rlast[v] % W_));
  for (size_t v_id = 0; v_id < vert.size(); v_id++) {  // grows while tracing
    const int vx = vert[v_id].x, vy = vert[v_id].y;
    int qx[8], qy[8], nq = 0;
    const int x0 = vx > 0 ? vx - 1 : vx + 1, y0 = vy > 0 ? vy - 1 : vy + 1;
    for (int x = x0; x <= vx + 1 && x < H_; x += 2)
      if (arc(x, vy)) qx[nq] = x, qy[nq++] = vy;
    for (int y = y0; y <= vy + 1 && y < W_; y += 2)
      if (arc(vx, y)) qx[nq] = vx, qy[nq++] = y;
    for (int x = x0; x <= vx + 1 && x < H_; x += 2)
      for (int y = y0; y <= vy + 1 && y < W_; y += 2)
        if (arc(x, y) && !arc(vx, y) && !arc(x, vy)) qx[nq] = x, qy[nq++] = y;
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
    auto av = [&](bool has, size_t j) { return has && bw_[j] && !is_e_[j]; };
    const size_t in = i + 1, is = i - 1, ie = i + W_, iw = i - W_;
    // each neighbour's state is read when its rule comes up (nothing
    // changes between the rules)
    const bool an = av(hn, in);
    if (an && !is_v_[in]) { y++; continue; }
    const bool as = av(hs, is);
    if (as && !is_v_[is]) { y--; continue; }
    const bool ae = av(he, ie);
    if (ae && !is_v_[ie]) { x++; continue; }
    const bool aw = av(hw, iw);
    if (aw && !is_v_[iw]) { x--; continue; }
    if (an) { y++; break; }
    if (as) { y--; break; }
    if (ae) { x++; break; }
    if (aw) { x--; break; }
    const bool ane = av(hn && he, ie + 1);
    if (ane && !is_v_[ie + 1]) { x++; y++; continue; }
    const bool anw = av(hn && hw, iw + 1);
    if (anw && !is_v_[iw + 1]) { x--; y++; continue; }
    const bool ase = av(hs && he, ie - 1);
    if (ase && !is_v_[ie - 1]) { x++; y--; continue; }
    const bool asw = av(hs && hw, iw - 1);
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
//
// The reference's angle test, acos(dot / (|a| |r|)) > pi/2 (the double
// nearest), is the sign of dot here: on the integer grid dot is an exact
// integer and |a| |r| < 2^33, so a non-zero dot puts the cosine at least
// 2^-33 from 0, where acos is many roundings away from pi/2 on either
// side; dot == 0 gives acos(0) = pi/2, not above it; a chord of length 0
// gives NaN, which never cuts.
void Contours::subdivide_local() {
  const double max_dev = 0.05, tol = 2.0;
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
        cut = len > 0 && ((ax * rx + ay * ry) < 0 || (bx * -rx + by * -ry) < 0);
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
    // each edge's (smaller, larger) end vertex as one number, taken before
    // the splits below: an edge split there is not compared again
    std::vector<uint64_t> key(edge.size());
    for (size_t e = 0; e < edge.size(); e++)
      key[e] = ((uint64_t)(uint32_t)std::min(edge[e].vs, edge[e].ve) << 32) |
               (uint32_t)std::max(edge[e].vs, edge[e].ve);
    auto key_cmp = [&](int a, int b) { return key[a] < key[b] ? -1 : (key[a] > key[b] ? 1 : 0); };
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
  // (2) until no chord crosses another chord's interior.  After the first
  // round only pairs with a chord split or added in the previous round, or
  // with a vertex added there, are tested: every other pair was tested with
  // the same end points and gave no split (a finding splits one of its two).
  std::vector<uint8_t> dirty(edge.size(), 1);  // chords changed since the last round
  size_t v_new = 0;                           // vertices from v_new on were added since the last round
  for (int round = 0;; round++) {
    if (round > 100000) return false;
    const size_t ne = edge.size(), nv = vert.size();
    // cells of 8 x 8 pixels (CSR); a chord is listed in every cell its bounding box covers
    const int CS = 8, GX = (H_ + CS - 1) / CS, GY = (W_ + CS - 1) / CS;
    std::vector<int> cstart((size_t)GX * GY + 1, 0), cell_items;
    std::vector<uint8_t> cell_dirty((size_t)GX * GY, 0);  // a changed chord covers the cell
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
            if (pass == 0 && dirty[e]) cell_dirty[c] = 1;
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
        const bool v_changed = v >= v_new;
        if (!v_changed && !cell_dirty[cv]) continue;
        for (const int* it = cell_begin(cv); it != cell_end(cv); ++it) {
          const int e = *it;
          if (!v_changed && !dirty[e]) continue;
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
          if (!cell_dirty[(size_t)cx * GY + cy]) continue;
          const int* c = cell_begin((size_t)cx * GY + cy);
          const size_t csz = (size_t)(cell_end((size_t)cx * GY + cy) - c);
          for (size_t i = 0; i < csz; i++)
            for (size_t j = i + 1; j < csz; j++) {
              if (!dirty[c[i]] && !dirty[c[j]]) continue;
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
    std::fill(dirty.begin(), dirty.end(), 0);
    for (size_t e = 0; e < ne; e++) {
      if (!mark[e]) continue;
      if (edge[e].px.empty()) return false;
      split((int)e, farthest(edge[e]));
      dirty[e] = 1;
    }
    dirty.resize(edge.size(), 1);  // the split-off tails
    v_new = nv;
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
// copy in each region's neighbour map; both copies are always updated
// together).  Its energy is total / length, recomputed where needed.
struct Pair {
  double total = 0;
  double pushed = -1.0;      // energy and first region of the pair's last queue entry
  double raise = -INFINITY;  // pending raise of the boundary list
  int32_t length = 0;        // boundary elements
  int first = -1;
  int head = -1, tail = -1;  // the pair's boundary: a linked list of segments
  double energy() const { return total / (double)length; }
};

// open-addressing map from an unordered region pair to its Pair index
class PairTable {
 public:
  explicit PairTable(size_t expect) {
    size_t c = 16;
    while (c < 2 * expect) c <<= 1;
    slot_.assign(c, Slot{kEmpty, -1});
  }
  static uint64_t key(int a, int b) {
    return a < b ? ((uint64_t)(uint32_t)a << 32) | (uint32_t)b : ((uint64_t)(uint32_t)b << 32) | (uint32_t)a;
  }
  void insert(uint64_t k, int v) {
    const size_t mask = slot_.size() - 1;
    size_t h = hash(k) & mask;
    while (slot_[h].key != kEmpty) h = (h + 1) & mask;
    slot_[h] = Slot{k, v};
    if (++used_ * 2 > slot_.size()) grow();
  }
  // index of pair {a, b}; a pair not yet in the map gets index `fresh`
  // (returned as -fresh - 1, so that the caller can tell)
  int find_or_add(uint64_t k, int fresh) {
    const size_t mask = slot_.size() - 1;
    size_t h = hash(k) & mask;
    for (;; h = (h + 1) & mask) {
      if (slot_[h].key == k) return slot_[h].val;
      if (slot_[h].key == kEmpty) break;
    }
    slot_[h] = Slot{k, fresh};
    if (++used_ * 2 > slot_.size()) grow();
    return -fresh - 1;
  }

 private:
  struct Slot {
    uint64_t key;
    int32_t val;
  };
  static constexpr uint64_t kEmpty = ~0ull;
  std::vector<Slot> slot_;
  size_t used_ = 0;
  static size_t hash(uint64_t k) { return (size_t)((k * 0x9E3779B97F4A7C15ull) >> 20); }
  void grow() {
    std::vector<Slot> s2(slot_.size() * 2, Slot{kEmpty, -1});
    const size_t mask = s2.size() - 1;
    for (const Slot& e : slot_) {
      if (e.key == kEmpty) continue;
      size_t h = hash(e.key) & mask;
      while (s2[h].key != kEmpty) h = (h + 1) & mask;
      s2[h] = e;
    }
    slot_.swap(s2);
  }
};

// A queue entry (energy, region1, region2) in two words: the energy's bits
// mapped to an unsigned order (negative values reversed, -0 taken as +0),
// and region1 beside the pair's index.  Region2 is the pair's other region,
// (region1 ^ (both regions' xor)); it decides only between entries of equal
// energy and region1.
struct Entry {
  uint64_t hi, lo;  // lo: region1 << 32 | pair
};

inline uint64_t energy_key(double d) {
  if (d == 0.0) d = 0.0;
  uint64_t b;
  memcpy(&b, &d, 8);
  return (b >> 63) ? ~b : b | (1ull << 63);
}

inline double key_energy(uint64_t k) {
  const uint64_t b = (k >> 63) ? k & ~(1ull << 63) : ~k;
  double d;
  memcpy(&d, &b, 8);
  return d;
}

// a 4-ary min-heap of entries in the reference's (energy, region1, region2)
// order; node i sits at slot i + 3 of a 64-byte aligned buffer, so that the
// four children of a node share one cache line
class Queue {
 public:
  explicit Queue(const std::vector<int32_t>& pair_xor) : xr_(pair_xor) {}
  ~Queue() { free(buf_); }
  Queue(const Queue&) = delete;
  Queue& operator=(const Queue&) = delete;
  bool empty() const { return n_ == 0; }
  size_t size() const { return n_; }
  void push(const Entry& e) {
    if (n_ == cap_) grow();
    size_t i = n_++;
    while (i > 0) {
      const size_t par = (i - 1) >> 2;
      if (!before(e, at(par))) break;
      at(i) = at(par);
      i = par;
    }
    at(i) = e;
  }
  // entries appended unordered, then ordered at once (bottom-up)
  void append(const Entry& e) {
    if (n_ == cap_) grow();
    at(n_++) = e;
  }
  void heapify() {
    if (n_ < 2) return;
    for (size_t i = (n_ - 2) >> 2;; i--) {
      down(i, at(i));
      if (i == 0) break;
    }
  }
  // drops the entries that keep() rejects, then reorders the rest
  template <class Keep>
  void filter(Keep keep) {
    size_t w = 0;
    for (size_t i = 0; i < n_; i++) {
      const Entry e = at(i);
      if (keep(e)) at(w++) = e;
    }
    n_ = w;
    heapify();
  }
  Entry pop() {
    const Entry top = at(0);
    n_--;
    if (n_ > 0) down(0, at(n_));
    return top;
  }

 private:
  const std::vector<int32_t>& xr_;
  Entry* buf_ = nullptr;
  size_t n_ = 0, cap_ = 0;
  Entry& at(size_t i) { return buf_[i + 3]; }
  bool before(const Entry& a, const Entry& b) const {
    if (a.hi != b.hi) return a.hi < b.hi;
    const uint32_t r1a = (uint32_t)(a.lo >> 32), r1b = (uint32_t)(b.lo >> 32);
    if (r1a != r1b) return r1a < r1b;
    return ((uint32_t)xr_[(uint32_t)a.lo] ^ r1a) < ((uint32_t)xr_[(uint32_t)b.lo] ^ r1b);
  }
  void grow() {
    const size_t cap = cap_ ? 2 * cap_ : 1024;
    Entry* nb = (Entry*)aligned_alloc(64, ((cap + 4) * sizeof(Entry) + 63) / 64 * 64);
    if (!nb) throw std::bad_alloc();
    if (buf_) memcpy(nb + 3, buf_ + 3, n_ * sizeof(Entry));
    free(buf_);
    buf_ = nb;
    cap_ = cap;
  }
  // place e at the hole i, moving smaller children up
  void down(size_t i, const Entry e) {
    for (;;) {
      const size_t c0 = 4 * i + 1;
      if (c0 >= n_) break;
      size_t best = c0;
      if (c0 + 3 < n_) {
        const size_t b01 = before(at(c0 + 1), at(c0)) ? c0 + 1 : c0;
        const size_t b23 = before(at(c0 + 3), at(c0 + 2)) ? c0 + 3 : c0 + 2;
        best = before(at(b23), at(b01)) ? b23 : b01;
      } else {
        for (size_t c = c0 + 1; c < n_; c++)
          if (before(at(c), at(best))) best = c;
      }
      if (!before(at(best), e)) break;
      at(i) = at(best);
      i = best;
    }
    at(i) = e;
  }
};

}  // namespace

// Parts of the merge's setup and output split into chunks: run on the host
// pool when one is given, in order otherwise.  Chunks are processed so that
// the result does not depend on their number.
constexpr int kChunks = 16;

static void for_chunks(const ParFor* par, int nt, const std::function<void(int)>& f) {
  if (par && nt > 1) (*par)(nt, f);
  else
    for (int t = 0; t < nt; t++) f(t);
}

// Stable counting sort of the sequence in[0..ne) (or 0..ne-1 without in) by
// key[e] < nkey: place(q, e) puts element e at position q.  Each chunk counts
// its keys; positions are handed out key by key, chunk by chunk, so equal
// keys keep their order.
template <class Place>
static void count_sort(const ParFor* par, int32_t ne, int nkey, const int32_t* key, const int32_t* in, Place place) {
  const int nt = par ? kChunks : 1;
  std::vector<int32_t> off((size_t)nt * nkey);
  auto lo = [&](int t) { return (int32_t)((int64_t)ne * t / nt); };
  for_chunks(par, nt, [&](int t) {
    int32_t* h = off.data() + (size_t)t * nkey;
    std::fill(h, h + nkey, 0);
    for (int32_t i = lo(t); i < lo(t + 1); i++) h[key[in ? in[i] : i]]++;
  });
  int32_t run = 0;
  for (int k = 0; k < nkey; k++)
    for (int t = 0; t < nt; t++) {
      int32_t& o = off[(size_t)t * nkey + k];
      const int32_t c = o;
      o = run;
      run += c;
    }
  for_chunks(par, nt, [&](int t) {
    int32_t* o = off.data() + (size_t)t * nkey;
    for (int32_t i = lo(t); i < lo(t + 1); i++) {
      const int32_t e = in ? in[i] : i;
      place(o[key[e]]++, e);
    }
  });
}

// ComputeUcm + CompleteContourMap (ucm_mean_pb.cpp:230-398) on the
// (2H+1) x (2W+1) grid, row-major here (the reference stores it
// column-major; the grid coordinates are the same).  lb: local boundary
// strengths; part: H x W region ids 0..n-1 (negative ids are skipped).
//
// The boundary elements (grid points between two 4-adjacent pixels of
// different regions) are numbered in the reference's column-major order:
// grid column 2y holds the (odd, even) points between horizontal
// neighbours (x, y-1), (x, y); grid column 2y+1 the (even, odd) ones
// between vertical neighbours (x-1, y), (x, y).  A stable two-pass
// counting sort by (smaller id, larger id) groups them by pair, each
// pair's elements still in that order, so every pair's sum of strengths
// runs in the reference's order.  The elements of one initial pair form a
// segment.
//
// The reference walks the son's whole boundary on every merge, raising the
// map to the merge's saliency.  Here each pair of regions keeps one linked
// list of segments: the son-father list takes the saliency when it
// closes, the son's other lists are joined to the father's in O(1).  With
// saliencies that never decrease -- the reference stops being defined
// otherwise: it frees its arrays and carries on -- every element ends at
// the saliency of the merge that joins its two sides, as there.  Each
// segment is closed exactly once, so its value is recorded per segment and
// written to the map at the end, in element order.
//
// After every merge the reference pushes (d, k, father) for each neighbour
// k of the father.  A push identical to the pair's last entry still in the
// queue changes nothing (the copy pops right after it and fails the energy
// or label check), so only pairs whose energy changed (the son's former
// neighbours) or whose last entry had the other order are pushed; the pop
// order, and so every merge, is the reference's.
//
// Out: the grid index of every boundary element, in row-major order, and
// the value it takes (elements are the only non-zero points before
// CompleteContourMap).
template <class Real>
static void merge_impl(const Real* lb, const int32_t* part, int H, int W, std::vector<int32_t>& ec,
                       std::vector<double>& eval, const ParFor* par) {
  const int GW = 2 * W + 1;
  ec.clear();
  eval.clear();
  // boundary elements in row-major grid order: regions (a < b), grid index,
  // grid column and strength.  Bands of pixel rows count theirs, then fill
  // their slices of the arrays.
  const int nband = par ? std::min(kChunks, H) : 1;
  auto band_lo = [&](int t) { return (int)((int64_t)H * t / nband); };
  std::vector<int64_t> bstart(nband + 1, 0);
  std::vector<int> bmax(nband, 0);
  // f(a, b, grid index, grid column) for each boundary element of pixel row x
  auto scan_row = [&](int x, auto&& f) {
    const int32_t* row = part + (size_t)x * W;
    if (x > 0) {  // grid row 2x: (even, odd) points between pixel rows x-1 and x
      const int32_t* above = row - W;
      const int32_t base = 2 * x * GW + 1;
      for (int y = 0; y < W; y++)
        if (above[y] != row[y] && above[y] >= 0 && row[y] >= 0) f(above[y], row[y], base + 2 * y, 2 * y + 1);
    }
    const int32_t base = (2 * x + 1) * GW;  // grid row 2x+1: (odd, even) points within pixel row x
    for (int y = 1; y < W; y++)
      if (row[y - 1] != row[y] && row[y - 1] >= 0 && row[y] >= 0) f(row[y - 1], row[y], base + 2 * y, 2 * y);
  };
  for_chunks(par, nband, [&](int t) {
    int64_t c = 0;
    int m = 0;
    for (int x = band_lo(t); x < band_lo(t + 1); x++) {
      const int32_t* row = part + (size_t)x * W;
      for (int y = 0; y < W; y++) m = std::max(m, row[y] + 1);
      scan_row(x, [&](int, int, int32_t, int32_t) { c++; });
    }
    bstart[t + 1] = c;
    bmax[t] = m;
  });
  int n = 0;
  for (int t = 0; t < nband; t++) {
    bstart[t + 1] += bstart[t];
    n = std::max(n, bmax[t]);
  }
  if (n <= 0) return;
  const int32_t ne = (int32_t)bstart[nband];
  std::vector<int32_t> ea(ne), eb(ne), ecol(ne);
  std::vector<double> ev(ne);
  ec.resize(ne);
  for_chunks(par, nband, [&](int t) {
    int64_t q = bstart[t];
    for (int x = band_lo(t); x < band_lo(t + 1); x++)
      scan_row(x, [&](int a, int b, int32_t coord, int32_t col) {
        ea[q] = std::min(a, b);
        eb[q] = std::max(a, b);
        ec[q] = coord;
        ecol[q] = col;
        ev[q] = (double)lb[coord];
        q++;
      });
  });
  // stable counting sorts by grid column, then b, then a: order[i] is the
  // i-th element in (a, b, column-major) order
  std::vector<int32_t> order(ne), seg(ne);
  count_sort(par, ne, GW, ecol.data(), nullptr, [&](int32_t q, int32_t e) { order[q] = e; });
  std::vector<int32_t>().swap(ecol);
  count_sort(par, ne, n, eb.data(), order.data(), [&](int32_t q, int32_t e) { seg[q] = e; });
  // the last pass, by a, carries each element's regions and strength along
  std::vector<int32_t> sa(ne), sb(ne);
  std::vector<double> sv(ne);
  count_sort(par, ne, n, ea.data(), seg.data(), [&](int32_t q, int32_t e) {
    order[q] = e;
    sa[q] = ea[e];
    sb[q] = eb[e];
    sv[q] = ev[e];
  });
  std::vector<int32_t>().swap(eb);
  std::vector<int32_t>().swap(ea);
  std::vector<double>().swap(ev);
  // the initial pairs in (a, b) order, one segment each; seg[e] is element
  // e's segment
  std::vector<Pair> P;
  std::vector<int32_t> pa, pxor;  // each pair's a, and a ^ b
  for (int32_t i = 0; i < ne;) {
    const int32_t a = sa[i], b = sb[i];
    const int32_t p = (int32_t)P.size();
    double total = 0.0;
    int32_t j = i;
    for (; j < ne && sa[j] == a && sb[j] == b; j++) {
      total += sv[j];
      seg[order[j]] = p;
    }
    Pair pr;
    pr.total = total;
    pr.length = j - i;
    pr.head = pr.tail = p;
    P.push_back(pr);
    pa.push_back(a);
    pxor.push_back(a ^ b);
    i = j;
  }
  std::vector<int32_t>().swap(order);
  std::vector<int32_t>().swap(sa);
  std::vector<int32_t>().swap(sb);
  std::vector<double>().swap(sv);
  const int np0 = (int)P.size();
  P.reserve(3 * (size_t)np0);
  pxor.reserve(3 * (size_t)np0);
  std::vector<int32_t> snext(np0, -1);  // segment lists
  std::vector<double> sval(np0);        // each segment's value when its list closes
  // neighbour lists (neighbour, pair index)
  std::vector<std::vector<std::pair<int, int>>> nb(n);
  {
    std::vector<int32_t> deg(n, 0);
    for (int p = 0; p < np0; p++) {
      deg[pa[p]]++;
      deg[pa[p] ^ pxor[p]]++;
    }
    for (int c = 0; c < n; c++) nb[c].reserve(deg[c] + 8);
  }
  // each region's pairs whose last entry has it first, as linked lists of
  // (pushing region, pair)
  struct Pend {
    int32_t b, pair, next;
  };
  std::vector<Pend> pend;
  pend.reserve((size_t)np0 * 3);
  std::vector<int32_t> phead(n, -1);
  std::vector<int> up(n);  // union-find; a root is a live region, its id the father's
  for (int c = 0; c < n; c++) up[c] = c;
  // entries of merged-away regions never pass the label check; they are
  // dropped from the queue in bulk once they make up a quarter to a half of
  // it.
  // qcnt: queue entries naming each region; dead: sum over entries of their
  // merged-away regions (between 1x and 2x the dead entries)
  std::vector<int32_t> qcnt(n, 0);
  size_t dead = 0;
  Queue Q(pxor);
  for (int p = 0; p < np0; p++) {
    const int a = pa[p], b = pa[p] ^ pxor[p];
    nb[a].push_back({b, p});
    nb[b].push_back({a, p});
    Pair& pr = P[p];
    const double d = pr.energy();
    Q.append({energy_key(d), ((uint64_t)(uint32_t)a << 32) | (uint32_t)p});
    qcnt[a]++;
    qcnt[b]++;
    pr.pushed = d;
    pr.first = a;
    pend.push_back({b, p, phead[a]});
    phead[a] = (int32_t)pend.size() - 1;
  }
  std::vector<int32_t>().swap(pa);
  Q.heapify();
  auto push = [&](int pi, double d, int a, int b) {  // entry (d, a, b); b is the region that pushes
    Q.push({energy_key(d), ((uint64_t)(uint32_t)a << 32) | (uint32_t)pi});
    qcnt[a]++;
    qcnt[b]++;
    P[pi].pushed = d;
    P[pi].first = a;
    pend.push_back({b, pi, phead[a]});
    phead[a] = (int32_t)pend.size() - 1;
  };
  auto close = [&](Pair& pr, double extra) {
    const double r = std::max(pr.raise, extra);
    for (int32_t s = pr.head; s >= 0; s = snext[s]) sval[s] = r;
    pr.head = pr.tail = -1;
  };
  std::vector<std::pair<int, int>> touched;
  // the father's pairs by neighbour, for the current merge (mark == merge count)
  std::vector<int32_t> fpair(n), mark(n, -1), nlive(n, 0);
  int32_t merges = 0;
  // the pairs of live regions by key, built when first needed
  PairTable T(0);
  bool table = false;
  while (!Q.empty()) {
    const Entry m = Q.pop();
    const int r1 = (int)(m.lo >> 32), pi = (int)(uint32_t)m.lo;
    const int r2 = r1 ^ pxor[pi];
    qcnt[r1]--;
    qcnt[r2]--;
    if (up[r1] != r1 || up[r2] != r2) {
      dead -= (up[r1] != r1) + (up[r2] != r2);
      continue;
    }
    const double saliency = P[pi].energy();  // both regions live, so the pair is current
    if (key_energy(m.hi) != saliency) continue;
    const int son = std::min(r1, r2), father = std::max(r1, r2);
    close(P[pi], saliency);  // the son-father boundary becomes interior
    up[son] = father;
    dead += qcnt[son];
    // the son's live neighbours other than the father join the father's;
    // the father's pairs come from its list, or, where that list is much
    // longer than the son's, from the table
    touched.clear();
    const bool by_list = nb[father].size() <= 16 * nb[son].size() + 64;
    if (by_list)
      for (const auto& kp : nb[father]) {
        fpair[kp.first] = kp.second;
        mark[kp.first] = merges;
      }
    for (const auto& kp : nb[son]) {
      const int k = kp.first, si = kp.second;
      if (up[k] != k || k == father) continue;
      int fi;
      if (by_list) {  // a live neighbour missing from the father's list has no pair yet
        if (mark[k] == merges) {
          fi = fpair[k];
        } else {
          fi = -(int)P.size() - 1;
          if (table) T.insert(PairTable::key(father, k), (int)P.size());
        }
      } else {
        if (!table) {
          for (int c = 0; c < n; c++)
            if (up[c] == c)
              for (const auto& kq : nb[c])
                if (kq.first > c && up[kq.first] == kq.first) T.insert(PairTable::key(c, kq.first), kq.second);
          table = true;
        }
        fi = T.find_or_add(PairTable::key(father, k), (int)P.size());
      }
      if (fi < 0) {
        fi = -fi - 1;
        P.emplace_back();
        pxor.push_back(father ^ k);
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
        else snext[f.tail] = s.head;
        f.tail = s.tail;
        f.raise = std::max(f.raise, std::max(s.raise, saliency));
        s.head = s.tail = -1;
      }
      touched.push_back({k, fi});
    }
    merges++;
    std::vector<std::pair<int, int>>().swap(nb[son]);
    phead[son] = -1;
    for (int32_t q = phead[father]; q >= 0; q = pend[q].next) touched.push_back({pend[q].b, pend[q].pair});
    phead[father] = -1;
    for (const auto& kp : touched) {
      const int k = kp.first;
      if (up[k] != k || k == father) continue;
      const Pair& f = P[kp.second];
      const double d = f.energy();
      if (!(f.pushed == d && f.first == k)) push(kp.second, d, k, father);
    }
    if (2 * dead >= Q.size() && Q.size() >= 1024) {
      Q.filter([&](const Entry& e) {
        const int a = (int)(e.lo >> 32), b = a ^ pxor[(uint32_t)e.lo];
        if (up[a] == a && up[b] == b) return true;
        qcnt[a]--;
        qcnt[b]--;
        return false;
      });
      dead = 0;
    }
    // drop merged-away neighbours from the father's list once it has grown
    // to twice its live length at the last drop (amortised O(1) a merge)
    if (nb[father].size() >= 2 * (size_t)nlive[father] + 64) {
      std::vector<std::pair<int, int>>& v = nb[father];
      size_t w = 0;
      for (size_t r = 0; r < v.size(); r++)
        if (up[v[r].first] == v[r].first) v[w++] = v[r];
      v.resize(w);
      nlive[father] = (int32_t)w;
    }
  }
  for (Pair& pr : P)  // boundaries never closed (a split adjacency graph)
    if (pr.head >= 0) close(pr, -INFINITY);
  eval.resize(ne);
  for (int32_t e = 0; e < ne; e++) eval[e] = sval[seg[e]];
}

// NormalizeOutput's calibration (contours2ucm.cpp:191-249) of one value:
// logistic, rescaled and clipped to [0, 1].  Most of the grid is 0 and
// boundary runs repeat one value, so a value equal to the previous one
// reuses its result (the same arithmetic either way).
class Calibrate {
 public:
  Calibrate() : f0_(f(0.0)), last_in_(0.0), last_out_(f0_) {}
  double operator()(double x) {
    if (x == 0.0) return f0_;
    if (x != last_in_) {
      last_in_ = x;
      last_out_ = f(x);
    }
    return last_out_;
  }

 private:
  static double f(double x) {
    const double z = 0.0 + 1.0 * -2.7487 + x * 11.1189;
    double v = 1.0 / (1.0 + exp(-z));
    v = (v - 0.0602) / (1.0 - 0.0602);
    return std::min(1.0, std::max(0.0, v));
  }
  double f0_, last_in_, last_out_;
};

enum MapForm { kRaw, kCalibrated, kCalibratedHalf };

// The map from the merge's element values, row by row: zeros, each element
// raised once (every element starts at 0), then CompleteContourMap on the
// even rows: every even-even point takes the largest of its four neighbours
// (from 0).  kRaw and kCalibrated write the (2H+1) x (2W+1) grid, the
// latter calibrated; kCalibratedHalf writes Contours2Ucm's (H+1) x (W+1)
// output (contours2ucm.cpp:476-486): calibrated point (2r+2, 2c+2) at
// (r, c) for r < H, c < W, and 0 in the last row and column, keeping three
// grid rows at a time.
//
// Bands of even rows x0 <= x < x1 run independently: a band owns grid rows
// x0 .. x1-1 and builds its own copy of the odd row above it, which the
// band before owns.
static void write_map(const std::vector<int32_t>& ec, const std::vector<double>& eval, int H, int W, MapForm form,
                      double* out, const ParFor* par) {
  const int GW = 2 * W + 1, GH = 2 * H + 1;
  const bool half = form == kCalibratedHalf;
  const int nband = par ? std::min(kChunks, H + 1) : 1;
  auto band_lo = [&](int t) { return 2 * (int)((int64_t)(H + 1) * t / nband); };  // even rows
  for_chunks(par, nband, [&](int t) {
    const int x0 = band_lo(t), x1 = band_lo(t + 1);
    std::vector<double> ring(half ? 3 * (size_t)GW : 0), above0(x0 > 0 ? GW : 0);
    auto row_at = [&](int r) {
      if (half) return ring.data() + (size_t)(r % 3) * GW;
      return r < x0 ? above0.data() : out + (size_t)r * GW;
    };
    Calibrate cal;
    auto fill_row = [&](int r) {
      double* row = row_at(r);
      memset(row, 0, sizeof(double) * GW);
      const int32_t base = r * GW, end = base + GW;
      for (size_t e = std::lower_bound(ec.begin(), ec.end(), base) - ec.begin(); e < ec.size() && ec[e] < end; e++)
        if (eval[e] > 0.0) row[ec[e] - base] = eval[e];
    };
    auto calibrate_row = [&](int r) {
      double* row = row_at(r);
      for (int y = 0; y < GW; y++) row[y] = cal(row[y]);
    };
    if (x0 > 0) fill_row(x0 - 1);
    for (int x = x0; x < x1 && x < GH; x += 2) {
      fill_row(x);
      if (x + 1 < GH) fill_row(x + 1);
      double* row = row_at(x);
      const double* below = x + 1 < GH ? row_at(x + 1) : nullptr;
      const double* above = x >= 1 ? row_at(x - 1) : nullptr;
      for (int y = 0; y < GW; y += 2) {
        double m = 0.0;
        if (below && m < below[y]) m = below[y];
        if (y + 1 < GW && m < row[y + 1]) m = row[y + 1];
        if (above && m < above[y]) m = above[y];
        if (y >= 1 && m < row[y - 1]) m = row[y - 1];
        row[y] = m;
      }
      // rows x - 1 and x are final: no later step of this band reads them
      if (form == kCalibrated) {
        if (x - 1 > x0) calibrate_row(x - 1);
        calibrate_row(x);
      } else if (half && x >= 2) {
        double* o = out + (size_t)(x / 2 - 1) * (W + 1);
        for (int c = 0; c < W; c++) o[c] = cal(row[2 * c + 2]);
        o[W] = 0.0;
      }
    }
    if (form == kCalibrated && x1 - 1 < GH && x1 - 1 > x0) calibrate_row(x1 - 1);  // the band's last odd row
  });
  if (half)
    for (int c = 0; c <= W; c++) out[(size_t)H * (W + 1) + c] = 0.0;
}

void mean_pb_merge(const double* lb, const int32_t* part, int H, int W, double* ucm) {
  std::vector<int32_t> ec;
  std::vector<double> ev;
  merge_impl(lb, part, H, W, ec, ev, nullptr);
  write_map(ec, ev, H, W, kRaw, ucm, nullptr);
}

void mean_pb_ucm(const float* lb, const int32_t* part, int H, int W, bool half, double* out, const ParFor* par) {
  std::vector<int32_t> ec;
  std::vector<double> ev;
  merge_impl(lb, part, H, W, ec, ev, par);
  write_map(ec, ev, H, W, half ? kCalibratedHalf : kCalibrated, out, par);
}

// The pixels painted along each edge -- its interior pixels, then its two
// end points -- each with the edge's orientation bin (contours2ucm.cpp:
// 331-399).  Edge e's entries start at off[e] + 2e, so bands of edges fill
// theirs independently.
void paint_list(const FitResult& f, int W, std::vector<int32_t>& pix, std::vector<uint8_t>& ori, const ParFor* par) {
  const int ne = (int)f.es.size();
  const size_t total = (size_t)f.off[ne] + 2 * (size_t)ne;
  pix.resize(total);
  ori.resize(total);
  const int nt = par ? std::min(kChunks, std::max(ne, 1)) : 1;
  for_chunks(par, nt, [&](int t) {
    for (int e = (int)((int64_t)ne * t / nt); e < (int)((int64_t)ne * (t + 1) / nt); e++) {
      const int a = f.es[e], b = f.ee[e];
      const uint8_t o = (uint8_t)edge_orientation(f.vx[a], f.vy[a], f.vx[b], f.vy[b]);
      size_t q = (size_t)f.off[e] + 2 * (size_t)e;
      for (int k = f.off[e]; k < f.off[e + 1]; k++, q++) {
        pix[q] = f.px[k];
        ori[q] = o;
      }
      pix[q] = f.vx[a] * W + f.vy[a];
      ori[q++] = o;
      pix[q] = f.vx[b] * W + f.vy[b];
      ori[q] = o;
    }
  });
}

// NormalizeOutput over a whole map
void normalize(double* u, size_t n) {
  Calibrate cal;
  for (size_t i = 0; i < n; i++) u[i] = cal(u[i]);
}

}  // namespace ucm
}  // namespace gpb
