/*
 * gpb_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker and the timed CPU
 * baseline).  Nothing in the CUDA library links, calls or loads this file.
 *
 * An FP64 restatement, in plain C, of the reference's CPU gPb path with its
 * defects fixed behind named flags (orc_params).  Every function cites the
 * reference file:line it follows.  The orders of floating-point operations
 * follow the reference where the reference's cores are compiled beside it
 * (oracle/_ref, see oracle/Makefile.ref), so the restatement can be pinned to
 * them bit for bit; OpenCV glue (absent here) is restated from its documented
 * semantics and is unpinned.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off (contraction off keeps x86 and
 * aarch64 results identical).
 */
#define _GNU_SOURCE
#include "gpb_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* include/UCM_CONSTANTS.h:4 -- the reference's truncated pi */
static const double REF_PI = 3.1415926535;
static const long double PI_L = 3.141592653589793238462643383279502884L;
static const long double PI_2L = 1.570796326794896619231321691639751442L;
static const long double PI_4L = 0.785398163397448309615660845819875721L;

void orc_default_params(orc_params* p) {
  p->fix_rb_swap = 1;
  p->fix_argmin = 1;
  p->nvec = 9;
  p->fix_clip_scale = 1;
  p->fix_eig_order = 1;
  p->damascene_weights = 0;
  p->sigmoid = 0;
  p->eig_tol = 1e-10;
  p->eig_maxit = 3000;
  p->threads = 0;
}

static void set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* cv::BORDER_REFLECT and lib_image border_mirror_2D (lib_image.cc:305-369):
 * ...cba|abc...  (edge sample repeated) */
static inline int refl(int i, int n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) {
    if (i < 0) i = -i - 1;
    else i = 2 * n - 1 - i;
  }
  return i;
}
/* cv::BORDER_REFLECT_101: ...dcb|abcd... (edge sample not repeated) */
static inline int refl101(int i, int n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) {
    if (i < 0) i = -i;
    else i = 2 * n - 2 - i;
  }
  return i;
}

/* ======================================================================= */
/* (a) Schmid textons                                                       */
/* ======================================================================= */

/* (sigma, tau) of the 13 S filters, src/SPFeatures.cpp:167-183 */
static const int SCHMID_ST[ORC_NSCHMID][2] = {{2, 1}, {4, 1}, {4, 2}, {6, 1}, {6, 2},
                                              {6, 3}, {8, 1}, {8, 2}, {8, 3}, {10, 1},
                                              {10, 2}, {10, 3}, {10, 4}};

/* SPFeatures::makefilter, src/SPFeatures.cpp:117-165: F = cos(pi tau r/sigma)
 * exp(-r^2/2sigma^2), minus its mean, divided by the sum of |F| taken BEFORE the
 * mean was removed (the reference's order). */
void orc_schmid_bank(double* F) {
  const int sup = ORC_SCHMID_SUP, h = sup / 2;
  for (int f = 0; f < ORC_NSCHMID; f++) {
    const int sigma = SCHMID_ST[f][0], tau = SCHMID_ST[f][1];
    double* g = F + (size_t)f * sup * sup;
    double fsum = 0, fsum_abs = 0;
    for (int i = 0; i < sup; i++)
      for (int j = 0; j < sup; j++) {
        const double x = j - h, y = i - h;
        const double r = sqrt(x * x + y * y);
        double v = cos(r * (REF_PI * tau / sigma));
        v *= exp(-r * r / (2 * sigma * sigma));
        g[i * sup + j] = v;
        fsum += v;
        fsum_abs += fabs(v);
      }
    const double mean = fsum / (sup * sup);
    const double inv = 1.0 / fsum_abs; /* cv::MatExpr A / s evaluates A * (1/s) */
    for (int k = 0; k < sup * sup; k++) g[k] = (g[k] - mean) * inv;
  }
}

/* The S filters depend on r only, so the 49x49 window splits into rings of
 * equal dy^2+dx^2; rings are numbered by ascending radius. */
int orc_schmid_rings(int* ring_of_offset, int* ring_s) {
  const int sup = ORC_SCHMID_SUP, h = sup / 2;
  int id_of_s[2 * 24 * 24 + 1];
  for (int s = 0; s <= 2 * h * h; s++) id_of_s[s] = -1;
  for (int i = 0; i < sup; i++)
    for (int j = 0; j < sup; j++) id_of_s[(i - h) * (i - h) + (j - h) * (j - h)] = 0;
  int n = 0;
  for (int s = 0; s <= 2 * h * h; s++)
    if (id_of_s[s] == 0) {
      id_of_s[s] = n;
      if (ring_s) ring_s[n] = s;
      n++;
    }
  for (int i = 0; i < sup; i++)
    for (int j = 0; j < sup; j++)
      ring_of_offset[i * sup + j] = id_of_s[(i - h) * (i - h) + (j - h) * (j - h)];
  return n;
}

/* cv::cvtColor(CV_BGR2GRAY) on 8-bit data (src/SPFeatures.cpp:27): OpenCV's
 * fixed-point Rec.601 luma, Y = (4899 R + 9617 G + 1868 B + 2^13) >> 14. */
void orc_grey_bgr(const uint8_t* bgr, int H, int W, uint8_t* grey) {
  for (long n = 0; n < (long)H * W; n++) {
    const int B = bgr[3 * n], G = bgr[3 * n + 1], R = bgr[3 * n + 2];
    grey[n] = (uint8_t)((R * 4899 + G * 9617 + B * 1868 + (1 << 13)) >> 14);
  }
}

/* SPFeatures::genTextonMap, src/SPFeatures.cpp:277-360: reflect-pad 24
 * (copyMakeBorder BORDER_REFLECT), correlate with the 13 S filters converted to
 * FP32, assign each pixel to the nearest codebook column (L2).  Responses are
 * formed in FP64 as sum over rings (ascending) of K32(ring) * S(ring), where
 * S(ring) is the exact integer sum of the grey values on that ring.  With
 * fix_argmin=0 the reference's defect (D4) is reproduced: label = K-1. */
void orc_texton_map(const uint8_t* grey, int H, int W, const float* cb, int K, int fix_argmin,
                    uint8_t* labels, double* resp) {
  const int sup = ORC_SCHMID_SUP, h = sup / 2, nw = sup * sup;
  double* F = (double*)malloc(sizeof(double) * ORC_NSCHMID * nw);
  orc_schmid_bank(F);
  int ring_of[ORC_SCHMID_SUP * ORC_SCHMID_SUP];
  const int nr = orc_schmid_rings(ring_of, NULL);
  double* K32 = (double*)malloc(sizeof(double) * ORC_NSCHMID * nr);
  for (int f = 0; f < ORC_NSCHMID; f++)
    for (int o = 0; o < nw; o++) K32[f * nr + ring_of[o]] = (double)(float)F[f * nw + o];
  free(F);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; y++) {
    long long S[1200];
    double R[ORC_NSCHMID];
    for (int x = 0; x < W; x++) {
      for (int k = 0; k < nr; k++) S[k] = 0;
      for (int i = 0; i < sup; i++) {
        const uint8_t* row = grey + (size_t)refl(y + i - h, H) * W;
        for (int j = 0; j < sup; j++) S[ring_of[i * sup + j]] += row[refl(x + j - h, W)];
      }
      for (int f = 0; f < ORC_NSCHMID; f++) {
        double acc = 0;
        for (int k = 0; k < nr; k++) acc += K32[f * nr + k] * (double)S[k];
        R[f] = acc;
        if (resp) resp[(size_t)f * H * W + (size_t)y * W + x] = acc;
      }
      int best = -1;
      double bd = INFINITY;
      for (int k = 0; k < K; k++) {
        double d = 0;
        for (int f = 0; f < ORC_NSCHMID; f++) {
          const double t = R[f] - (double)cb[f * K + k];
          d += t * t;
        }
        if (fix_argmin) {
          if (d < bd) {
            bd = d;
            best = k;
          }
        } else {
          if (sqrt(d) < bd) best = k; /* minDistance never updated */
        }
      }
      labels[(size_t)y * W + x] = (uint8_t)best;
    }
  }
  free(K32);
}

/* ======================================================================= */
/* (b) local cues                                                           */
/* ======================================================================= */

/* Colour chain of mex_pb_parts_final_selected.cpp:97-134 on one pixel:
 * convertTo(1/255) (globalPb.cpp:20), rgb_gamma_correct 2.5
 * (lib_image.cc:123-140), rgb_to_xyz + xyz_to_lab (lib_image.cc:172-248),
 * lab_normalize (lib_image.cc:143-167), quantize_values (lib_image.cc:2315-2343). */
static void lab_bin_pixel(int B8, int G8, int R8, int nbins, int fix_rb, uint8_t* q) {
  const double s = 1.0 / 255.0;
  const double Bv = B8 * s, Gv = G8 * s, Rv = R8 * s;
  double r = fix_rb ? Rv : Bv, g = Gv, b = fix_rb ? Bv : Rv;
  r = pow(r, 2.5);
  g = pow(g, 2.5);
  b = pow(b, 2.5);
  const double X = (0.412453 * r) + (0.357580 * g) + (0.180423 * b);
  const double Y = (0.212671 * r) + (0.715160 * g) + (0.072169 * b);
  const double Z = (0.019334 * r) + (0.119193 * g) + (0.950227 * b);
  const double x = X / 0.950456, y = Y / 1.000000, z = Z / 1.088754;
  const double th = 0.008856;
  const double fx = (x > th) ? pow(x, (1.0 / 3.0)) : (7.787 * x + (16.0 / 116.0));
  const double fy = (y > th) ? pow(y, (1.0 / 3.0)) : (7.787 * y + (16.0 / 116.0));
  const double fz = (z > th) ? pow(z, (1.0 / 3.0)) : (7.787 * z + (16.0 / 116.0));
  const double L = (y > th) ? (116 * pow(y, (1.0 / 3.0)) - 16) : (903.3 * y);
  const double A = 500 * (fx - fy);
  const double Bb = 200 * (fy - fz);
  double v[3];
  v[0] = L / 100.0;
  v[1] = (A - (-73.0)) / 168.0;
  v[2] = (Bb - (-73.0)) / 168.0;
  for (int c = 0; c < 3; c++) {
    if (v[c] < 0) v[c] = 0;
    else if (v[c] > 1) v[c] = 1;
    unsigned long bin = (unsigned long)floor(v[c] * (double)nbins);
    if (bin == (unsigned long)nbins) bin = nbins - 1;
    q[c] = (uint8_t)bin;
  }
}

void orc_lab_bins(const uint8_t* bgr, int H, int W, int nbins, int fix_rb, uint8_t* Lq,
                  uint8_t* aq, uint8_t* bq) {
#pragma omp parallel for schedule(static)
  for (long n = 0; n < (long)H * W; n++) {
    uint8_t q[3];
    lab_bin_pixel(bgr[3 * n], bgr[3 * n + 1], bgr[3 * n + 2], nbins, fix_rb, q);
    Lq[n] = q[0];
    aq[n] = q[1];
    bq[n] = q[2];
  }
}

void orc_mirror_u8(const uint8_t* src, int H, int W, int b, uint8_t* dst) {
  const int Wp = W + 2 * b;
  for (int y = 0; y < H + 2 * b; y++)
    for (int x = 0; x < Wp; x++) dst[(size_t)y * Wp + x] = src[(size_t)refl(y - b, H) * W + refl(x - b, W)];
}

/* orientation_slice_map, lib_image.cc:3052-3081, evaluated at the window
 * position that compute_hist_gradient_2D (lib_image.cc:3120-3235, a
 * convolution) pairs with the label at offset (drow, dcol) from the centre:
 * window index (r-drow, r-dcol), i.e. the point (-drow-0.5, -dcol-0.5).  The
 * reference mixes double and long double in this expression; as compiled
 * (x86-64, -O2) its map equals floor((atan2(y,x) + pi) / pi * 8) in double
 * at every offset within radius 20, the exact diagonals included (checked
 * against the compiled reference cores), which is what this evaluates. */
int orc_slice_index(int r, int drow, int dcol) {
  (void)r;
  const double x = -(double)drow - 0.5, y = -(double)dcol - 0.5;
  int idx = (int)floor((atan2(y, x) + M_PI) / M_PI * 8.0);
  if (idx > 15) idx = 15;
  return idx;
}

/* lib_image::gaussian(sigma, 0, false) (lib_image.cc:1374-1441): support
 * ceil(3 sigma), unit L1 norm. */
int orc_gaussian_kernel(double sigma, double* k) {
  const unsigned long support = (unsigned long)ceil(3 * sigma);
  const double sigma2_inv = 1.0 / (sigma * sigma);
  const double neg_two_sigma2_inv = -0.5 * sigma2_inv;
  const int size = (int)(2 * support + 1);
  double x = -(double)support;
  for (int n = 0; n < size; n++, x++) k[n] = exp(x * x * neg_two_sigma2_inv);
  double s = 0;
  for (int n = 0; n < size; n++) s += fabs(k[n]);
  for (int n = 0; n < size; n++) k[n] /= s;
  return size;
}

/* lib_image::hist_gradient_2D (lib_image.cc:3575-3686) and
 * compute_hist_gradient_2D (lib_image.cc:3120-3235) for the interior pixels of
 * a mirrored label image: integer half-disc slice counts (weight_matrix_disc,
 * lib_image.cc:3027-3047), 1-D smoothing along bins (conv_in_place_1D,
 * lib_image.cc:3084-3115), per-slice L1 normalisation, the 8-step spin and the
 * chi-squared distance (matrix_X2_distance, matrix_distance_functors.hh:95-107).
 * The histogram length is max(label)+1 over the padded image, as in the
 * reference.  Returns that length. */
int orc_hist_gradient(const uint8_t* lab, int Hp, int Wp, int border, int r, const double* kern,
                      int klen, double* out, int32_t* counts, int threads) {
  set_threads(threads);
  const int H = Hp - 2 * border, W = Wp - 2 * border;
  int nb = 0;
  for (long n = 0; n < (long)Hp * Wp; n++)
    if (lab[n] + 1 > nb) nb = lab[n] + 1;
  /* disc offsets and their slices */
  const int dn = 2 * r + 1;
  int* off_r = (int*)malloc(sizeof(int) * dn * dn);
  int* off_c = (int*)malloc(sizeof(int) * dn * dn);
  int* off_s = (int*)malloc(sizeof(int) * dn * dn);
  int no = 0;
  for (int a = -r; a <= r; a++)
    for (int b = -r; b <= r; b++)
      if (a * a + b * b <= r * r) {
        off_r[no] = a;
        off_c[no] = b;
        off_s[no] = orc_slice_index(r, a, b);
        no++;
      }
#pragma omp parallel
  {
    double* sh = (double*)malloc(sizeof(double) * 16 * nb);
    double* tmp = (double*)malloc(sizeof(double) * nb);
    double* hl = (double*)malloc(sizeof(double) * nb);
    double* hr = (double*)malloc(sizeof(double) * nb);
#pragma omp for schedule(dynamic, 2)
    for (int y = 0; y < H; y++)
      for (int x = 0; x < W; x++) {
        for (int i = 0; i < 16 * nb; i++) sh[i] = 0;
        const int cy = y + border, cx = x + border;
        for (int k = 0; k < no; k++) {
          const int lbl = lab[(size_t)(cy + off_r[k]) * Wp + cx + off_c[k]];
          sh[off_s[k] * nb + lbl] += 1.0;
        }
        if (counts) {
          int32_t* cp = counts + ((size_t)y * W + x) * 16 * nb;
          for (int i = 0; i < 16 * nb; i++) cp[i] = (int32_t)sh[i];
        }
        if (klen > 0) {
          for (int o = 0; o < 16; o++) {
            double* s = sh + o * nb;
            for (int n = 0; n < nb; n++) tmp[n] = 0;
            const int pos_start = klen / 2;
            for (int n = 0, pos = pos_start; n < nb; n++, pos++) {
              const int omin = (pos + 1 > nb) ? (pos + 1 - nb) : 0;
              const int omax = (pos < klen) ? pos : (klen - 1);
              for (int i1 = omin, i0 = pos - omin; i1 <= omax; i1++, i0--) tmp[n] += s[i0] * kern[i1];
            }
            for (int n = 0; n < nb; n++) s[n] = tmp[n];
          }
        }
        for (int o = 0; o < 16; o++) {
          double* s = sh + o * nb;
          double sum = 0;
          for (int n = 0; n < nb; n++) sum += s[n];
          if (sum != 0)
            for (int n = 0; n < nb; n++) s[n] /= sum;
        }
        for (int n = 0; n < nb; n++) hl[n] = hr[n] = 0;
        for (int o = 0; o < 8; o++)
          for (int n = 0; n < nb; n++) {
            hl[n] += sh[o * nb + n];
            hr[n] += sh[(o + 8) * nb + n];
          }
        for (int o = 0; o < 8; o++) {
          double dist = 0;
          for (int n = 0; n < nb; n++) {
            const double diff = hr[n] - hl[n];
            const double sm = hr[n] + hl[n];
            if (diff != 0) dist += diff * diff / sm;
          }
          out[(size_t)o * H * W + (size_t)y * W + x] = dist / 2;
          for (int n = 0; n < nb; n++) {
            hl[n] -= sh[o * nb + n];
            hl[n] += sh[(o + 8) * nb + n];
            hr[n] += sh[o * nb + n];
            hr[n] -= sh[(o + 8) * nb + n];
          }
        }
      }
    free(sh);
    free(tmp);
    free(hl);
    free(hr);
  }
  free(off_r);
  free(off_c);
  free(off_s);
  return nb;
}

/* mex_pb_parts_final_selected.cpp:76-235 with the Schmid-codebook textons
 * (genTextonMap, src/SPFeatures.cpp:277-360) in place of k-means (D8): mirror 30, Lab quantised to 25 bins,
 * bg r={3,5,10} (sigma 0.1*25), cga/cgb r={5,10,20} (sigma 0.05*25),
 * tg r={5,10,20} on the mirrored texton map, unsmoothed. */
void orc_local_cues(const uint8_t* bgr, const uint8_t* texton, int H, int W, const orc_params* p,
                    double* cues) {
  const int border = 30, nbins = 25;
  const int Hp = H + 2 * border, Wp = W + 2 * border;
  const size_t N = (size_t)H * W, Np = (size_t)Hp * Wp;
  uint8_t* q = (uint8_t*)malloc(3 * N);
  uint8_t* qp = (uint8_t*)malloc(4 * Np);
  orc_lab_bins(bgr, H, W, nbins, p->fix_rb_swap, q, q + N, q + 2 * N);
  for (int c = 0; c < 3; c++) orc_mirror_u8(q + c * N, H, W, border, qp + c * Np);
  orc_mirror_u8(texton, H, W, border, qp + 3 * Np);
  double kbg[64], kcg[64];
  const int nkbg = orc_gaussian_kernel(0.1 * nbins, kbg);
  const int nkcg = orc_gaussian_kernel(0.05 * nbins, kcg);
  static const int r_bg[3] = {3, 5, 10}, r_cg[3] = {5, 10, 20};
  for (int s = 0; s < 3; s++) {
    orc_hist_gradient(qp, Hp, Wp, border, r_bg[s], kbg, nkbg, cues + (size_t)(0 + s) * 8 * N, NULL,
                      p->threads);
    orc_hist_gradient(qp + Np, Hp, Wp, border, r_cg[s], kcg, nkcg, cues + (size_t)(3 + s) * 8 * N,
                      NULL, p->threads);
    orc_hist_gradient(qp + 2 * Np, Hp, Wp, border, r_cg[s], kcg, nkcg,
                      cues + (size_t)(6 + s) * 8 * N, NULL, p->threads);
    orc_hist_gradient(qp + 3 * Np, Hp, Wp, border, r_cg[s], NULL, 0, cues + (size_t)(9 + s) * 8 * N,
                      NULL, p->threads);
  }
  free(q);
  free(qp);
}

/* weighted cue sum, left to right (multiscalePb.cpp:217-245) */
void orc_combine(const double* cues, int H, int W, const double* w, double* out) {
  const size_t N = (size_t)H * W;
  for (int o = 0; o < 8; o++)
    for (size_t n = 0; n < N; n++) {
      double acc = w[0] * cues[(size_t)(0 * 8 + o) * N + n];
      for (int k = 1; k < 12; k++) acc = acc + w[k] * cues[(size_t)(k * 8 + o) * N + n];
      out[(size_t)o * N + n] = acc;
    }
}

/* nonmax_channels (src/nonmax_channels.cpp:8-80, D6 fixed: per-pixel reset),
 * lib_image::nonmax_oriented_2D (lib_image.cc:4083-4197, tolerance PI/8 with
 * the reference's truncated PI), then the clip of multiscalePb.cpp:249-261
 * (fix_clip_scale: MATLAB's max(0,min(1,1.2 v)), D7). */
void orc_nonmax(const double* mo, int H, int W, int fix_clip_scale, double* nmax) {
  const size_t N = (size_t)H * W;
  double* a = (double*)malloc(sizeof(double) * N);
  double* ind = (double*)malloc(sizeof(double) * N);
  double oris[8];
  for (int i = 0; i < 8; i++) oris[i] = (double)i * REF_PI / (double)8;
  for (size_t n = 0; n < N; n++) {
    double mv = -DBL_MAX;
    int mi = 0;
    for (int i = 0; i < 8; i++) {
      const double d = mo[(size_t)i * N + n];
      if (d > mv) {
        mv = d;
        mi = i;
      }
    }
    if (mv < 0) mv = 0;
    a[n] = mv;
    ind[n] = oris[mi];
  }
  const double o_tol = REF_PI / 8;
  const long sx = H, sy = W;
  size_t n = 0;
  for (long x = 0; x < sx; x++)
    for (long y = 0; y < sy; y++, n++) {
      const double ori = ind[n];
      double theta = (long double)ori + PI_2L;
      theta = (long double)theta - floorl((long double)theta / PI_L) * PI_L;
      const double v = a[n];
      size_t i0a = 0, i0b = 0, i1a = 0, i1b = 0;
      double d = 0;
      int valid0 = 0, valid1 = 0;
      if (theta == 0) {
        valid0 = (x > 0);
        valid1 = (x < sx - 1);
        if (valid0) i0a = i0b = n - sy;
        if (valid1) i1a = i1b = n + sy;
      } else if (theta < PI_4L) {
        d = tan(theta);
        valid0 = (x > 0) && (y > 0);
        valid1 = (x < sx - 1) && (y < sy - 1);
        if (valid0) { i0a = n - sy; i0b = i0a - 1; }
        if (valid1) { i1a = n + sy; i1b = i1a + 1; }
      } else if (theta < PI_2L) {
        d = tanl(PI_2L - theta);
        valid0 = (x > 0) && (y > 0);
        valid1 = (x < sx - 1) && (y < sy - 1);
        if (valid0) { i0a = n - 1; i0b = i0a - sy; }
        if (valid1) { i1a = n + 1; i1b = i1a + sy; }
      } else if (theta == PI_2L) {
        valid0 = (y > 0);
        valid1 = (y < sy - 1);
        if (valid0) i0a = i0b = n - 1;
        if (valid1) i1a = i1b = n + 1;
      } else if (theta < 3.0L * PI_4L) {
        d = tanl(theta - PI_2L);
        valid0 = (x < sx - 1) && (y > 0);
        valid1 = (x > 0) && (y < sy - 1);
        if (valid0) { i0a = n - 1; i0b = i0a + sy; }
        if (valid1) { i1a = n + 1; i1b = i1a - sy; }
      } else {
        d = tanl(PI_L - theta);
        valid0 = (x < sx - 1) && (y > 0);
        valid1 = (x > 0) && (y < sy - 1);
        if (valid0) { i0a = n + sy; i0b = i0a - 1; }
        if (valid1) { i1a = n - sy; i1b = i1a + 1; }
      }
      double out = 0;
      if (valid0 && valid1) {
        double v0a = 0, v0b = 0, v1a = 0, v1b = 0, o0a = 0, o0b = 0, o1a = 0, o1b = 0;
        v0a = a[i0a]; v0b = a[i0b];
        o0a = ind[i0a] - ori; o0b = ind[i0b] - ori;
        v1a = a[i1a]; v1b = a[i1b];
        o1a = ind[i1a] - ori; o1b = ind[i1b] - ori;
        double* os[4] = {&o0a, &o0b, &o1a, &o1b};
        for (int k = 0; k < 4; k++) {
          double t = *os[k];
          t = (long double)t - floorl((long double)t / (2 * PI_L)) * (2 * PI_L);
          if (t >= PI_L) t = 2 * PI_L - t;
          if (t >= PI_2L) t = PI_L - t;
          t = (t <= o_tol) ? 0 : (t - o_tol);
          *os[k] = t;
        }
        const double v0 = (1.0 - d) * v0a * cos(o0a) + d * v0b * cos(o0b);
        const double v1 = (1.0 - d) * v1a * cos(o1a) + d * v1b * cos(o1b);
        if ((v > v0) && (v > v1)) out = v;
      }
      if (fix_clip_scale) {
        out = (1.2 * out > 1) ? 1 : 1.2 * out;
      } else if (1.2 * out > 1) {
        out = 1;
      }
      if (out < 0) out = 0;
      nmax[n] = out;
    }
  free(a);
  free(ind);
}

/* ======================================================================= */
/* (c) buildW: intervening contour (buildW/src/ic.cc, affinity.cc, smatrix.cc) */
/* ======================================================================= */

void orc_stencil(int* dy, int* dx) {
  int n = 0;
  for (int u = -ORC_STENCIL_R; u <= ORC_STENCIL_R; u++)
    for (int v = -ORC_STENCIL_R; v <= ORC_STENCIL_R; v++)
      if (u * u + v * v <= ORC_STENCIL_R * ORC_STENCIL_R) {
        dy[n] = u;
        dx[n] = v;
        n++;
      }
}

typedef struct {
  int x, y;
  float sim;
} pt_ic;

typedef struct {
  const float* mpb; /* H x W, FP32 as Util::Image stores it */
  int width, height;
} lattice;

/* DualLattice of src/buildW.cpp:55-116: H(x,y) = mPb[y-1][x] (row 0 zero),
 * V(x,y) = mPb[y][x-1] (column 0 zero). */
static inline float latH(const lattice* L, int x, int y) {
  return y > 0 ? L->mpb[(size_t)(y - 1) * L->width + x] : 0.0f;
}
static inline float latV(const lattice* L, int x, int y) {
  return x > 0 ? L->mpb[(size_t)y * L->width + (x - 1)] : 0.0f;
}
static inline float fmaxf_(float a, float b) { return a > b ? a : b; }

/* Group::ic_walk, buildW/src/ic.cc:86-363 */
static void ic_walk(const lattice* L, float thresh, int x0, int y0, int x1, int y1, int x2, int y2,
                    int x3, int y3, int wr, pt_ic* points, int* scanCount, pt_ic* scanLines) {
  const long long dx1 = x1 - x0, dy1 = y1 - y0, dx2 = x2 - x0, dy2 = y2 - y0, dx3 = x3 - x0,
                  dy3 = y3 - y0;
  const long long dot11 = dx1 * dx1 + dy1 * dy1, dot22 = dx2 * dx2 + dy2 * dy2,
                  dot33 = dx3 * dx3 + dy3 * dy3;
  const int dx = x2 - x0, dy = y2 - y0, adx = abs(dx), ady = abs(dy);
  int octant = -1;
  if (dx > 0 && dy >= 0) octant = (adx > ady) ? 0 : 1;
  else if (dx <= 0 && dy > 0) octant = (adx < ady) ? 2 : 3;
  else if (dy <= 0 && dx < 0) octant = (adx > ady) ? 4 : 5;
  else if (dx >= 0 && dy < 0) octant = (adx < ady) ? 6 : 7;
  int t = 0;
  switch (octant) {
    case 0: case 3: case 4: case 7: t = -adx; break;
    default: t = -ady; break;
  }
  float maxpb = 0.0f;
  int xi = x0, yi = y0, count = 0, oldx = xi, oldy = yi;
  while (xi != x2 || yi != y2) {
    switch (octant) {
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
    const int good = (doti2 * doti2 == dotii * dot22) ||
                     (dot11 * doti2 * doti2 > dot22 * doti1 * doti1 &&
                      dot33 * doti2 * doti2 >= dot22 * doti3 * doti3);
    float inter = 0.0f;
    if (oldx == xi) {
      if (yi > oldy) inter = latH(L, xi, yi);
      else if (yi < oldy) inter = latH(L, oldx, oldy);
    } else if (oldy == yi) {
      if (xi > oldx) inter = latV(L, xi, yi);
      else if (xi < oldx) inter = latV(L, oldx, oldy);
    } else {
      if ((xi > oldx) && (yi > oldy)) {
        inter = fmaxf_(latH(L, oldx, yi), inter);
        inter = fmaxf_(latH(L, xi, yi), inter);
        inter = fmaxf_(latV(L, xi, oldy), inter);
        inter = fmaxf_(latV(L, xi, yi), inter);
      } else if ((xi > oldx) && (yi < oldy)) {
        inter = fmaxf_(latH(L, oldx, oldy), inter);
        inter = fmaxf_(latH(L, xi, oldy), inter);
        inter = fmaxf_(latV(L, xi, oldy), inter);
        inter = fmaxf_(latV(L, xi, yi), inter);
      } else if ((xi < oldx) && (yi > oldy)) {
        inter = fmaxf_(latH(L, oldx, yi), inter);
        inter = fmaxf_(latH(L, xi, yi), inter);
        inter = fmaxf_(latV(L, oldx, oldy), inter);
        inter = fmaxf_(latV(L, oldx, yi), inter);
      } else if ((xi < oldx) && (yi < oldy)) {
        inter = fmaxf_(latH(L, oldx, oldy), inter);
        inter = fmaxf_(latH(L, xi, oldy), inter);
        inter = fmaxf_(latV(L, oldx, oldy), inter);
        inter = fmaxf_(latV(L, oldx, yi), inter);
      }
    }
    maxpb = fmaxf_(maxpb, inter);
    oldx = xi;
    oldy = yi;
    if (!good) continue;
    if (maxpb > thresh) break;
    points[count].x = xi;
    points[count].y = yi;
    points[count].sim = 1.0f - maxpb;
    count++;
  }
  const int wd = 2 * wr + 1;
  if (octant == 0 || octant == 1 || octant == 6 || octant == 7) {
    for (int i = 0; i < count; i++) {
      const int yind = points[i].y - y0 + wr;
      scanLines[yind * wd + scanCount[yind]++] = points[i];
    }
  } else {
    for (int i = count - 1; i >= 0; i--) {
      const int yind = points[i].y - y0 + wr;
      scanLines[yind * wd + scanCount[yind]++] = points[i];
    }
  }
}

static void push_pt(pt_ic* scanLines, int* scanCount, int wd, int wr, int y0, int x, int y) {
  pt_ic p;
  p.x = x;
  p.y = y;
  p.sim = 1.0f;
  const int yind = y - y0 + wr;
  scanLines[yind * wd + scanCount[yind]++] = p;
}

/* Group::interveningContour, buildW/src/ic.cc:375-545: the walk order around
 * the clipped box, then scanline concatenation. Returns the count. */
static int intervening(const lattice* L, float thresh, int x0, int y0, int wr, pt_ic* adj,
                       pt_ic* scanLines, int* scanCount, pt_ic* scratch) {
  const int width = L->width, height = L->height, wd = 2 * wr + 1;
  for (int i = 0; i < wd; i++) scanCount[i] = 0;
  const int rxa = x0 - wr > 0 ? x0 - wr : 0;
  const int rya = y0 - wr > 0 ? y0 - wr : 0;
  const int rxb = x0 + wr < width - 1 ? x0 + wr : width - 1;
  const int ryb = y0 + wr < height - 1 ? y0 + wr : height - 1;
#define WALK(a, b, c, d, e, f) ic_walk(L, thresh, x0, y0, a, b, c, d, e, f, wr, scratch, scanCount, scanLines)
  if (x0 > rxa) {
    if ((y0 > 0) && (y0 < ryb)) WALK(rxa, y0 - 1, rxa, y0, rxa, y0 + 1);
    for (int y = y0 - 1; y > rya; y--) WALK(rxa, y - 1, rxa, y, rxa, y + 1);
  }
  if (x0 > rxa + 1 || y0 > rya + 1 || ((x0 > rxa) && (y0 > rya))) WALK(rxa, rya + 1, rxa, rya, rxa + 1, rya);
  if (((x0 == rxa) && (y0 == rya + 1)) || ((x0 == rxa + 1) && (y0 == rya)))
    push_pt(scanLines, scanCount, wd, wr, y0, rxa, rya);
  if (y0 > rya)
    for (int x = rxa + 1; x < rxb; x++) WALK(x - 1, rya, x, rya, x + 1, rya);
  if ((y0 > rya + 1) || (x0 < rxb - 1) || ((y0 > rya) && (x0 < rxb))) WALK(rxb - 1, rya, rxb, rya, rxb, rya + 1);
  if (((x0 == rxb - 1) && (y0 == rya)) || ((x0 == rxb) && (y0 == rya + 1)))
    push_pt(scanLines, scanCount, wd, wr, y0, rxb, rya);
  if (x0 < rxb)
    for (int y = rya + 1; y < y0; y++) WALK(rxb, y - 1, rxb, y, rxb, y + 1);
  if (x0 > rxa)
    for (int y = y0 + 1; y < ryb; y++) WALK(rxa, y - 1, rxa, y, rxa, y + 1);
  if ((x0 > rxa + 1) || (y0 < ryb - 1) || ((x0 > rxa) && (y0 < ryb))) WALK(rxa, ryb - 1, rxa, ryb, rxa + 1, ryb);
  if (((x0 == rxa) && (y0 == ryb - 1)) || ((x0 == rxa + 1) && (y0 == ryb)))
    push_pt(scanLines, scanCount, wd, wr, y0, rxa, ryb);
  if (y0 < ryb)
    for (int x = rxa + 1; x < rxb; x++) WALK(x - 1, ryb, x, ryb, x + 1, ryb);
  if ((y0 < ryb - 1) || (x0 < rxb - 1) || ((y0 < ryb) && (x0 < rxb))) WALK(rxb - 1, ryb, rxb, ryb, rxb, ryb - 1);
  if (((x0 == rxb - 1) && (y0 == ryb)) || ((x0 == rxb) && (y0 == ryb - 1)))
    push_pt(scanLines, scanCount, wd, wr, y0, rxb, ryb);
  if (x0 < rxb) {
    for (int y = ryb - 1; y > y0; y--) WALK(rxb, y - 1, rxb, y, rxb, y + 1);
    if ((y0 > 0) && (y0 < ryb)) WALK(rxb, y0 - 1, rxb, y0, rxb, y0 + 1);
  }
#undef WALK
  int count = 0;
  for (int y = 0; y < wd; y++)
    for (int i = 0; i < scanCount[y]; i++) adj[count++] = scanLines[y * wd + i];
  return count;
}

/* Group::C_IC_SS, buildW/src/affinity.cc:40-51 */
static float c_ic_ss(float ic) {
  float val = 1.8682f;
  val = (float)((double)val + ((double)ic / 0.3130) * -1.3113);
  const float post = (float)(1.0 / (1.0 + exp(-(double)val)));
  if (!isfinite(post)) return 0;
  if (post < 0) return 0;
  if (post > 1) return 1;
  return post;
}

/* Group::computeSupport (ic.cc:42-73) + computeAffinities2 (affinity.cc:58-156,
 * including its scanline lookup) + SMatrix::symmetrize (smatrix.cc:95-117),
 * with dThresh 5, sigma 0.1, threshold 1.0 (src/buildW.cpp:23-24,123-126).
 * The result is stored in stencil (DIA) form: Wd[p*81 + k] for offset k. */
void orc_buildW(const double* mpb, int H, int W, double* Wd, int threads) {
  set_threads(threads);
  const int wr = ORC_STENCIL_R, wd = 2 * wr + 1;
  const size_t N = (size_t)H * W;
  float* mf = (float*)malloc(sizeof(float) * N);
  for (size_t n = 0; n < N; n++) mf[n] = (float)mpb[n];
  lattice L = {mf, W, H};
  int sdy[ORC_STENCIL_N], sdx[ORC_STENCIL_N];
  orc_stencil(sdy, sdx);
  const float sigma = 0.1f;
#pragma omp parallel
  {
    pt_ic* adj = (pt_ic*)malloc(sizeof(pt_ic) * wd * wd);
    pt_ic* scan = (pt_ic*)malloc(sizeof(pt_ic) * wd * wd);
    int* scnt = (int*)malloc(sizeof(int) * wd);
    pt_ic* scratch = (pt_ic*)malloc(sizeof(pt_ic) * (4 * wr + 2) * 4);
#pragma omp for schedule(dynamic, 4)
    for (int y = 0; y < H; y++)
      for (int x = 0; x < W; x++) {
        const int cnt = intervening(&L, 1.0f, x, y, wr, adj, scan, scnt, scratch);
        double* row = Wd + ((size_t)y * W + x) * ORC_STENCIL_N;
        int icIndex = 0;
        for (int k = 0; k < ORC_STENCIL_N; k++) {
          const int u = sdy[k], v = sdx[k];
          const int yy = y + u, xx = x + v;
          row[k] = 0;
          if (xx < 0 || xx >= W || yy < 0 || yy >= H) continue;
          while (icIndex < cnt && adj[icIndex].y < yy) icIndex++;
          while (icIndex < cnt && adj[icIndex].x < xx) icIndex++;
          float pss;
          if (u == 0 && v == 0) {
            pss = 1.0f;
          } else {
            float icsim = 0.0f;
            if (icIndex < cnt && adj[icIndex].x == xx && adj[icIndex].y == yy) {
              icsim = adj[icIndex].sim;
              icIndex++;
            }
            pss = c_ic_ss(1 - icsim);
          }
          const float val = (float)exp((double)(-(1 - pss) / sigma));
          row[k] = (double)val;
        }
      }
    free(adj);
    free(scan);
    free(scnt);
    free(scratch);
  }
  /* symmetrize: W(p,q) = W(q,p) = 0.5 (W(p,q)+W(q,p)) */
  int kneg[ORC_STENCIL_N];
  for (int k = 0; k < ORC_STENCIL_N; k++)
    for (int j = 0; j < ORC_STENCIL_N; j++)
      if (sdy[j] == -sdy[k] && sdx[j] == -sdx[k]) kneg[k] = j;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++)
      for (int k = ORC_STENCIL_N / 2 + 1; k < ORC_STENCIL_N; k++) {
        const int yy = y + sdy[k], xx = x + sdx[k];
        if (xx < 0 || xx >= W || yy < 0 || yy >= H) continue;
        double* a = Wd + ((size_t)y * W + x) * ORC_STENCIL_N + k;
        double* b = Wd + ((size_t)yy * W + xx) * ORC_STENCIL_N + kneg[k];
        const double m = 0.5 * (*a + *b);
        *a = m;
        *b = m;
      }
  free(mf);
}

/* ======================================================================= */
/* (d) FP64 eigensolver: Krylov-Schur (thick-restart Lanczos, full           */
/* reorthogonalisation) for the smallest eigenpairs of the normalised        */
/* Laplacian.  It stands in for Spectra's implicitly restarted               */
/* SymGEigsSolver<SMALLEST_MAGN, GEIGS_CHOLESKY> (src/spectralPb.cpp:221-245) */
/* on the full symmetric D-W (D2 fixed); it is pinned against Spectra in     */
/* tests on small graphs.                                                     */
/* ======================================================================= */

#define NCHUNK 64
static double pdot(const double* a, const double* b, size_t n) {
  double part[NCHUNK];
#pragma omp parallel for schedule(static)
  for (int c = 0; c < NCHUNK; c++) {
    const size_t lo = n * c / NCHUNK, hi = n * (c + 1) / NCHUNK;
    double s = 0;
    for (size_t i = lo; i < hi; i++) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0;
  for (int c = 0; c < NCHUNK; c++) s += part[c];
  return s;
}

/* One classical Gram-Schmidt pass of w against the nv basis vectors
 * V[0..nv) (each of length n): h[i] (+)= <V_i, w>, then w -= sum_i c_i V_i
 * with c the pass's own coefficients.  Both sweeps run over the same NCHUNK
 * fixed row chunks as pdot, so the sums do not depend on the thread count. */
static void cgs_pass(const double* V, int nv, double* w, size_t n, double* h, int accumulate) {
  double* part = (double*)malloc(sizeof(double) * NCHUNK * nv);
  double* c = (double*)malloc(sizeof(double) * nv);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NCHUNK; k++) {
    const size_t lo = n * k / NCHUNK, hi = n * (k + 1) / NCHUNK;
    for (int i = 0; i < nv; i++) {
      const double* vi = V + (size_t)i * n;
      double s = 0;
      for (size_t q = lo; q < hi; q++) s += vi[q] * w[q];
      part[(size_t)k * nv + i] = s;
    }
  }
  for (int i = 0; i < nv; i++) {
    double s = 0;
    for (int k = 0; k < NCHUNK; k++) s += part[(size_t)k * nv + i];
    c[i] = s;
    h[i] = accumulate ? h[i] + s : s;
  }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NCHUNK; k++) {
    const size_t lo = n * k / NCHUNK, hi = n * (k + 1) / NCHUNK;
    for (int i = 0; i < nv; i++) {
      const double* vi = V + (size_t)i * n;
      const double ci = c[i];
      for (size_t q = lo; q < hi; q++) w[q] -= ci * vi[q];
    }
  }
  free(c);
  free(part);
}

/* cyclic Jacobi eigenvalue algorithm for a dense symmetric n x n matrix
 * (Golub & Van Loan, Matrix Computations, sec. 8.5); ascending order */
static void jacobi_eig(double* A, int n, double* evals, double* V) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) V[i * n + j] = (i == j);
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0, tot = 0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        tot += A[i * n + j] * A[i * n + j];
        if (i != j) off += A[i * n + j] * A[i * n + j];
      }
    if (off <= 1e-30 * tot || off == 0) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = A[p * n + q];
        if (fabs(apq) < 1e-300) continue;
        const double app = A[p * n + p], aqq = A[q * n + q];
        const double theta = (aqq - app) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        const double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; k++) {
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  /* sort ascending (selection sort on columns) */
  for (int i = 0; i < n; i++) evals[i] = A[i * n + i];
  for (int i = 0; i < n; i++) {
    int m = i;
    for (int j = i + 1; j < n; j++)
      if (evals[j] < evals[m]) m = j;
    if (m != i) {
      double t = evals[i];
      evals[i] = evals[m];
      evals[m] = t;
      for (int k = 0; k < n; k++) {
        t = V[k * n + i];
        V[k * n + i] = V[k * n + m];
        V[k * n + m] = t;
      }
    }
  }
}

#ifndef ORC_KRYLOV_M
#define ORC_KRYLOV_M(nev) (4 * (nev) + 28)
#endif

typedef struct {
  const double* Wd;
  const double* dis; /* D^-1/2 */
  const double* diag;
  int H, W;
  int sdy[ORC_STENCIL_N], sdx[ORC_STENCIL_N];
} lap_op;

/* y = A x with A = I - D^-1/2 W D^-1/2 */
static void lap_apply(const lap_op* op, const double* x, double* y) {
  const int H = op->H, W = op->W;
#pragma omp parallel for schedule(static)
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++) {
      const size_t p = (size_t)r * W + c;
      const double* w = op->Wd + p * ORC_STENCIL_N;
      double acc = 0;
      for (int k = 0; k < ORC_STENCIL_N; k++) {
        if (k == ORC_STENCIL_N / 2) continue;
        const int rr = r + op->sdy[k], cc = c + op->sdx[k];
        if (rr < 0 || rr >= H || cc < 0 || cc >= W) continue;
        const size_t q = (size_t)rr * W + cc;
        acc += w[k] * op->dis[q] * x[q];
      }
      y[p] = op->diag[p] * x[p] - op->dis[p] * acc;
    }
}

int orc_eigs(const double* Wd, int H, int W, int nev, double tol, int maxit, int threads,
             double* evals, double* evecs, double* resid) {
  set_threads(threads);
  const size_t N = (size_t)H * W;
  lap_op op;
  op.Wd = Wd;
  op.H = H;
  op.W = W;
  orc_stencil(op.sdy, op.sdx);
  double* dis = (double*)malloc(sizeof(double) * N);
  double* diag = (double*)malloc(sizeof(double) * N);
  for (size_t p = 0; p < N; p++) {
    double d = 0;
    for (int k = 0; k < ORC_STENCIL_N; k++) d += Wd[p * ORC_STENCIL_N + k];
    dis[p] = 1.0 / sqrt(d);
    diag[p] = (d - Wd[p * ORC_STENCIL_N + ORC_STENCIL_N / 2]) / d;
  }
  op.dis = dis;
  op.diag = diag;
  int m = ORC_KRYLOV_M(nev);
  if ((size_t)m > N) m = (int)N;
  int keep = nev + (m - nev) / 2;
  double* V = (double*)malloc(sizeof(double) * N * (m + 1));
  double* w = (double*)malloc(sizeof(double) * N);
  double* T = (double*)calloc((size_t)m * m, sizeof(double));
  double* Tc = (double*)malloc(sizeof(double) * m * m);
  double* Y = (double*)malloc(sizeof(double) * m * m);
  double* th = (double*)malloc(sizeof(double) * m);
  double* h = (double*)malloc(sizeof(double) * (m + 1));
  /* deterministic start vector: a Weyl sequence (not the trivial D^1/2 1) */
  {
    double nrm = 0;
    for (size_t i = 0; i < N; i++) {
      double t = fmod(0.5 + (double)i * 0.6180339887498949, 1.0) - 0.5;
      V[i] = t;
      nrm += t * t;
    }
    nrm = sqrt(nrm);
    for (size_t i = 0; i < N; i++) V[i] /= nrm;
  }
  int k = 0, matvecs = 0, converged = 0;
  double beta = 0;
  for (int it = 0; it < maxit; it++) {
    for (int j = k; j < m; j++) {
      double* vj = V + (size_t)j * N;
      lap_apply(&op, vj, w);
      matvecs++;
      /* full reorthogonalisation: classical Gram-Schmidt, repeated once
       * when the pass removed more than 1 - 1/sqrt(2) of the norm (the DGKS
       * test, Daniel, Gragg, Kaufman & Stewart 1976) */
      {
        const double n0 = sqrt(pdot(w, w, N));
        cgs_pass(V, j + 1, w, N, h, 0);
        if (sqrt(pdot(w, w, N)) < 0.7071067811865476 * n0) cgs_pass(V, j + 1, w, N, h, 1);
      }
      for (int i = 0; i <= j; i++) {
        T[i * m + j] = h[i];
        T[j * m + i] = h[i];
      }
      beta = sqrt(pdot(w, w, N));
      double* vn = V + (size_t)(j + 1) * N;
      if (beta < 1e-300) beta = 1e-300;
#pragma omp parallel for schedule(static)
      for (long q = 0; q < (long)N; q++) vn[q] = w[q] / beta;
    }
    memcpy(Tc, T, sizeof(double) * m * m);
    /* symmetrise the projected matrix before the dense solve */
    for (int i = 0; i < m; i++)
      for (int j = i + 1; j < m; j++) Tc[i * m + j] = Tc[j * m + i] = 0.5 * (Tc[i * m + j] + Tc[j * m + i]);
    jacobi_eig(Tc, m, th, Y);
    int nconv = 0;
    for (int i = 0; i < nev; i++) {
      const double r = fabs(beta * Y[(m - 1) * m + i]);
      if (resid) resid[i] = r;
      if (r <= tol) nconv++;
    }
    const int done = (nconv >= nev) || (it == maxit - 1);
    const int nk = done ? nev : keep;
    /* Ritz vectors: V[:, 0..nk) <- V[:, 0..m) Y[:, 0..nk) */
    double* X = (double*)malloc(sizeof(double) * N * nk);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)N; q++)
      for (int c = 0; c < nk; c++) {
        double s = 0;
        for (int i = 0; i < m; i++) s += V[(size_t)i * N + q] * Y[i * m + c];
        X[(size_t)c * N + q] = s;
      }
    if (done) {
      for (int i = 0; i < nev; i++) evals[i] = th[i];
      memcpy(evecs, X, sizeof(double) * N * nev);
      free(X);
      converged = (nconv >= nev);
      break;
    }
    memcpy(V, X, sizeof(double) * N * nk);
    memcpy(V + (size_t)nk * N, V + (size_t)m * N, sizeof(double) * N);
    free(X);
    memset(T, 0, sizeof(double) * m * m);
    for (int i = 0; i < nk; i++) {
      T[i * m + i] = th[i];
      T[i * m + nk] = T[nk * m + i] = beta * Y[(m - 1) * m + i];
    }
    k = nk;
  }
  free(dis);
  free(diag);
  free(V);
  free(w);
  free(T);
  free(Tc);
  free(Y);
  free(th);
  free(h);
  return converged ? matvecs : -1;
}

/* ======================================================================= */
/* (e) sPb + gPb                                                            */
/* ======================================================================= */

/* Oriented first derivative of a Gaussian (sigma 1, support 3) as Berkeley's
 * oeFilter computes it: 70x70 sub-samples binned into the 7x7 grid by their
 * unrotated position, the separable function evaluated on the rotated grid
 * through a finer lookup domain, zero mean, unit L1 norm.  The C++ port in
 * src/oeFilter.cpp:21-196 bins on the rotated grid (:53-58), reads sy for sv
 * (:62), leaves the accumulator uninitialised (:145) and visits only 49 of the
 * 4900 samples (:146-153) (D3); this is the algorithm it ports.  f is indexed
 * f[a*7+b] with a the sampling-grid x bin and b the y bin (MATLAB reshape),
 * and is used as a correlation kernel with a as the row offset. */
void orc_oefilter(double theta, double* out) {
  const double sigma = 1.0;
  const int support = 3;
  const int hsz = (int)ceil(support * sigma), sz = 2 * hsz + 1;
  const int maxsamples = 1000, maxrate = 10, frate = 10;
  int rate = maxsamples / sz;
  if (rate < 1) rate = 1;
  if (rate > maxrate) rate = maxrate;
  const int samples = sz * rate;
  const double r = floor(sz / 2.0) + 0.5 * (1 - 1.0 / rate);
  double* dom = (double*)malloc(sizeof(double) * samples);
  for (int i = 0; i < samples; i++) dom[i] = -r + (2 * r) * i / (samples - 1); /* linspace */
  const double R = r * sqrt(2.0) * 1.01;
  int fsamples = (int)ceil(R * rate * frate);
  fsamples = fsamples + (fsamples + 1) % 2;
  double* fx = (double*)malloc(sizeof(double) * fsamples);
  double* fy = (double*)malloc(sizeof(double) * fsamples);
  for (int i = 0; i < fsamples; i++) {
    const double t = -R + (2 * R) * i / (fsamples - 1);
    fx[i] = exp(-t * t / (2 * sigma * sigma));
    fy[i] = exp(-t * t / (2 * sigma * sigma)) * (-t / (sigma * sigma));
  }
  const double gap = 2 * R / (fsamples - 1);
  double acc[49];
  for (int i = 0; i < sz * sz; i++) acc[i] = 0;
  const double st = sin(theta), ct = cos(theta);
  for (int i = 0; i < samples; i++)     /* meshgrid row: sy = dom[i] */
    for (int j = 0; j < samples; j++) { /* meshgrid col: sx = dom[j] */
      const double sx = dom[j], sy = dom[i];
      const int mx = (int)round(sx), my = (int)round(sy);
      const int memb = (mx + hsz + 1) + (my + hsz) * sz; /* 1-based, column-major */
      if (memb < 1 || memb > sz * sz) continue;
      const double su = sx * st + sy * ct, sv = sx * ct - sy * st;
      const int xi = (int)round(su / gap) + fsamples / 2;
      const int yi = (int)round(sv / gap) + fsamples / 2;
      const double f = fx[xi] * fy[yi];
      const int li = memb - 1;
      const int a = li % sz, b = li / sz; /* column-major: a = row, b = column */
      acc[a * sz + b] += f;
    }
  double mean = 0;
  for (int i = 0; i < sz * sz; i++) mean += acc[i];
  mean /= sz * sz;
  double s = 0;
  for (int i = 0; i < sz * sz; i++) {
    acc[i] -= mean;
    s += fabs(acc[i]);
  }
  for (int i = 0; i < sz * sz; i++) out[i] = s > 0 ? acc[i] / s : acc[i];
  free(dom);
  free(fx);
  free(fy);
}

/* src/spectralPb.cpp:269-322: eigenvectors 1..nvec-1 (ascending, D11),
 * v = D^-1/2 y min-max normalised then divided by sqrt(lambda); 8 oriented
 * filters at theta = o*pi/8 applied with filter2D semantics (correlation,
 * BORDER_REFLECT_101) and |.| accumulated into slot ch_per[o].  The
 * reference's ch_per {3,2,1,0,7,6,5,4} (spectralPb.cpp:289) goes with its own
 * defective filter; with the fixed filter (D3) the slot that makes sPb_o
 * peak at the same orientation as the local cues is (4 - o) mod 8. */
void orc_spb(const double* evals, const double* evecs, const double* dis, int H, int W, int nvec,
             double* spb) {
  static const int ch_per[8] = {4, 3, 2, 1, 0, 7, 6, 5};
  const size_t N = (size_t)H * W;
  double filt[8][49];
  for (int o = 0; o < 8; o++) orc_oefilter((REF_PI / 8) * (double)o, filt[o]);
  memset(spb, 0, sizeof(double) * 8 * N);
  double* v = (double*)malloc(sizeof(double) * N);
  for (int i = 1; i < nvec; i++) {
    if (!(evals[i] > DBL_EPSILON)) continue;
    double mn = INFINITY, mx = -INFINITY;
    for (size_t p = 0; p < N; p++) {
      v[p] = evecs[(size_t)i * N + p] * dis[p];
      if (v[p] < mn) mn = v[p];
      if (v[p] > mx) mx = v[p];
    }
    const double sq = sqrt(evals[i]);
    for (size_t p = 0; p < N; p++) v[p] = ((v[p] - mn) / (mx - mn)) / sq;
    for (int o = 0; o < 8; o++) {
      double* dst = spb + (size_t)ch_per[o] * N;
#pragma omp parallel for schedule(static)
      for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
          double acc = 0;
          for (int a = 0; a < 7; a++) {
            const double* row = v + (size_t)refl101(y + a - 3, H) * W;
            for (int b = 0; b < 7; b++) acc += filt[o][a * 7 + b] * row[refl101(x + b - 3, W)];
          }
          dst[(size_t)y * W + x] += fabs(acc);
        }
    }
  }
  free(v);
}

/* weight sets: CPU mPb (multiscalePb.cpp:19-26), CPU gPb (globalPb.cpp:31-36),
 * GPU mPb coefficients and gPb weights (combine.cu:16-21, globalPb.cu:13) */
static const double W_MPB_CPU[12] = {0.0146, 0.0145, 0.0163, 0.0210, 0.0243, 0.0287,
                                     0.0166, 0.0185, 0.0204, 0.0101, 0.0111, 0.0141};
static const double W_GPB_CPU[13] = {0, 0, 0.0039, 0.0050, 0.0058, 0.0069, 0.0040,
                                     0.0044, 0.0049, 0.0024, 0.0027, 0.0170, 0.0074};
static const double W_MPB_GPU[12] = {0.0123, 0.0110, 0.0117, 0.0169, 0.0176, 0.0198,
                                     0.0138, 0.0138, 0.0145, 0.0144, 0.0149, 0.0158};
static const double W_GPB_GPU[13] = {0, 0, 0.0028, 0.0041, 0.0042, 0.0047, 0.0033,
                                     0.0033, 0.0035, 0.0035, 0.0035, 0.0188, 0.0139};

/* GlobalPbWithNmax (src/globalPb.cpp:128-245) with the full oracle chain; in
 * Damascene mode the gPb planes follow CalcGPb + SigmoidGpbAll
 * (globalPb.cu:5-49, skeleton.cu:229-249). Returns eigensolver matvecs. */
int orc_globalpb(const uint8_t* bgr, int H, int W, const float* codebook, int K, const orc_params* p,
                 double* gpb_o, double* nmax, uint8_t* texton_out, double* cues_out, double* mpb_out,
                 double* Wd_out, double* evals_out, double* evecs_out, double* spb_out) {
  set_threads(p->threads);
  const size_t N = (size_t)H * W;
  uint8_t* grey = (uint8_t*)malloc(N);
  uint8_t* tex = (uint8_t*)malloc(N);
  orc_grey_bgr(bgr, H, W, grey);
  orc_texton_map(grey, H, W, codebook, K, p->fix_argmin, tex, NULL);
  if (texton_out) memcpy(texton_out, tex, N);
  double* cues = cues_out ? cues_out : (double*)malloc(sizeof(double) * 12 * 8 * N);
  orc_local_cues(bgr, tex, H, W, p, cues);
  const double* wm = p->damascene_weights ? W_MPB_GPU : W_MPB_CPU;
  const double* wg = p->damascene_weights ? W_GPB_GPU : W_GPB_CPU;
  double* mo = (double*)malloc(sizeof(double) * 8 * N);
  orc_combine(cues, H, W, wm, mo);
  double* mpb = mpb_out ? mpb_out : (double*)malloc(sizeof(double) * N);
  orc_nonmax(mo, H, W, p->fix_clip_scale, mpb);
  double* Wd = Wd_out ? Wd_out : (double*)malloc(sizeof(double) * N * ORC_STENCIL_N);
  orc_buildW(mpb, H, W, Wd, p->threads);
  const int nvec = p->nvec;
  double* ev = (double*)malloc(sizeof(double) * nvec);
  double* evec = evecs_out ? evecs_out : (double*)malloc(sizeof(double) * nvec * N);
  const int iters = orc_eigs(Wd, H, W, nvec, p->eig_tol, p->eig_maxit, p->threads, ev, evec, NULL);
  if (evals_out) memcpy(evals_out, ev, sizeof(double) * nvec);
  double* dis = (double*)malloc(sizeof(double) * N);
  for (size_t q = 0; q < N; q++) {
    double d = 0;
    for (int k = 0; k < ORC_STENCIL_N; k++) d += Wd[q * ORC_STENCIL_N + k];
    dis[q] = 1.0 / sqrt(d);
  }
  double* spb = spb_out ? spb_out : (double*)malloc(sizeof(double) * 8 * N);
  orc_spb(ev, evec, dis, H, W, nvec, spb);
  double* gp = gpb_o ? gpb_o : (double*)malloc(sizeof(double) * 8 * N);
  for (int o = 0; o < 8; o++)
    for (size_t q = 0; q < N; q++) {
      double acc = wg[0] * cues[(size_t)(0 * 8 + o) * N + q];
      for (int k = 1; k < 12; k++) acc = acc + wg[k] * cues[(size_t)(k * 8 + o) * N + q];
      acc = acc + wg[12] * spb[(size_t)o * N + q];
      gp[(size_t)o * N + q] = acc;
    }
  if (nmax) {
    for (size_t q = 0; q < N; q++) {
      double m = p->damascene_weights ? -200 : 0;
      for (int o = 0; o < 8; o++) {
        const double g = gp[(size_t)o * N + q];
        if (p->damascene_weights) {
          if (g > m) m = g;
        } else if (fabs(g) > m) {
          m = fabs(g);
        }
      }
      if (p->damascene_weights && !(mpb[q] > 0.05)) m = 0;
      nmax[q] = m;
    }
  }
  if (p->sigmoid)
    for (size_t q = 0; q < 8 * N; q++) {
      double v = gp[q];
      v = (v * 1.2 > 1) ? 1 : v * 1.2;
      if (v < 0) v = 0;
      v = 1.0 / (1.0 + exp(2.6433 - 10.7998 * v));
      gp[q] = (v - 0.0667) / 0.9333;
    }
  if (!gpb_o) free(gp);
  if (!spb_out) free(spb);
  free(dis);
  free(ev);
  if (!evecs_out) free(evec);
  if (!Wd_out) free(Wd);
  if (!mpb_out) free(mpb);
  free(mo);
  if (!cues_out) free(cues);
  free(grey);
  free(tex);
  return iters;
}
