/*
 * gpb_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU restatement of the reference's CPU gPb path (globalPb / det_mPb /
 * multiscalePb / spectralPb of yanyp/UCM-MPI-GPU, the src/ C++ files, plus the Berkeley
 * lib_image and buildW cores it calls).  It is the checker for the CUDA
 * library and the timed CPU baseline; the product never links or calls it.
 *
 * Layout conventions: images are row-major H x W (pixel (y,x) at y*W+x);
 * per-orientation planes are stacked [o][y][x]; the 12 cue maps are stacked
 * [cue][o][y][x] in the reference order bg1 bg2 bg3 cga1 cga2 cga3 cgb1 cgb2
 * cgb3 tg1 tg2 tg3 (src/multiscalePb.cpp:44-58).
 */
#ifndef GPB_ORACLE_H_
#define GPB_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NORI 8
#define ORC_NCUE 12
#define ORC_NSCHMID 13
#define ORC_SCHMID_SUP 49
#define ORC_STENCIL_R 5
#define ORC_STENCIL_N 81

/* Named fixes of the reference CPU path (1 = fixed, the default). */
typedef struct {
  int fix_rb_swap;     /* D1: det_mPb.cpp:10-19 passes B,G,R as r,g,b            */
  int fix_argmin;      /* D4: SPFeatures.cpp:328-339 never updates minDistance    */
  int nvec;            /* D5: 17 on the CPU path, 9 on the GPU path            */
  int fix_clip_scale;  /* D7: multiscalePb.cpp:252-261 forgets the x1.2          */
  int fix_eig_order;   /* D11: Spectra returns descending order, sPb skips [0]  */
  int damascene_weights; /* D10: 0 = CPU weight sets, 1 = GPU (combine.cu)      */
  int sigmoid;         /* Damascene SigmoidGpbAll (skeleton.cu:229-249)          */
  double eig_tol;      /* residual tolerance of the FP64 Krylov-Schur solver     */
  int eig_maxit;       /* max restarts                                          */
  int threads;         /* 0 = all                                                */
} orc_params;

void orc_default_params(orc_params* p);

/* --- (a) textons ------------------------------------------------------- */
void orc_schmid_bank(double* F /* 13 x 49 x 49 */);
void orc_grey_bgr(const uint8_t* bgr, int H, int W, uint8_t* grey);
/* responses_opt (13 x H x W, may be NULL) */
void orc_texton_map(const uint8_t* grey, int H, int W, const float* codebook /* 13 x K */,
                    int K, int fix_argmin, uint8_t* labels, double* responses_opt);
int orc_schmid_rings(int* ring_of_offset /* 49*49 */, int* ring_s /* out, <= 1153 */);

/* --- (b) local cues ---------------------------------------------------- */
void orc_lab_bins(const uint8_t* bgr, int H, int W, int nbins, int fix_rb, uint8_t* Lq,
                  uint8_t* aq, uint8_t* bq);
void orc_mirror_u8(const uint8_t* src, int H, int W, int b, uint8_t* dst);
int orc_slice_index(int r, int drow, int dcol);
int orc_gaussian_kernel(double sigma, double* k /* >= 2*ceil(3 sigma)+1 */);
/* labels padded by `border`; out = 8 x H x W for the interior; counts_opt =
 * optional raw integer slice counts for every interior pixel (16 x nbins each) */
int orc_hist_gradient(const uint8_t* lab_padded, int Hp, int Wp, int border, int r,
                      const double* kern, int klen, double* out, int32_t* counts_opt,
                      int threads);
/* all 12 cue maps (12 x 8 x H x W) from the image and the texton labels */
void orc_local_cues(const uint8_t* bgr, const uint8_t* texton, int H, int W,
                    const orc_params* p, double* cues);
void orc_combine(const double* cues, int H, int W, const double* w12, double* out /* 8xHxW */);
void orc_nonmax(const double* mpb_o, int H, int W, int fix_clip_scale, double* mpb);

/* --- (c) buildW -------------------------------------------------------- */
void orc_stencil(int* dy, int* dx /* 81 each, scanline order */);
/* W (N x 81, symmetrized, 0 where the neighbour is outside the image) */
void orc_buildW(const double* mpb, int H, int W, double* Wd, int threads);

/* --- (d) eigensolver --------------------------------------------------- */
/* smallest nev eigenpairs of A = D^-1/2 (D-W) D^-1/2; evecs (nev x N) are the
 * unit eigenvectors y of A; returns iterations (matvecs) or -1 */
int orc_eigs(const double* Wd, int H, int W, int nev, double tol, int maxit, int threads,
             double* evals, double* evecs, double* resid_opt);
void orc_oefilter(double theta, double* f /* 7 x 7 */);

/* --- (e) sPb + gPb ----------------------------------------------------- */
void orc_spb(const double* evals, const double* evecs /* A's unit eigvecs */,
             const double* dinv_sqrt, int H, int W, int nvec, double* spb /* 8 x H x W */);
/* whole pipeline; any output may be NULL */
int orc_globalpb(const uint8_t* bgr, int H, int W, const float* codebook, int K,
                 const orc_params* p, double* gpb_o /* 8xHxW */, double* nmax /* HxW */,
                 uint8_t* texton_out, double* cues_out, double* mpb_out, double* Wd_out,
                 double* evals_out, double* evecs_out, double* spb_out);

#ifdef __cplusplus
}
#endif
#endif
