// kernels.h -- launchers and table uploads of the libgpb kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gpb_internal.h"

namespace gpb {

// k_front.cu
void upload_front(const HostTables& t, cudaStream_t s);
void upload_codebook(const float* cb, int K, cudaStream_t s);
cudaError_t launch_convert(const uint32_t* packed, long long n, uint8_t* grey, uint32_t* lab4,
                           cudaStream_t s);
// the Lab bins of all 2^24 colours (a 64 MB table), and the convert step as
// a gather from it
cudaError_t launch_lab_table(uint32_t* table, cudaStream_t s);
cudaError_t launch_convert_lut(const uint32_t* packed, long long n, const uint32_t* table, uint8_t* grey,
                               uint32_t* lab4, cudaStream_t s);
// variant 0, 1, 2: 32, 64 or 128 threads per 16 x 16 tile (identical labels)
constexpr int kTextonVariants = 3;
cudaError_t launch_texton(const PatchDev* patches, const int4* work, int nwork, const uint8_t* grey,
                          uint32_t* lab4, int* repair_list, int* repair_count, int repair_cap,
                          cudaStream_t s, int variant = 1);
cudaError_t launch_texton_repair(const PatchDev* patches, const uint8_t* grey, uint32_t* lab4,
                                 const int* repair_list, const int* repair_count, int repair_cap,
                                 const double* k32_ring, const int* ring_of, int n_rings,
                                 cudaStream_t s);

// k_cues.cu
constexpr int kCueTileH = 8, kCueTileW = 16;
void upload_cues(const HostTables& t, cudaStream_t s);
cudaError_t launch_maxlabel(const PatchDev* patches, int npatch, const uint32_t* lab4, int* nbins,
                            cudaStream_t s);
cudaError_t launch_cues(const PatchDev* patches, const int4* work, int nwork, const uint32_t* lab4,
                        const int* nbins, float* mpbo, float* go, float* raw, uint8_t* counts, cudaStream_t s);
cudaError_t launch_nms(const PatchDev* patches, const int4* work, int nwork, const float* mpbo,
                       float* mpb, cudaStream_t s);

// k_buildw.cu
void upload_buildw(const HostTables& t, cudaStream_t s);
cudaError_t launch_buildw(const PatchDev* patches, const int4* work, int nwork, const float* mpb,
                          const IcPath* ic, float* wsym_up, float* deg, long long lvec,
                          cudaStream_t s);
cudaError_t launch_scale(const PatchDev* patches, const int4* work, int nwork, const float* wsym_up,
                         const float* deg, float* a_up, float* a_diag, float* dis, long long lvec,
                         float* wfull, cudaStream_t s);

// k_spb.cu
void upload_spb(const HostTables& t, cudaStream_t s);
cudaError_t launch_minmax(const PatchDev* patches, int npatch, const float* evecs, long long lvec,
                          const float* dis, int nvec, float* mm, cudaStream_t s);
cudaError_t launch_spb(const PatchDev* patches, const int4* work, int nwork, const float* evecs,
                       long long lvec, const float* dis, const float* evals, const float* mm,
                       int nvec, const float* go, const float* mpb, int compat, float* spb_out,
                       float* gpbo_out, float* out_nmax, float* out_orient, cudaStream_t s);

// k_stitch.cu: a sub-box (x, y, w, h, patch coordinates) of a patch placed
// at (ox, oy) in the image
struct StitchBox {
  int ox, oy, x, y, w, h;
};
cudaError_t launch_stitch_copy(const PatchDev* patches, int pi, const float* nmax, const float* orient, int colmajor,
                               const StitchBox& bx, int img_w, int img_h, float* out_nmax, float* out_orient,
                               cudaStream_t s);
cudaError_t launch_stitch_acc(const PatchDev* patches, int pi, long long npix, const float* nmax, const float* orient,
                              int colmajor, const StitchBox& bx, int img_w, int img_h, float ramp, float* acc,
                              cudaStream_t s);
cudaError_t launch_stitch_norm(const float* acc, long long plane, float* out_nmax, float* out_orient, cudaStream_t s);

// k_spfeat.cu
cudaError_t launch_sp_features(const PatchDev* patches, int pi, long long npix, const int32_t* labels, int n,
                               const uint32_t* lab4, const uint8_t* grey, const uint32_t* packed, int bin_step,
                               int K, int nbins, uint32_t* counts, unsigned long long* csum, double* out,
                               cudaStream_t s);

}  // namespace gpb
