// ucm_dev.h -- device scratch and launchers of the OWT-UCM stages (k_ucm.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gpb {

struct UcmImage {
  int H, W;
  long long pix;  // first pixel of the image in the per-pixel arrays
  int row0;       // first row in the per-row arrays
};

struct UcmScratch {
  unsigned* mm;        // ordered min, max of pb
  float* pb;           // N
  uint8_t* q;          // N
  int32_t* off;        // H x 257
  uint16_t* cols;      // N
  UcmImage* img;       // this image's entry of the batch's image table
  int32_t* ws;         // N
  uint8_t* bw;         // N
  float* wswt;         // N
  int32_t* paint_pix;  // painted pixels
  uint8_t* paint_ori;  // their orientation planes
  float* pb2;          // 4N
  int32_t* rowcnt;     // 2H
  int32_t* nart;       // 1
  int32_t* art;        // 4N at most
  int32_t* par;        // 4N
  int32_t* rank;       // 4N
  int32_t* bsum;       // 4N / 4096 + 1
  int32_t* nreg;       // 1
  int32_t* labels;     // N
  float* wswt2;        // (2H+1)(2W+1)
};

// per image: max over orientations, quantisation, per-row level sort
cudaError_t ucm_prepare(const float* d_orient, int H, int W, UcmScratch& s, cudaStream_t st);
// all images of a batch: flooding (one CTA each) and the watershed-pixel map;
// base is image 0's view, whose arrays start the batch's concatenated ones
cudaError_t ucm_flood(int nimg, long long total_pix, const UcmScratch& base, cudaStream_t st);
cudaError_t ucm_paint(const float* d_orient, int H, int W, int npaint, UcmScratch& s, cudaStream_t st);
cudaError_t ucm_mid(int H, int W, UcmScratch& s, cudaStream_t st);

}  // namespace gpb
