// k_static.h -- the texton stage on a fixed device scratch area (k_static.cu)
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gpb {

// largest image of gpb_texton_labels_static: 2^20 pixels (1024 x 1024), at
// most 8192 tiles of 16 x 16
constexpr int kStaticMaxPix = 1 << 20;
constexpr int kStaticMaxTiles = 8192;

size_t static_scratch_bytes();
cudaError_t static_scratch(unsigned char** base);
cudaError_t launch_texton_static(const uint32_t* packed, int W, int H, uint32_t* lab4, const double* k32_ring,
                                 const int* ring_of, int n_rings, cudaStream_t s);

}  // namespace gpb
