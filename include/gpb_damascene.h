/*
 * gpb_damascene.h -- drop-in replacements, with the original C++ signatures,
 * for the engine entry points that GlobalPbCuda (src/globalPb.cpp:247-313)
 * calls:
 *
 *   damascene/include/globalPb.h:35
 *     void computeGPb(unsigned int rank, unsigned int width, unsigned int height,
 *                     unsigned int* data, float** hostGPb, float** hostGPbAllConcat);
 *   damascene/include/globalPb.h:44
 *     int getCudaDeviceCount();
 *
 * Semantics kept from damascene/src/damascene.cu:242-661: device
 * rank % deviceCount; data[y*width+x] = B<<16|G<<8|R; *hostGPb (H*W,
 * row-major) and *hostGPbAllConcat (8*H*W, plane i = orientation
 * {4,5,6,7,0,1,2,3}[i], column-major, sigmoid-rescaled) are malloc()ed for
 * the caller to free(); on failure a C++ exception of type int64_t (value 1)
 * is thrown, which GlobalPbCuda catches (src/globalPb.cpp:283-286).
 *
 * The texton codebook the reference reads per image
 * (<piece>_texton_codebook.yml, src/SPFeatures.cpp:300-313) is taken from the
 * file named by the environment variable GPB_TEXTON_CODEBOOK, or set with
 * gpbSetTextonCodebook() before the first call.
 */
#ifndef GPB_DAMASCENE_H_
#define GPB_DAMASCENE_H_

void computeGPb(unsigned int rank, unsigned int width, unsigned int height, unsigned int* data,
                float** hostGPb, float** hostGPbAllConcat);
int getCudaDeviceCount();
/* 13 x K FP32 codebook (row-major, K <= 32) for every later computeGPb call */
int gpbSetTextonCodebook(const float* codebook, int K);

#endif
