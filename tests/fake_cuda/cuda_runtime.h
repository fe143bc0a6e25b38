// A stand-in for the few CUDA runtime calls autotune.h makes, so that its
// bookkeeping can be checked by the host compiler alone: an event records
// the value of a clock that the check advances by hand.
#pragma once
#include <stdlib.h>

typedef void* cudaStream_t;
struct FakeCudaEvent {
  double t;
  bool recorded;
};
typedef FakeCudaEvent* cudaEvent_t;
enum cudaError_t { cudaSuccess = 0, cudaErrorNotReady = 600 };

inline double& fake_cuda_clock() {
  static double t = 0;
  return t;
}
inline cudaError_t cudaEventCreate(cudaEvent_t* e) {
  *e = new FakeCudaEvent{0, false};
  return cudaSuccess;
}
inline cudaError_t cudaEventDestroy(cudaEvent_t e) {
  delete e;
  return cudaSuccess;
}
inline cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t) {
  e->t = fake_cuda_clock();
  e->recorded = true;
  return cudaSuccess;
}
inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
  if (!a->recorded || !b->recorded) return cudaErrorNotReady;
  *ms = (float)(b->t - a->t);
  return cudaSuccess;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
