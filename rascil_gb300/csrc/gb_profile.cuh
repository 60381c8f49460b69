// Kernel profiling scopes (see gb_profile.cu).
#pragma once

#include <cuda_runtime.h>

namespace gb {

enum ProfId {
  kProfWrange = 0,
  kProfCountKernel,
  kProfScan,
  kProfScatter,
  kProfChunks,
  kProfCorr,
  kProfPrepVis,
  kProfGrid,
  kProfFftInv,
  kProfScreenAcc,
  kProfFinalize,
  kProfPrepImage,
  kProfScreenPad,
  kProfFftFwd,
  kProfDegrid,
  kProfDftComp,
  kProfDftPix,
  kProfColInvA,
  kProfColInvB,
  kProfColPredA,
  kProfColPredB,
  kProfZeroMargins,
  kProfRowsInv,
  kProfRowsFwd,
  kProfGridZero,
  kProfWeightGrid,
  kProfWeightSums,
  kProfWeightApply,
  kProfWeightRecip,
  kProfRotate,
  kProfCount
};

extern const char *kProfNames[kProfCount];

// True while process-wide profiling is enabled.
bool prof_on();

// Records an event pair around its lifetime on stream `s` when profiling
// is on; `bytes` is the algorithmic traffic of the enclosed launch.
class ProfScope {
 public:
  ProfScope(int id, cudaStream_t s, double bytes);
  ~ProfScope();

 private:
  int id_;
  cudaStream_t s_;
  double bytes_;
  bool active_ = false;
  cudaEvent_t a_ = nullptr;
};

}  // namespace gb
