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
// is on; `bytes` is the algorithmic traffic of the enclosed launch and
// `updates` (gridding / degridding kernels only) the number of
// (item, polarisation, grid cell) kernel-weighted updates it performs.
class ProfScope {
 public:
  ProfScope(int id, cudaStream_t s, double bytes, double updates = 0.0);
  ~ProfScope();

 private:
  int id_;
  cudaStream_t s_;
  double bytes_, updates_;
  bool active_ = false;
  cudaEvent_t a_ = nullptr;
};

}  // namespace gb
