// Launcher for the reference's DFT kernel (oracle/_ref/dft_kernel_ref.cu,
// extracted from the reference at build time): same launch shape as
// dft_gpu_raw_kernel (rascil/processing_components/imaging/dft.py:313-331).
#include <cuda_runtime.h>
#include "../_ref/dft_kernel_ref.cu"

extern "C" int ref_dft_launch(int ncomp, int npol, int nchan, int nbl, int ntimes,
                              const void *dirs, const void *fluxes, const void *uvw_lambda,
                              void *vis, void *stream) {
  dim3 threads(128, 2, 2);
  dim3 blocks((nbl + 127) / 128, (nchan + 1) / 2, (ntimes + 1) / 2);
  dft_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(
      ncomp, npol, nchan, nbl, ntimes, (const double3 *)dirs, (const complex<double> *)fluxes,
      (const double3 *)uvw_lambda, (complex<double> *)vis);
  return (int)cudaGetLastError();
}
