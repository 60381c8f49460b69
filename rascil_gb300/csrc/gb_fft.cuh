// Column transforms of the FP32 form (gb_fft.cu) and the row order they
// leave in predict grids.
#pragma once

#include "gb_plan.cuh"

namespace gb {

// Bits of a plan's device status word.
constexpr uint32_t kErrTmaTimeout = 1u;  // a TMA completion wait ran past its limit

struct ColGeom {
  int n, N1, N2;   // column length n = N1 N2
  int ox, oy;      // image block offset in the grid
  int nx, ny;      // image size
  int64_t plane;   // ngx * ngy
  int ngx;
  // (plane, row tile) occupancy: invert step A takes rows outside it as zero
  const uint8_t *mask;
  int b0, NP, T, ntv;
  __device__ __forceinline__ bool row_used(int pp, int q) const {
    return !mask || mask[(int64_t)(b0 + pp / NP) * ntv + q / T];
  }
};

// True when a column of length n has a supported split n = N1 N2
// (power of two, 256 <= n <= 32768; N1 <= 128, N2 <= 256).
bool column_split(int n, int &N1, int &N2);
ColGeom col_geom(const Geom &g);
RowPerm row_perm(const gb_plan *p);

// Shared-memory opt-ins of the column kernels (plan creation).
int setup_col_kernels(gb_plan *p);
// Zero the rows of the batch buffer that the occupancy mask marks as used
// (the others are never read); column mode's replacement for a memset.
int run_zero_rows(gb_plan *p, void *grid, int b0, int nb, cudaStream_t s);
// Row lengths with a k_rows instantiation (4096, 8192, 16384).
bool row_kernel_fits(int n);
// Occupancy / opt-ins of the row kernels (plan creation).
int setup_row_kernels(gb_plan *p);
// Row transforms of nb planes x NP pols of the batch buffer: dir > 0
// invert (e^{+}, full rows in, image columns out), dir < 0 predict (e^{-},
// image columns in, full rows out); rows empty in the occupancy mask are
// skipped.
int run_rows(gb_plan *p, void *grid, int b0, int nb, int dir, cudaStream_t s);
// Invert: step A in place, then step B fused with the w-screen and the
// image accumulation (first != 0 starts acc from zero).
int run_cols_invert(gb_plan *p, void *grid, int b0, int nb, float *acc, int first,
                    cudaStream_t s);
// Predict: the screened image through both column steps into the grid's
// central columns (permuted rows), and zeros in the other columns.
int run_cols_predict(gb_plan *p, const float *img, int b0, int nb, void *grid, cudaStream_t s);

}  // namespace gb
