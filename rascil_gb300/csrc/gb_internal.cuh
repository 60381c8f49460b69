// Internal definitions shared by the gridder's translation units.
//
// Algorithm (restated from the published method behind ducc0.wgridder,
// which rascil/processing_components/imaging/ng.py:91-120,232-275 calls):
// exponential-of-semicircle (ES) kernel gridding on a sigma-oversampled
// uv grid, w-stacking with the same kernel along w, 2-D FFTs per w-plane,
// a w-screen per plane and a final correction by the kernel's Fourier
// transform.  The data layout is GB300-first:
//
//  * visibilities are addressed as items (row, channel); the plan sorts
//    them once into buckets (w-slab, uv-tile) and stores one compact
//    record per item in bucket order (ItemF / ItemD);
//  * uv-grids are [plane][pol][v][u] complex, u fastest, so a pixel row of
//    the image is a contiguous run of the FFT output;
//  * grids carry a (-1)^(p+q) checkerboard, which moves the image to the
//    central block of the FFT output (no fftshift pass);
//  * images are [pol][y][x] internally (RASCIL's order), x fastest.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rascil_gb300.h"

namespace gb {

constexpr double kSpeedOfLight = 299792458.0;  // rascil/phyconst.py:6
constexpr int kThreads = 256;                   // block size of the tile kernels
constexpr int kWarps = kThreads / 32;
constexpr int kChunkItems = 256;                // items per work chunk
constexpr int kMaxSupport = 16;
constexpr int kMaxQuad = 48;                    // Gauss-Legendre nodes (half interval)
constexpr int kMaxSlab = 128;                   // w-planes per bucket slab
constexpr int kMaxTile = 128;                   // uv tile side (cells)
constexpr int kMaxSubSide = kMaxTile + kMaxSupport - 1;  // tile plus support halo

struct Geom {
  int nx, ny;        // image
  int ngx, ngy;      // oversampled grid
  double dx, dy;     // pixel size (rad)
  int W;             // kernel support (cells)
  double beta;       // ES shape
  double sigma;
  int do_w;
  double tc;         // centre of the image's (n-1) range
  double dw;         // w-plane spacing (wavelengths)
  double w_lo, w_hi; // visibility w range (wavelengths)
  int nplanes;
  int T;             // uv tile side (cells)
  int S;             // w-planes per bucket slab
  int ntu, ntv, nslabs;
  int64_t nbuckets;
  int64_t R;         // rows
  int C;             // channels
  int NP;            // image polarisations
  uint32_t nitems;   // R * C
  int B;             // planes per batch
  int nquad;         // quadrature nodes for the w correction
  int shifted;       // a phase shift is fused into the item factors
  double shift[3];   // its (u, v, w) coefficients, plan uvw frame
};

// Item record in bucket order.  `loc` packs the item's first support cell
// inside its tile (bits 0-7 u, 8-15 v), its first w-plane inside its
// slab (bits 16-23) and whether it is mirrored to -uvw (bit 31, kLocFlip:
// invert grids conj(value), predict conjugates its result).  du, dv, dwf
// are the offsets of the item's continuous grid coordinate from its first
// support cell (in (W/2-1, W/2]); ph is exp(-2 pi i w tc), the rotation
// that centres the (n-1) band (w after the mirroring).
constexpr uint32_t kLocFlip = 0x80000000u;
struct __align__(16) ItemF {
  uint32_t idx, loc;
  float du, dv, dwf, pad;
  float2 ph;
};
struct __align__(16) ItemD {
  uint32_t idx, loc;
  double du, dv, dwf;
  double2 ph;
};

template <typename R> struct Traits;
template <> struct Traits<float> {
  using C = float2;
  using Item = ItemF;
};
template <> struct Traits<double> {
  using C = double2;
  using Item = ItemD;
};

// A unit of work for the tile kernels: up to kChunkItems consecutive items
// of one bucket.
struct Chunk {
  uint32_t begin, end, bucket, pad;
};

// Half-interval Gauss-Legendre quadrature of the ES kernel (nodes in cells,
// weights times kernel values), passed to kernels by value: the kernel's
// Fourier transform is phihat(nu) = 2 sum_q w_q cos(2 pi x_q nu).
struct Quad {
  int n;
  double x[kMaxQuad];
  double w[kMaxQuad];
};

// Polarisation conversion matrix (nout x nin complex, row-major); the
// identity is flagged so kernels skip the multiply.
struct PolMat {
  int nout, nin, identity, pad;
  double re[16], im[16];
  float fre[16], fim[16];  // the same, rounded once on the host for the FP32 kernels
};

// Element i of the pol matrix in the kernel's real type (the FP32 kernels
// read the host-rounded copy: a double-to-float conversion is an FP64-pipe
// instruction, 16 cycles a warp on this part, per item otherwise).
template <typename R> __device__ __forceinline__ R pm_re(const PolMat &pm, int i);
template <typename R> __device__ __forceinline__ R pm_im(const PolMat &pm, int i);
template <> __device__ __forceinline__ float pm_re<float>(const PolMat &pm, int i) {
  return pm.fre[i];
}
template <> __device__ __forceinline__ float pm_im<float>(const PolMat &pm, int i) {
  return pm.fim[i];
}
template <> __device__ __forceinline__ double pm_re<double>(const PolMat &pm, int i) {
  return pm.re[i];
}
template <> __device__ __forceinline__ double pm_im<double>(const PolMat &pm, int i) {
  return pm.im[i];
}

// ---------------------------------------------------------------------
// Per-item coordinates, FP64, with every rounding step explicit so the
// result is bit-identical to the CPU restatement (no FMA contraction).
struct Coord {
  int p0, q0;      // first support cell, wrapped into [0, ng)
  int k0;          // first w-plane
  int flip;        // the item is mirrored to -uvw (see row_flipped)
  double du, dv, dwf;
  double w;        // w in wavelengths (after the mirroring)
};

__host__ __device__ inline double gb_mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ inline double gb_add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
__host__ __device__ inline double gb_sub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
__host__ __device__ inline double gb_div(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// Hermitian mirroring.  Every image the gridder makes or reads is real
// (ms2dirty keeps the real part; dirty2ms takes a real image), so an item at
// (u, v, w) with value V contributes exactly what an item at (-u, -v, -w)
// with value conj(V) does, and the prediction at -uvw is the conjugate of
// the one at uvw.  With w-stacking, rows with w < 0 are mirrored: the w
// range then spans |w| only, which halves the number of w-planes (and their
// transforms) for a w range symmetric about zero.  Negation is exact, so a
// mirrored coordinate is bit-identical to the product formed from -uvw.
__host__ __device__ inline bool row_flipped(const Geom &g, const double *uvw, uint32_t r) {
  return g.do_w && uvw[3 * (size_t)r + 2] < 0.0;
}

// Turns of an item's rotation factor exp(-2 pi i turns), reduced to
// [-1/2, 1/2]: the w-centring term w tc and, when `shift`, minus the fused
// phase shift (u, v, w) . s (wavelengths).  Formed in FP64 before the
// reduction; the FP32 form rounds only the reduced value.
// `fscale` is f/c per channel (freq / kSpeedOfLight, one IEEE division per
// channel: the same value a division per item would give).
__host__ __device__ inline double item_turns(const Geom &g, const double *uvw,
                                             const double *fscale, uint32_t i, bool shift) {
  const uint32_t r = i / (uint32_t)g.C;
  const uint32_t c = i - r * (uint32_t)g.C;
  const double k = fscale[c];
  const double sg = row_flipped(g, uvw, r) ? -1.0 : 1.0;  // exact: a sign change
  const double w = sg * gb_mul(uvw[3 * (size_t)r + 2], k);
  double t = g.do_w ? gb_mul(w, g.tc) : 0.0;
  if (shift) {
    const double u = sg * gb_mul(uvw[3 * (size_t)r + 0], k);
    const double v = sg * gb_mul(uvw[3 * (size_t)r + 1], k);
    const double d = gb_add(gb_add(gb_mul(u, g.shift[0]), gb_mul(v, g.shift[1])),
                            gb_mul(w, g.shift[2]));
    t = gb_sub(t, d);
  }
  return gb_sub(t, rint(t));
}

__host__ __device__ inline void item_coord(const Geom &g, const double *uvw,
                                           const double *fscale, uint32_t i,
                                           Coord &o) {
  const uint32_t r = i / (uint32_t)g.C;
  const uint32_t c = i - r * (uint32_t)g.C;
  const double s = fscale[c];
  o.flip = row_flipped(g, uvw, r) ? 1 : 0;
  const double sg = o.flip ? -1.0 : 1.0;  // exact: a sign change
  const double u = sg * gb_mul(uvw[3 * (size_t)r + 0], s);
  const double v = sg * gb_mul(uvw[3 * (size_t)r + 1], s);
  const double w = sg * gb_mul(uvw[3 * (size_t)r + 2], s);
  const double halfW = 0.5 * g.W;
  double fu = gb_mul(u, g.dx);
  fu = gb_sub(fu, floor(fu));
  const double U = gb_mul(fu, (double)g.ngx);
  const double p0 = ceil(gb_sub(U, halfW));
  o.du = gb_sub(U, p0);
  double fv = gb_mul(v, g.dy);
  fv = gb_sub(fv, floor(fv));
  const double V = gb_mul(fv, (double)g.ngy);
  const double q0 = ceil(gb_sub(V, halfW));
  o.dv = gb_sub(V, q0);
  int ip = (int)p0, iq = (int)q0;
  ip = ip < 0 ? ip + g.ngx : (ip >= g.ngx ? ip - g.ngx : ip);
  iq = iq < 0 ? iq + g.ngy : (iq >= g.ngy ? iq - g.ngy : iq);
  o.p0 = ip;
  o.q0 = iq;
  o.w = w;
  if (g.do_w) {
    const double a = gb_div(gb_sub(w, g.w_lo), g.dw);
    const double k0 = ceil(a);
    o.dwf = gb_add(gb_sub(a, k0), halfW);
    int ik = (int)k0;
    const int kmax = g.nplanes - g.W;
    ik = ik < 0 ? 0 : (ik > kmax ? kmax : ik);
    o.k0 = ik;
  } else {
    o.dwf = 0.0;
    o.k0 = 0;
  }
}

__host__ __device__ inline uint32_t bucket_of(const Geom &g, const Coord &o) {
  const uint32_t tu = (uint32_t)(o.p0 / g.T);
  const uint32_t tv = (uint32_t)(o.q0 / g.T);
  const uint32_t sl = (uint32_t)(o.k0 / g.S);
  return (sl * (uint32_t)g.ntv + tv) * (uint32_t)g.ntu + tu;
}

// ---------------------------------------------------------------------
// ES kernel at support-normalised x in [-1, 1).
__device__ __forceinline__ float es_kernel(float x, float beta) {
  const float t = 1.0f - x * x;
  return t > 0.0f ? expf(beta * (sqrtf(t) - 1.0f)) : 0.0f;
}
__device__ __forceinline__ double es_kernel(double x, double beta) {
  const double t = 1.0 - x * x;
  return t > 0.0 ? exp(beta * (sqrt(t) - 1.0)) : 0.0;
}

__device__ __forceinline__ void sincos_2pi(float frac, float *s, float *c) {
  sincospif(2.0f * frac, s, c);
}
__device__ __forceinline__ void sincos_2pi(double frac, double *s, double *c) {
  sincospi(2.0 * frac, s, c);
}

// n - 1 for pixel (ix, iy), cancellation-free form.
__device__ __forceinline__ double pixel_nm1(const Geom &g, int ix, int iy) {
  const double x = (double)(ix - g.nx / 2) * g.dx;
  const double y = (double)(iy - g.ny / 2) * g.dy;
  const double r2 = x * x + y * y;
  return -r2 / (1.0 + sqrt(1.0 - r2));
}

// frac(x) as 64-bit fixed-point turns (x in turns, FP64).
__device__ __forceinline__ unsigned long long fixed_turns(double x) {
  const double f = x - floor(x);  // [0, 1]; 1 wraps to 0 below
  return ((unsigned long long)(f * 9223372036854775808.0)) << 1;
}

// The w-screen phases of planes b0, b0 + 1, ... at one pixel (plane k sits at
// w_k = w_lo + (k - W/2) dw; its phase at offset t' = n - 1 - tc is w_k t'
// turns): plane b0's phase w_b0 t' and the step dw t' are formed once in FP64 and held as
// 64-bit fixed-point turns, so plane b0 + j's phase is an exact integer sum
// (no FP64 instruction per plane; on this part a warp's FP64 instruction
// costs 16 cycles of the SM's FP64 pipe), exact to the FP64 rounding of the
// two products.
struct PlaneTurns {
  unsigned long long a, d;
  __device__ __forceinline__ void start(const Geom &g, int b0, double tprime) {
    const double wk = g.w_lo + ((double)b0 - 0.5 * g.W) * g.dw;
    a = fixed_turns(wk * tprime);
    d = fixed_turns(g.dw * tprime);
  }
  // turns of plane b0 + j in [-1/2, 1/2)
  __device__ __forceinline__ float turns_f32(int j) const {
    const unsigned long long ph = a + (unsigned long long)(unsigned)j * d;
    return (float)(int)(unsigned)(ph >> 32) * 0x1p-32f;
  }
  __device__ __forceinline__ double turns_f64(int j) const {
    const unsigned long long ph = a + (unsigned long long)(unsigned)j * d;
    return (double)(long long)ph * 0x1p-64;
  }
  __device__ __forceinline__ float turns(int j, float) const { return turns_f32(j); }
  __device__ __forceinline__ double turns(int j, double) const { return turns_f64(j); }
};

// ---------------------------------------------------------------------
// Tile kernels: lane map and shared-memory layout.
//
// A warp works on one item at a time.  Its lanes form G = 32/AW groups of
// AW lanes (AW = 8 for W <= 8, 16 for W <= 16); lane (g, a) owns support
// column a and, depending on NP, either a subset of the polarisations
// (NP >= G: pols g, g + G, ...) or one polarisation and every RS-th support
// row (NP < G).  The tile's sub-grid is stored as 2 NP planes (the real
// parts of every pol, then the imaginary parts) of SW rows x `pitch`
// words; pitch and the plane stride are chosen so that the lanes of one
// instruction fall in 32 distinct shared-memory banks.

inline __host__ __device__ constexpr int congruent_up(int x, int m) {
  return x + ((((m % 32) - (x % 32)) % 32) + 32) % 32;
}

inline __host__ __device__ constexpr int group_lanes(int W) { return W <= 8 ? 8 : 16; }

// Floats per item in the FP32 gridder's shared-memory item cache: the
// packed location word (padded to 16 bytes), then the u, v and w kernel
// values, AW each (zero beyond W), so every group starts on 16 bytes.
inline __host__ __device__ constexpr int kcache_stride(int AW) { return 4 + 3 * AW; }

struct TileLayout {
  int SW, pitch, plane;
};

inline __host__ __device__ constexpr TileLayout tile_layout(int T, int W, int NP) {
  const int AW = group_lanes(W), G = 32 / AW;
  const int RS = NP >= G ? 1 : G / NP;
  const int SW = T + W - 1, pitch = congruent_up(SW, AW);
  return TileLayout{SW, pitch, congruent_up(SW * pitch, AW * RS)};
}

template <int NP, int AW>
struct LaneMap {
  static constexpr int G = 32 / AW;
  static constexpr int NPL = NP >= G ? NP / G : 1;  // polarisations per lane
  static constexpr int RS = NP >= G ? 1 : G / NP;   // support-row stride
  int g, a, p0, r0;
  __device__ __forceinline__ explicit LaneMap(int lane) {
    g = lane / AW;
    a = lane % AW;
    p0 = NP >= G ? g : g % NP;
    r0 = NP >= G ? 0 : g / NP;
  }
  __device__ __forceinline__ int pol(int i) const { return p0 + i * G; }
};

// Row order of a predict grid after the column transforms: logical row
// q = k1 + N1 k2 sits at physical row N2 k1 + k2 = ((q & (N1-1)) << s2) |
// (q >> s1).  s1 < 0: natural order.
struct RowPerm {
  int s1, s2;
  __host__ __device__ __forceinline__ int row(int q) const {
    return s1 < 0 ? q : (((q & ((1 << s1) - 1)) << s2) | (q >> s1));
  }
};

// Error reporting -------------------------------------------------------
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

}  // namespace gb
