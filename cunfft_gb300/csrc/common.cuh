// common.cuh -- shared definitions for the GB300 NFFT kernels and host runtime.
//
// Data layout in HBM (per transform instance):
//   x      [M][d]  float64 nodes (the reference's layout, src/cunfft_typedefs.h:129-131)
//   f_hat  row-major over I_N, dim 0 slowest (k_t + N_t/2 is the index along dim t)
//   g      row-major n0 x n1 x n2 oversampled grid; frequency k lives at k mod n
//   f      [M] samples
// Batched plans store B instances back to back (B*N_total coefficients, B*n_total
// grid points, sum_i M_i nodes/samples).  Complex values are interleaved (re, im)
// pairs of the plan's real type: double2 for the FP64 form, float2 for the FP32 form.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cg {

constexpr int kMaxDim = 3;
constexpr int kMaxTaps = 32;        // W = 2m+2 <= 32, i.e. 1 <= m <= 15
constexpr int kWarp = 32;

template <typename T> struct Cx;
template <> struct Cx<float>  { using t = float2; };
template <> struct Cx<double> { using t = double2; };

// Geometry of one plan, passed by value to every kernel.
struct Geom {
  int d;                 // 1..3
  int m;                 // window cut-off
  int W;                 // taps per dimension, 2m+2
  int batch;             // number of instances
  int64_t N[kMaxDim];    // bandwidths (1 for unused dims)
  int64_t n[kMaxDim];    // oversampled grid sizes, any n_t >= N_t (1 for unused dims)
  int64_t Ntot, ntot;    // per instance
  double b[kMaxDim];     // Gaussian shape parameter per dim
  double norm;           // Gaussian: prod_t sqrt(b'_t), b' = (2 sigma-1)/(2 sigma m) = 1/(pi b); ES: 1
  float cbf[kMaxDim];    // log2(e) / b_t, rounded to FP32 (FP32 tap weights exp2(-y^2 cb))
  // window: kWinGauss (the reference's) or kWinES, exponential of semicircle
  // phi(y) = exp(beta_t (sqrt(1 - y^2 / alpha^2) - 1)) for |y| < alpha = m + 1/2, else 0
  int window;
  double es_beta[kMaxDim];  // beta_t
  double es_ia2;            // 1 / alpha^2
  float es_bl[kMaxDim];     // beta_t log2(e), FP32
  float es_ia2f;            // 1 / alpha^2, FP32
};

constexpr int kWinGauss = 0;
constexpr int kWinES = 1;

// FP32 tap constants of one dimension: Gaussian exp2(-y^2 a); ES
// exp2(-b q / (1 + sqrt(1 - q))), q = y^2 a (the ES exponent beta (sqrt(1 - q) - 1)
// without the cancellation near the centre), zero for q >= 1.
struct TapK {
  float a, b;
};
// FP32 tap of the window at distance y (grid units) from the node
// 2^x by the hardware approximation (ex2.approx.ftz: about 2 ulp, subnormal results
// flushed to zero); tap exponents lie in [-45, 0], where the flushed range holds
// weights below 1e-38 that no FP32 sum can see
__device__ __forceinline__ float tap_exp2(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <int WIN>
__device__ __forceinline__ float win_tap(float y, TapK k) {
  if (WIN == kWinGauss) return tap_exp2(-(y * y) * k.a);
  const float q = (y * y) * k.a, z = 1.f - q;
  const float e = tap_exp2(__fdividef(-k.b * q, 1.f + z * rsqrtf(z)));  // NaN for z <= 0, not selected
  return z > 0.f ? e : 0.f;
}

// tap constants of dimension t for a window fixed at compile time
template <int WIN>
__host__ __device__ inline TapK tap_k(const Geom& g, int t) {
  TapK k;
  if (WIN == kWinES) {
    k.a = g.es_ia2f;
    k.b = t == 0 ? g.es_bl[0] : (t == 1 ? g.es_bl[1] : g.es_bl[2]);
  } else {
    k.a = t == 0 ? g.cbf[0] : (t == 1 ? g.cbf[1] : g.cbf[2]);
    k.b = 0.f;
  }
  return k;
}

// ... and for the plan's window
__host__ __device__ inline TapK tap_k(const Geom& g, int t) {
  TapK k;
  if (g.window == kWinES) {
    k.a = g.es_ia2f;
    k.b = t == 0 ? g.es_bl[0] : (t == 1 ? g.es_bl[1] : g.es_bl[2]);
  } else {
    k.a = t == 0 ? g.cbf[0] : (t == 1 ? g.cbf[1] : g.cbf[2]);
    k.b = 0.f;
  }
  return k;
}

// Compile-time extents of the inner tile dimensions of the shared-memory
// gridding kernels (the outermost extent T0 stays a runtime, tunable value):
// d = 3: T1 x T2 = 8 x 16 (4 x 8 for windows wider than 16 taps); d = 2: T1 = 64.
// With them the row stride S and plane stride PS are constants, so every tap's
// shared-memory offset is an immediate.
__host__ __device__ constexpr int fixed_t_last(int d, int W) { return d == 3 ? (W <= 16 ? 16 : 8) : (d == 2 ? 64 : 1); }
__host__ __device__ constexpr int fixed_t_mid(int d, int W) { return d == 3 ? (W <= 16 ? 8 : 4) : 1; }
// smallest S >= E with S == W (mod 16): lane i of the (row, tap) mapping lands in bank group i
__host__ __device__ constexpr int conflict_free_stride(int E, int W) {
  return E + ((((W - E) % 16) + 16) % 16);
}
__host__ __device__ constexpr int fixed_row_stride(int d, int W) {
  return d == 1 ? 0 : conflict_free_stride(fixed_t_last(d, W) + W - 1, W);
}
__host__ __device__ constexpr int fixed_plane_stride(int d, int W) {
  return d == 3 ? (fixed_t_mid(d, W) + W - 1) * fixed_row_stride(d, W) : fixed_row_stride(d, W);
}

// Tiling of the oversampled grid used by the gridding kernels.
struct Tiling {
  int T[kMaxDim];        // tile extent per dim (power of two, <= n_t)
  int nb[kMaxDim];       // tiles per dim = ceil(n_t / T_t)
  int E[kMaxDim];        // padded extent per dim = T_t + W - 1
  int S;                 // shared-memory row stride (elements) for the innermost dim
  int R1;                // rows per plane (E[d-2] for d = 3, unused otherwise)
  int64_t tiles_per_inst;
  int64_t tiles_total;   // batch * tiles_per_inst
  int chunk;             // max nodes per work item
  int threads;           // CTA size of the gridding kernels
  size_t smem_tile;      // bytes of the staged tile
  int use_global;        // 1: no shared-memory tile fits, grid in global memory
  int spread_kernel;     // spreading kernel in use: CUNFFT_X_SPREAD_SHARED, _REGISTER, _TENSOR or _GLOBAL
  int interp_kernel;     // interpolation kernel in use: CUNFFT_X_INTERP_SHARED, _TENSOR or _GLOBAL
  // Sub-bins (sub_on = 1): the counting sort orders the nodes of a tile by sub-bin of
  // 2^ssh[0] x 2^ssh[1] window starts (dimensions 0 and 1), sub-bin (s0, s1) = s0 snb1 + s1
  // of ns per tile.  2D FP32 plans the tensor-core interpolation covers take 16 x 16
  // sub-tiles, and the binning also makes their interpolation items (sub_items = 1).
  // sub_on = 0: tile order only (ns = 1).
  int sub_on;
  int sub_items;
  int ns;
  int ssh[2];
  int snb1;
};

// Sorted node records, produced by the binning kernels.
struct Bins {
  int32_t* sidx;         // [M] original node index of the k-th sorted node
  int32_t* soff;         // [M] packed tile-local window start (10 bits per dim)
  void*    sfrac;        // [M*d] T: c_t - m with c_t = n_t x_t - u_t (FP64 reduction)
  int32_t* count;        // [tiles_total + 1]
  int32_t* tile_off;     // [tiles_total + 1] exclusive scan of counts
  int32_t* item_off;     // [tiles_total + 1] exclusive scan of items per tile
  int4*    items;        // [max_items] (tile, start, end, 0)
  int32_t* num_items;    // [1]
  int32_t* work;         // [2] persistent work-queue counters (forward, adjoint)
  int2*    tile_rank;    // [M] per node (tile, rank) scratch
  void*    fperm;        // [M] complex: the samples in sorted order (filled per call by the tensor-core spreading)
  int32_t* inst_off;     // [batch + 1] node offsets per instance
  int32_t* status;       // [1] device-side error flag
  uint32_t* fmax;        // [1] largest |Re|, |Im| of the samples being spread (float bits), per call
  // sub-bins (Tiling::sub_on): the counting sort's key is tile * ns + sub-bin
  int32_t* scount;       // [tiles_total * ns + 1] nodes per sub-bin
  int32_t* sub_pre;      // [tiles_total * ns] nodes of the tile's sub-bins before this one
  int32_t* icount;       // [tiles_total + 1] interpolation items per tile (Tiling::sub_items)
  int32_t* iitem_off;    // [tiles_total + 1] exclusive scan of icount
  int32_t* iscratch;     // [tiles_total + 1] the scan's second output, unused
  int4*    iitems;       // [max_iitems] (sub-bin key, start, end, 0): at most kSubItem nodes of one sub-tile
  int32_t* num_iitems;   // [1]
  int64_t  max_iitems;
  int64_t  M;            // total nodes
  int64_t  max_items;
  int      valid;        // nodes binned for the current tiling
};

// nodes per interpolation item of a sub-bin (the MMA's M)
constexpr int kSubItem = 128;

// i mod n in [0, n) for any i: a mask when n is a power of two, else the remainder.
__host__ __device__ inline int64_t wrap_n(int64_t i, int64_t n) {
  if ((n & (n - 1)) == 0) return i & (n - 1);
  const int64_t r = i % n;
  return r < 0 ? r + n : r;
}

// i mod n for 0 <= i: tile origin plus an offset inside the padded tile, at most one
// tile extent past n except on grids smaller than the tile; no division.
__host__ __device__ __forceinline__ int64_t wrap_up(int64_t i, int64_t n) {
  if ((n & (n - 1)) == 0) return i & (n - 1);
  while (i >= n) i -= n;
  return i;
}

}  // namespace cg
