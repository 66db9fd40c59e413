// kernels_grid.cuh -- tiled Gaussian gridding: interpolation (forward) and spreading (adjoint).
//
// Method (the reference's, src/cunfft_kernel.cu:514-1149): node j touches the
// (2m+2)^d grid points (u_t + l_t) mod n_t, l_t = 0..2m+1, with weight
// prod_t psi_t(l_t), psi(l) = sqrt(b') exp(-(c - l)^2 / b), c = n x - u.
//
// GB300 design:
//  * Work items: a tile of the grid (T0 x T1 x T2 window starts) plus at most
//    `chunk` of its sorted nodes.  A persistent grid of CTAs pulls items from an
//    atomic queue, so clustered node sets (thousands of nodes in one tile) spread
//    over many CTAs instead of serialising on one.
//  * The CTA stages the padded tile (T_t + W - 1 per dim, wrapped mod n) in shared
//    memory.  The inner strides are compile-time constants (common.cuh): row
//    stride S == W (mod 16) elements, so the lane -> tap mapping below touches
//    consecutive banks (no conflicts for float2 or double2 elements), and every
//    tap offset is an immediate.
//  * Lane i < R*W (R = 32/W) owns innermost tap l_last = i % W and rows
//    r = i / W, r + R, ... of the remaining taps (for d = 3 a row is an (l0, l1)
//    pair walked over the 2m+2 planes l0).
//  * Interpolation: one warp per node at a time; the warp reduces the node's sum
//    with shuffles.  Node records and tap weights of a batch of nodes are staged
//    per warp in shared memory; the next batch's records are fetched into
//    registers while the current batch runs.
//  * Spreading: no shared-memory atomics (a float atomic add on shared memory is a
//    compare-and-swap loop).  Every warp walks all nodes of a CTA-wide batch but
//    writes only the planes (d = 3) or row groups (d = 2) it owns, with plain
//    load / FMA / store; for d = 1 each warp accumulates into a private copy of
//    the tile.  Batches are double-buffered (one barrier per batch).  The tile is
//    then added to the global grid with vector atomics, so neighbouring items'
//    halos combine.
//  * Tap weights: one hardware exp2 per tap in the FP32 form; in the FP64 form the reference's
//    fast-Gaussian-gridding recurrence (2 exp per node and dim, src/cunfft_kernel.cu:
//    491-505), which keeps the scarce FP64 pipe on the taps.
#pragma once

#include "runtime.h"

namespace cg {

// bits of the packed tile-local window start, per dimension
__host__ __device__ constexpr int off_bits(int d) { return d == 1 ? 30 : (d == 2 ? 15 : 10); }

template <typename T> struct WeightMath;

template <> struct WeightMath<float> {
  // Gaussian: psi(l) / sqrt(b') = exp(-(fr + m - l)^2 / b) = exp2(-(y*y) * log2(e)/b);
  // ES: exp(beta (sqrt(1 - y^2/alpha^2) - 1)), y = fr + m - l
  static __device__ __forceinline__ void taps(float fr, int m, const Geom& g, int t, int W, float* out) {
    const TapK k = tap_k(g, t);
    if (g.window == kWinES) {
#pragma unroll 4
      for (int l = 0; l < W; ++l) out[l] = win_tap<kWinES>(fr + (float)(m - l), k);
    } else {
#pragma unroll 4
      for (int l = 0; l < W; ++l) out[l] = win_tap<kWinGauss>(fr + (float)(m - l), k);
    }
  }
};

template <> struct WeightMath<double> {
  // FGG form: psi_l = phi * E^l * exp(-l^2/b), phi = exp(-c^2/b), E = exp(2c/b), c = m + fr.
  static __device__ __forceinline__ void taps(double fr, int m, const Geom& g, int t, int W, double* out) {
    if (g.window == kWinES) {  // exp(beta (sqrt(1 - y^2/alpha^2) - 1)), zero outside |y| < alpha
      const double beta = t == 0 ? g.es_beta[0] : (t == 1 ? g.es_beta[1] : g.es_beta[2]);
      const double c = (double)m + fr;
      for (int l = 0; l < W; ++l) {
        const double y = c - (double)l, z = 1.0 - (y * y) * g.es_ia2;
        out[l] = z > 0.0 ? exp(beta * (sqrt(z) - 1.0)) : 0.0;
      }
      return;
    }
    const double b = t == 0 ? g.b[0] : (t == 1 ? g.b[1] : g.b[2]);
    const double c = (double)m + fr;
    const double ib = 1.0 / b;
    const double phi = exp(-(c * c) * ib);
    const double E = exp(2.0 * c * ib);
    const double q = exp(-ib);            // exp(-l^2/b) by the recurrence of src/cunfft.cu:60-76
    double e = 1.0, gl = 1.0, qstep = q;  // gl = exp(-l^2/b), qstep = exp(-(2l+1)/b)
    out[0] = phi;
#pragma unroll 4
    for (int l = 1; l < W; ++l) {
      e *= E;
      gl *= qstep;
      qstep *= q * q;
      out[l] = phi * e * gl;
    }
  }
};

__device__ __forceinline__ float2 cmul_add(float2 acc, float w, float2 v) {
  return __ffma2_rn(make_float2(w, w), v, acc);
}
__device__ __forceinline__ double2 cmul_add(double2 acc, double w, double2 v) {
  acc.x = fma(w, v.x, acc.x);
  acc.y = fma(w, v.y, acc.y);
  return acc;
}
// A weight ready for the complex multiply-add: the (w, w) pair of a packed
// f32x2 FMA in the FP32 form, the scalar in the FP64 form.
template <typename T> struct WPair;
template <> struct WPair<float> {
  using t = float2;
  static __device__ __forceinline__ float2 make(float w) { return make_float2(w, w); }
};
template <> struct WPair<double> {
  using t = double;
  static __device__ __forceinline__ double make(double w) { return w; }
};
__device__ __forceinline__ float2 cmul_addp(float2 acc, float2 ww, float2 v) { return __ffma2_rn(ww, v, acc); }
__device__ __forceinline__ double2 cmul_addp(double2 acc, double w, double2 v) {
  acc.x = fma(w, v.x, acc.x);
  acc.y = fma(w, v.y, acc.y);
  return acc;
}

// Asynchronous global -> shared copy of one complex element (cp.async, 8 or 16 bytes).
template <typename C>
__device__ __forceinline__ void cp_async_elem(C* dst, const C* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(C) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ float2 cscale(float2 v, float w) { return __fmul2_rn(make_float2(w, w), v); }
__device__ __forceinline__ double2 cscale(double2 v, double w) { return make_double2(v.x * w, v.y * w); }

__device__ __forceinline__ void global_add(float2* p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void global_add(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

template <typename C>
__device__ __forceinline__ C czero() {
  C z;
  z.x = 0;
  z.y = 0;
  return z;
}

template <typename C>
__device__ __forceinline__ C shfl_xor_c(C v, int o) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, o);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, o);
  return v;
}

// Tile origin a_t of a work item's tile and its instance.
struct TileOrigin {
  int64_t inst;
  int64_t a[kMaxDim];
};

template <int D>
__device__ __forceinline__ TileOrigin decode_tile(const Geom& geo, const Tiling& tl, int64_t tile) {
  TileOrigin o;
  o.inst = tile / tl.tiles_per_inst;
  int64_t lt = tile - o.inst * tl.tiles_per_inst;
  o.a[0] = o.a[1] = o.a[2] = 0;
  if (D == 3) {
    o.a[2] = (lt % tl.nb[2]) * tl.T[2];
    lt /= tl.nb[2];
  }
  if (D >= 2) {
    o.a[1] = (lt % tl.nb[1]) * tl.T[1];
    lt /= tl.nb[1];
  }
  o.a[0] = lt * tl.T[0];
  return o;
}

// Rows of the staged tile: [E0][E1] for d = 3, [E0] for d = 2, one for d = 1.
// The shared-memory row of (p0, p1) starts at p0 * PS + p1 * S.
template <int D>
__device__ __forceinline__ int tile_rows(const Tiling& tl) {
  return D == 3 ? tl.E[0] * tl.E[1] : (D == 2 ? tl.E[0] : 1);
}

template <int D>
__device__ __forceinline__ void row_coords(const Tiling& tl, int row, int* p0, int* p1) {
  if (D == 3) {
    *p0 = row / tl.E[1];
    *p1 = row - *p0 * tl.E[1];
  } else {
    *p0 = row;
    *p1 = 0;
  }
}

template <int D>
__device__ __forceinline__ int64_t row_gbase(const Geom& geo, const TileOrigin& o, int p0, int p1) {
  if (D == 3) return (wrap_up(o.a[0] + p0, geo.n[0]) * geo.n[1] + wrap_up(o.a[1] + p1, geo.n[1])) * geo.n[2];
  if (D == 2) return wrap_up(o.a[0] + p0, geo.n[0]) * geo.n[1];
  return 0;
}

template <int D, int W, typename C>
__device__ __forceinline__ void load_tile(C* tile, const C* __restrict__ gi, const Geom& geo, const Tiling& tl,
                                          const TileOrigin& o) {
  constexpr int S = fixed_row_stride(D, W), PS = fixed_plane_stride(D, W);
  const int E_last = tl.E[D - 1];
  const int64_t n_last = geo.n[D - 1], a_last = o.a[D - 1];
  if (D == 1) {
    for (int p = threadIdx.x; p < E_last; p += blockDim.x) cp_async_elem(tile + p, gi + wrap_up(a_last + p, n_last));
    cp_async_wait_all();
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int rows = tile_rows<D>(tl);
  for (int row = warp; row < rows; row += nwarps) {
    int p0, p1;
    row_coords<D>(tl, row, &p0, &p1);
    const int64_t gbase = row_gbase<D>(geo, o, p0, p1);
    C* dst = tile + (D == 3 ? p0 * PS + p1 * S : p0 * S);
    for (int p = lane; p < E_last; p += kWarp) cp_async_elem(dst + p, gi + gbase + wrap_up(a_last + p, n_last));
  }
  cp_async_wait_all();  // this thread's copies landed; the caller's barrier publishes them
}

// Add the tile into the global grid.  FP32 pairs (even offset on a 16-byte aligned grid
// whose last size is even, so 16-byte aligned and never split by the wrap) go as one
// float4 atomic.
template <int D, int W, typename C>
__device__ __forceinline__ void flush_tile(const C* tile, C* __restrict__ gi, const Geom& geo, const Tiling& tl,
                                           const TileOrigin& o) {
  constexpr int S = fixed_row_stride(D, W), PS = fixed_plane_stride(D, W);
  const int E_last = tl.E[D - 1];
  const int64_t n_last = geo.n[D - 1], a_last = o.a[D - 1];
  const int rows = tile_rows<D>(tl);
  constexpr bool kF32 = sizeof(C) == 8;
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool pairs_ok = kF32 && (n_last & 1) == 0 && (tl.T[D - 1] & 1) == 0 &&  // even tile origin and row length
                       (reinterpret_cast<uintptr_t>(gi) & 15u) == 0;
  const int per_row = pairs_ok ? (E_last + 1) >> 1 : E_last;
  const int total = rows * per_row;
  for (int e = tid; e < total; e += nt) {
    const int row = e / per_row, k = e - row * per_row;
    int p0, p1;
    row_coords<D>(tl, row, &p0, &p1);
    const C* src = tile + (D == 3 ? p0 * PS + p1 * S : (D == 2 ? p0 * S : 0));
    const int64_t gb = row_gbase<D>(geo, o, p0, p1);
    if (pairs_ok) {
      const int p = 2 * k;
      const C v0 = src[p];
      const int64_t gidx = gb + wrap_up(a_last + p, n_last);
      if (p + 1 < E_last) {
        const C v1 = src[p + 1];
        if (v0.x != 0 || v0.y != 0 || v1.x != 0 || v1.y != 0)
          atomicAdd(reinterpret_cast<float4*>(gi + gidx), make_float4(v0.x, v0.y, v1.x, v1.y));
      } else if (v0.x != 0 || v0.y != 0) {
        global_add(gi + gidx, v0);
      }
    } else {
      const C v = src[k];
      if (v.x != 0 || v.y != 0) global_add(gi + gb + wrap_up(a_last + k, n_last), v);
    }
  }
}

// Grab the next work item; returns false when the queue is drained.
__device__ __forceinline__ bool next_item(const Bins& bins, int slot, int4* cur) {
  if (threadIdx.x == 0) {
    const int it = atomicAdd(&bins.work[slot], 1);
    *cur = it < *bins.num_items ? bins.items[it] : make_int4(-1, 0, 0, 0);
  }
  __syncthreads();
  return cur->x >= 0;
}

// Shared-memory bytes beyond the tile, per kernel kind (the host sizes launches with it).
__host__ __device__ constexpr int nodes_per_warp_batch(int d) { return d == 1 ? 32 : (d == 2 ? 8 : 5); }
constexpr int kNodesPerCtaBatch = 16;

__host__ __device__ inline size_t grid_extra_smem(int d, int W, size_t real, int nwarps, size_t tile_bytes,
                                                  bool spread) {
  if (!spread) {
    const int nb = nodes_per_warp_batch(d);
    return (size_t)nwarps * ((size_t)nb * d * W * real + (size_t)nb * 2 * sizeof(int));
  }
  // two batch buffers: weights, values, offsets
  const size_t batch = (size_t)kNodesPerCtaBatch * d * W * real + (size_t)kNodesPerCtaBatch * (sizeof(int) + 2 * real);
  return (d == 1 ? (size_t)(nwarps - 1) * tile_bytes : 0) + 2 * batch;
}

// ---------------------------------------------------------------------------
// Interpolation, d = 1..3
// ---------------------------------------------------------------------------
template <int D, int W, typename T>
__global__ void __launch_bounds__(512) k_interp(const typename Cx<T>::t* __restrict__ g,
                                                typename Cx<T>::t* __restrict__ f, Geom geo, Tiling tl, Bins bins) {
  using C = typename Cx<T>::t;
  constexpr int R = kWarp / W;           // rows (d >= 2) or nodes (d = 1) per warp pass
  constexpr int NIT = (W + R - 1) / R;   // passes over the W rows of a plane
  constexpr bool FULL = R * NIT == W;    // every lane's every pass is a real row
  constexpr int NB = nodes_per_warp_batch(D);
  constexpr int SH = off_bits(D);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr int S = fixed_row_stride(D, W), PS = fixed_plane_stride(D, W);
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int4 cur;
  C* tile = reinterpret_cast<C*>(smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  T* wb = reinterpret_cast<T*>(smem + tl.smem_tile) + warp * (NB * D * W);
  int* nrec = reinterpret_cast<int*>(reinterpret_cast<T*>(smem + tl.smem_tile) + nwarps * (NB * D * W)) + warp * 2 * NB;
  const int r = lane / W, l_last = lane - r * W;
  const bool lane_on = r < R;
  const T* sfrac = reinterpret_cast<const T*>(bins.sfrac);
  const T norm = (T)geo.norm;
  const int qd = lane / D, td = lane - qd * D;  // (node, dim) of this lane in the weight pass

  while (next_item(bins, 0, &cur)) {
    const int4 item = cur;
    const TileOrigin o = decode_tile<D>(geo, tl, item.x);
    load_tile<D, W, C>(tile, g + o.inst * geo.ntot, geo, tl, o);
    // records of this warp's first batch
    int bs = item.y + warp * NB;
    int pf_idx = 0, pf_off = 0;
    T pf_fr = 0;
    if (bs < item.z) {
      const int nb0 = min(NB, item.z - bs);
      if (lane < nb0) {
        pf_idx = bins.sidx[bs + lane];
        pf_off = bins.soff[bs + lane];
      }
      if (qd < nb0) pf_fr = sfrac[(int64_t)(bs + qd) * D + td];
    }
    __syncthreads();
    for (; bs < item.z; bs += nwarps * NB) {
      const int nb = min(NB, item.z - bs);
      if (lane < nb) {
        nrec[lane] = pf_idx;
        nrec[NB + lane] = pf_off;
      }
      if (qd < nb) WeightMath<T>::taps(pf_fr, geo.m, geo, td, W, wb + (qd * D + td) * W);
      // fetch the next batch's records while this batch runs
      const int bn = bs + nwarps * NB;
      if (bn < item.z) {
        const int nbn = min(NB, item.z - bn);
        if (lane < nbn) {
          pf_idx = bins.sidx[bn + lane];
          pf_off = bins.soff[bn + lane];
        }
        if (qd < nbn) pf_fr = sfrac[(int64_t)(bn + qd) * D + td];
      }
      __syncwarp();
      if (D == 1) {
        for (int q0 = 0; q0 < nb; q0 += R) {
          const int q = q0 + r;
          const bool on = lane_on && q < nb;
          const int qq = on ? q : q0;
          const int o0 = nrec[NB + qq] & MASK;
          C acc = on ? cscale(tile[o0 + l_last], wb[qq * W + l_last]) : czero<C>();
#pragma unroll
          for (int s = 1; s < W; s <<= 1) {
            C o2;
            o2.x = __shfl_down_sync(0xffffffffu, acc.x, s);
            o2.y = __shfl_down_sync(0xffffffffu, acc.y, s);
            if (l_last + s < W) {
              acc.x += o2.x;
              acc.y += o2.y;
            }
          }
          if (on && l_last == 0) f[nrec[qq]] = cscale(acc, norm);
        }
      } else {
        for (int q = 0; q < nb; ++q) {
          const uint32_t off = (uint32_t)nrec[NB + q];
          const T* wq = wb + q * D * W;
          const T w_last = wq[(D - 1) * W + (lane_on ? l_last : 0)];
          T wrow[NIT];
#pragma unroll
          for (int it = 0; it < NIT; ++it) {
            const int lr = r + it * R;
            wrow[it] = (FULL || lr < W) ? wq[(D - 2) * W + (FULL ? lr : min(lr, W - 1))] : (T)0;
          }
          typename WPair<T>::t wpl[D == 3 ? W : 1];
          if (D == 3) {
#pragma unroll
            for (int l0 = 0; l0 < W; ++l0) wpl[l0] = WPair<T>::make(wq[l0]);
          }
          int base;
          if (D == 3) {
            const int o0 = off & MASK, o1 = (off >> SH) & MASK, o2 = off >> (D == 3 ? 2 * SH : 0);
            base = o0 * PS + (o1 + r) * S + o2 + l_last;
          } else {
            const int o0 = off & MASK, o1 = (off >> SH) & MASK;
            base = (o0 + r) * S + o1 + l_last;
          }
          C acc = czero<C>();
          if (lane_on) {
            const C* tb = tile + base;
#pragma unroll
            for (int it = 0; it < NIT; ++it) {
              if (FULL || r + it * R < W) {
                C ra;
                if (D == 3) {
                  ra = czero<C>();
#pragma unroll
                  for (int l0 = 0; l0 < W; ++l0) ra = cmul_addp(ra, wpl[l0], tb[it * R * S + l0 * PS]);
                } else {
                  ra = tb[it * R * S];
                }
                acc = cmul_add(acc, wrow[it], ra);
              }
            }
            acc = cscale(acc, w_last);
          }
#pragma unroll
          for (int s = 16; s >= 1; s >>= 1) {
            const C o2 = shfl_xor_c<C>(acc, s);
            acc.x += o2.x;
            acc.y += o2.y;
          }
          if (lane == 0) f[nrec[q]] = cscale(acc, norm);
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Spreading, d = 1..3
// ---------------------------------------------------------------------------
template <int D, int W, typename T>
__global__ void __launch_bounds__(512) k_spread(const typename Cx<T>::t* __restrict__ f,
                                                typename Cx<T>::t* __restrict__ g, Geom geo, Tiling tl, Bins bins) {
  using C = typename Cx<T>::t;
  constexpr int R = kWarp / W;
  constexpr int NIT = (W + R - 1) / R;
  constexpr bool FULL = R * NIT == W;
  constexpr int NBC = kNodesPerCtaBatch;
  constexpr int SH = off_bits(D);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr int S = fixed_row_stride(D, W), PS = fixed_plane_stride(D, W);
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int4 cur;
  C* tile = reinterpret_cast<C*>(smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int tile_elems = D == 1 ? tl.E[0] : (D == 2 ? tl.E[0] * S : tl.E[0] * PS);
  // d = 1: one private tile copy per warp (copy 0 is `tile`)
  const size_t extra = D == 1 ? (size_t)(nwarps - 1) * tl.smem_tile : 0;
  unsigned char* bptr = smem + tl.smem_tile + extra;
  const size_t batch_bytes = (size_t)NBC * D * W * sizeof(T) + (size_t)NBC * (sizeof(int) + sizeof(C));
  const int r = lane / W, l_last = lane - r * W;
  const bool lane_on = r < R;
  const T* sfrac = reinterpret_cast<const T*>(bins.sfrac);
  const T norm = (T)geo.norm;
  C* mytile = D == 1 ? reinterpret_cast<C*>(smem + (size_t)warp * tl.smem_tile) : tile;
  // this thread's staging role: (node, dim) for weights, node for records
  const int sq = threadIdx.x / D, st = threadIdx.x - sq * D;

  while (next_item(bins, 1, &cur)) {
    const int4 item = cur;
    const TileOrigin o = decode_tile<D>(geo, tl, item.x);
    {
      const C z = czero<C>();
      if (D == 1) {
        for (int e = lane; e < tile_elems; e += kWarp) mytile[e] = z;
      } else {
        for (int e = threadIdx.x; e < tile_elems; e += blockDim.x) tile[e] = z;
      }
    }
    // records of the first batch
    T pf_fr = 0;
    int pf_off = 0;
    C pf_val = czero<C>();
    {
      const int nb0 = min(NBC, item.z - item.y);
      if (sq < nb0) pf_fr = sfrac[(int64_t)(item.y + sq) * D + st];
      if ((int)threadIdx.x < nb0) {
        pf_off = bins.soff[item.y + threadIdx.x];
        pf_val = f[bins.sidx[item.y + threadIdx.x]];
      }
    }
    int buf = 0;
    for (int bs = item.y; bs < item.z; bs += NBC, buf ^= 1) {
      const int nb = min(NBC, item.z - bs);
      unsigned char* bb = bptr + buf * batch_bytes;
      T* cw = reinterpret_cast<T*>(bb);                      // [NBC][D][W]
      C* cval = reinterpret_cast<C*>(cw + NBC * D * W);      // [NBC]
      int* coff = reinterpret_cast<int*>(cval + NBC);        // [NBC]
      if (sq < nb) WeightMath<T>::taps(pf_fr, geo.m, geo, st, W, cw + (sq * D + st) * W);
      if ((int)threadIdx.x < nb) {
        coff[threadIdx.x] = pf_off;
        cval[threadIdx.x] = cscale(pf_val, norm);
      }
      // fetch the next batch's records
      const int bn = bs + NBC;
      if (bn < item.z) {
        const int nbn = min(NBC, item.z - bn);
        if (sq < nbn) pf_fr = sfrac[(int64_t)(bn + sq) * D + st];
        if ((int)threadIdx.x < nbn) {
          pf_off = bins.soff[bn + threadIdx.x];
          pf_val = f[bins.sidx[bn + threadIdx.x]];
        }
      }
      __syncthreads();  // batch staged (and, for the first batch, the tile cleared)
      if (D == 1) {
        // warp w takes nodes w, w + nwarps, ...; lanes are the node's taps
        for (int q = warp; q < nb; q += nwarps) {
          const int o0 = coff[q] & MASK;
          if (lane < W) {
            C* p = mytile + o0 + lane;
            *p = cmul_add(*p, cw[q * W + lane], cval[q]);
          }
        }
      } else if (D == 2) {
        // warp w owns the row groups {g : g % nwarps == w}, group g = rows g*R .. g*R+R-1
        for (int q = 0; q < nb; ++q) {
          const uint32_t off = (uint32_t)coff[q];
          const int o0 = off & MASK, o1 = (off >> SH) & MASK;
          const int g_first = o0 / R, g_last = (o0 + W - 1) / R;
          const int g0 = g_first + ((warp - g_first % nwarps) + nwarps) % nwarps;
          if (g0 > g_last || !lane_on) continue;
          const T* wq = cw + q * 2 * W;
          const C v = cscale(cval[q], wq[W + l_last]);
          C* tb = tile + o1 + l_last;
          for (int gg = g0; gg <= g_last; gg += nwarps) {
            const int p0 = gg * R + r;
            if (p0 >= o0 && p0 < o0 + W) {
              C* p = tb + p0 * S;
              *p = cmul_add(*p, wq[p0 - o0], v);
            }
          }
        }
      } else {
        // warp w owns the planes {p : p % nwarps == w}
        for (int q = 0; q < nb; ++q) {
          const uint32_t off = (uint32_t)coff[q];
          const int o0 = off & MASK, o1 = (off >> SH) & MASK, o2 = off >> (D == 3 ? 2 * SH : 0);
          int p = o0 + ((warp - o0 % nwarps) + nwarps) % nwarps;
          if (p >= o0 + W || !lane_on) continue;
          const T* wq = cw + q * 3 * W;
          const C v = cscale(cval[q], wq[2 * W + l_last]);
          C vr[NIT];
#pragma unroll
          for (int it = 0; it < NIT; ++it) {
            const int l1 = r + it * R;
            vr[it] = cscale(v, (FULL || l1 < W) ? wq[W + (FULL ? l1 : min(l1, W - 1))] : (T)0);
          }
          C* tb = tile + (o1 + r) * S + o2 + l_last;
          for (; p < o0 + W; p += nwarps) {
            const typename WPair<T>::t w0 = WPair<T>::make(wq[p - o0]);
            C* tp = tb + p * PS;
#pragma unroll
            for (int it = 0; it < NIT; ++it) {
              if (FULL || r + it * R < W) {
                C* t = tp + it * R * S;
                *t = cmul_addp(*t, w0, vr[it]);
              }
            }
          }
        }
      }
    }
    __syncthreads();
    if (D == 1) {
      // fold the private copies into copy 0, then flush
      for (int e = threadIdx.x; e < tile_elems; e += blockDim.x) {
        C s = tile[e];
        for (int w = 1; w < nwarps; ++w) {
          const C v = reinterpret_cast<const C*>(smem + (size_t)w * tl.smem_tile)[e];
          s.x += v.x;
          s.y += v.y;
        }
        tile[e] = s;
      }
      __syncthreads();
    }
    flush_tile<D, W, C>(tile, g + o.inst * geo.ntot, geo, tl, o);
    __syncthreads();
  }
}

}  // namespace cg
