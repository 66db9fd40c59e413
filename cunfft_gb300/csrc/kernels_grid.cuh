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
//    memory.  Row stride S == W (mod 16) elements, so the lane -> tap mapping below
//    touches consecutive shared-memory banks: no bank conflicts for 8-byte
//    (float2) or 16-byte (double2) elements.
//  * One warp per node at a time.  Lane i < R*W (R = 32/W) owns innermost tap
//    l_last = i % W and rows r = i / W, r + R, r + 2R, ... of the remaining taps;
//    for d = 3 each row is a (l0, l1) pair and the lane loops over the 2m+2 planes
//    l0 with the plane weights held in registers.  The warp reduces the node's
//    sum with shuffles (interpolation) or adds the taps into the staged tile with
//    shared-memory atomics (spreading); the spread tile is then added to the
//    global grid with vector atomics, so neighbouring items' halos combine.
//  * Tap weights of a batch of 32/d nodes are computed by lane (node, dim) pairs
//    and parked in shared memory: exp2f per tap in the FP32 form; in the FP64 form
//    the reference's fast-Gaussian-gridding recurrence (2 exp per node and dim,
//    src/cunfft_kernel.cu:491-505), which keeps the scarce FP64 pipe on the taps.
#pragma once

#include "runtime.h"

namespace cg {

template <typename T> struct WeightMath;

template <> struct WeightMath<float> {
  // psi(l) / sqrt(b') = exp(-(fr + m - l)^2 / b) = exp2(-(y*y) * log2(e)/b)
  static __device__ __forceinline__ void taps(float fr, int m, double b, int W, float* out) {
    const float cb = (float)(1.4426950408889634 / b);
#pragma unroll 4
    for (int l = 0; l < W; ++l) {
      float y = fr + (float)(m - l);
      out[l] = exp2f(-(y * y) * cb);
    }
  }
};

template <> struct WeightMath<double> {
  // FGG form: psi_l = phi * E^l * exp(-l^2/b), phi = exp(-c^2/b), E = exp(2c/b), c = m + fr.
  static __device__ __forceinline__ void taps(double fr, int m, double b, int W, double* out) {
    const double c = (double)m + fr;
    const double ib = 1.0 / b;
    const double phi = exp(-(c * c) * ib);
    const double E = exp(2.0 * c * ib);
    const double q = exp(-ib);           // exp(-l^2/b) by the recurrence of src/cunfft.cu:60-76
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
__device__ __forceinline__ float2 cscale(float2 v, float w) { return __fmul2_rn(make_float2(w, w), v); }
__device__ __forceinline__ double2 cscale(double2 v, double w) { return make_double2(v.x * w, v.y * w); }

__device__ __forceinline__ void global_add(float2* p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void global_add(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

template <typename C>
__device__ __forceinline__ C shfl_xor_c(C v, int o);
template <>
__device__ __forceinline__ float2 shfl_xor_c<float2>(float2 v, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}
template <>
__device__ __forceinline__ double2 shfl_xor_c<double2>(double2 v, int o) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}

// Decode the work item's tile into instance and tile origin a_t.
struct TileOrigin {
  int64_t inst;
  int64_t a[kMaxDim];
};

__device__ __forceinline__ TileOrigin decode_tile(const Geom& geo, const Tiling& tl, int64_t tile) {
  TileOrigin o;
  o.inst = tile / tl.tiles_per_inst;
  int64_t lt = tile - o.inst * tl.tiles_per_inst;
  for (int t = geo.d - 1; t >= 0; --t) {
    int64_t b = lt % tl.nb[t];
    lt /= tl.nb[t];
    o.a[t] = b * tl.T[t];
  }
  return o;
}

// Shared-memory layout: [E0][E1][S] (d = 3), [E0][S] (d = 2), [S] (d = 1) complex
// elements, followed by the per-warp weight buffers [nwarps][32/d][d][W] of T.
template <int D, typename C>
__device__ __forceinline__ void load_tile(C* tile, const C* __restrict__ gi, const Geom& geo, const Tiling& tl,
                                          const TileOrigin& o, int warp, int nwarps, int lane) {
  const int E_last = tl.E[D - 1];
  const int64_t n_last = geo.n[D - 1];
  if (D == 1) {
    for (int p = threadIdx.x; p < E_last; p += blockDim.x) tile[p] = gi[wrap_pow2(o.a[0] + p, n_last)];
    return;
  }
  const int rows = D == 3 ? tl.E[0] * tl.E[1] : tl.E[0];
  for (int row = warp; row < rows; row += nwarps) {
    int64_t gbase;
    if (D == 3) {
      const int p0 = row / tl.E[1], p1 = row - p0 * tl.E[1];
      gbase = (wrap_pow2(o.a[0] + p0, geo.n[0]) * geo.n[1] + wrap_pow2(o.a[1] + p1, geo.n[1])) * geo.n[2];
    } else {
      gbase = wrap_pow2(o.a[0] + row, geo.n[0]) * geo.n[1];
    }
    C* dst = tile + (int64_t)row * tl.S;
    for (int p = lane; p < E_last; p += kWarp) dst[p] = gi[gbase + wrap_pow2(o.a[D - 1] + p, n_last)];
  }
}

template <int D, typename C>
__device__ __forceinline__ void flush_tile(const C* tile, C* __restrict__ gi, const Geom& geo, const Tiling& tl,
                                           const TileOrigin& o, int warp, int nwarps, int lane) {
  const int E_last = tl.E[D - 1];
  const int64_t n_last = geo.n[D - 1];
  if (D == 1) {
    for (int p = threadIdx.x; p < E_last; p += blockDim.x) {
      C v = tile[p];
      if (v.x != 0 || v.y != 0) global_add(&gi[wrap_pow2(o.a[0] + p, n_last)], v);
    }
    return;
  }
  const int rows = D == 3 ? tl.E[0] * tl.E[1] : tl.E[0];
  for (int row = warp; row < rows; row += nwarps) {
    int64_t gbase;
    if (D == 3) {
      const int p0 = row / tl.E[1], p1 = row - p0 * tl.E[1];
      gbase = (wrap_pow2(o.a[0] + p0, geo.n[0]) * geo.n[1] + wrap_pow2(o.a[1] + p1, geo.n[1])) * geo.n[2];
    } else {
      gbase = wrap_pow2(o.a[0] + row, geo.n[0]) * geo.n[1];
    }
    const C* src = tile + (int64_t)row * tl.S;
    for (int p = lane; p < E_last; p += kWarp) {
      C v = src[p];
      if (v.x != 0 || v.y != 0) global_add(&gi[gbase + wrap_pow2(o.a[D - 1] + p, n_last)], v);
    }
  }
}

template <int D, int W, typename T>
__device__ __forceinline__ void compute_batch_weights(T* wb, const T* __restrict__ sfrac, int64_t first, int nb,
                                                      const Geom& geo, int lane) {
  const int q = lane / D, t = lane - q * D;
  if (q < nb) {
    const T fr = sfrac[(first + q) * D + t];
    WeightMath<T>::taps(fr, geo.m, geo.b[t], W, wb + (q * D + t) * W);
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

// ---------------------------------------------------------------------------
// d = 2, 3: warp per node
// ---------------------------------------------------------------------------
template <int D, int W, typename T, bool SPREAD>
__global__ void __launch_bounds__(512) k_grid(const typename Cx<T>::t* __restrict__ in,
                                              typename Cx<T>::t* __restrict__ out,
                                              Geom geo, Tiling tl, Bins bins) {
  using C = typename Cx<T>::t;
  static_assert(D == 2 || D == 3, "warp-per-node kernel is for d = 2, 3");
  constexpr int R = kWarp / W;              // rows per warp pass
  constexpr int NIT = (W + R - 1) / R;      // passes over the W rows of a plane
  constexpr int NB = kWarp / D;             // nodes per weight batch
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int4 cur;
  C* tile = reinterpret_cast<C*>(smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  T* wb = reinterpret_cast<T*>(smem + tl.smem_tile) + warp * (NB * D * W);
  const int r = lane / W, l_last = lane - r * W;
  const bool lane_on = r < R;
  const int S = tl.S;
  const int64_t PS = (int64_t)tl.R1 * S;    // plane stride (d = 3)
  const T* sfrac = reinterpret_cast<const T*>(bins.sfrac);
  const T norm = (T)geo.norm;

  while (next_item(bins, SPREAD ? 1 : 0, &cur)) {
    const int4 item = cur;
    const TileOrigin o = decode_tile(geo, tl, item.x);
    if (SPREAD) {
      const int rows = D == 3 ? tl.E[0] * tl.E[1] : tl.E[0];
      C z;
      z.x = (T)0;
      z.y = (T)0;
      for (int e = threadIdx.x; e < rows * S; e += blockDim.x) tile[e] = z;
    } else {
      load_tile<D, C>(tile, in + o.inst * geo.ntot, geo, tl, o, warp, nwarps, lane);
    }
    __syncthreads();

    for (int64_t bs = item.y + (int64_t)warp * NB; bs < item.z; bs += (int64_t)nwarps * NB) {
      const int nb = (int)min((int64_t)NB, item.z - bs);
      compute_batch_weights<D, W, T>(wb, sfrac, bs, nb, geo, lane);
      __syncwarp();
      for (int q = 0; q < nb; ++q) {
        const int64_t k = bs + q;
        const int idx = bins.sidx[k];
        const uint32_t off = (uint32_t)bins.soff[k];
        const T* wq = wb + q * D * W;
        const T w_last = wq[(D - 1) * W + (lane_on ? l_last : 0)];
        T wrow[NIT];
#pragma unroll
        for (int it = 0; it < NIT; ++it) {
          const int lr = r + it * R;
          wrow[it] = (lane_on && lr < W) ? wq[(D - 2) * W + lr] : (T)0;
        }
        int64_t base;
        if (D == 3) {
          const int o0 = off & 1023, o1 = (off >> 10) & 1023, o2 = off >> 20;
          base = o0 * PS + (int64_t)(o1 + r) * S + o2 + l_last;
        } else {
          const int o0 = off & 1023, o1 = (off >> 10) & 1023;
          base = (int64_t)(o0 + r) * S + o1 + l_last;
        }
        T wpl[D == 3 ? W : 1];  // plane weights (d = 3), held in registers
        if (D == 3) {
#pragma unroll
          for (int l0 = 0; l0 < W; ++l0) wpl[l0] = wq[l0];
        }
        if (!SPREAD) {
          C acc;
          acc.x = (T)0;
          acc.y = (T)0;
          if (lane_on) {
#pragma unroll
            for (int it = 0; it < NIT; ++it) {
              if (r + it * R < W) {
                const C* row = tile + base + (int64_t)it * R * S;
                C ra;
                if (D == 3) {
                  ra.x = (T)0;
                  ra.y = (T)0;
#pragma unroll
                  for (int l0 = 0; l0 < W; ++l0) ra = cmul_add(ra, wpl[l0], row[l0 * PS]);
                } else {
                  ra = row[0];
                }
                acc = cmul_add(acc, wrow[it], ra);
              }
            }
            acc = cscale(acc, w_last);
          }
#pragma unroll
          for (int s = 16; s >= 1; s >>= 1) {
            C o2 = shfl_xor_c<C>(acc, s);
            acc.x += o2.x;
            acc.y += o2.y;
          }
          if (lane == 0) out[idx] = cscale(acc, norm);
        } else {
          const C v = cscale(in[idx], norm * w_last);
          if (lane_on) {
#pragma unroll
            for (int it = 0; it < NIT; ++it) {
              if (r + it * R < W) {
                C* row = tile + base + (int64_t)it * R * S;
                const C vr = cscale(v, wrow[it]);
                if (D == 3) {
#pragma unroll
                  for (int l0 = 0; l0 < W; ++l0) {
                    const C t = cscale(vr, wpl[l0]);
                    atomicAdd(&row[l0 * PS].x, t.x);
                    atomicAdd(&row[l0 * PS].y, t.y);
                  }
                } else {
                  atomicAdd(&row[0].x, vr.x);
                  atomicAdd(&row[0].y, vr.y);
                }
              }
            }
          }
        }
      }
      __syncwarp();
    }
    __syncthreads();
    if (SPREAD) {
      flush_tile<D, C>(tile, out + o.inst * geo.ntot, geo, tl, o, warp, nwarps, lane);
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// d = 1: R = 32/W nodes per warp pass, lane (node r, tap l)
// ---------------------------------------------------------------------------
template <int W, typename T, bool SPREAD>
__global__ void __launch_bounds__(512) k_grid1(const typename Cx<T>::t* __restrict__ in,
                                               typename Cx<T>::t* __restrict__ out,
                                               Geom geo, Tiling tl, Bins bins) {
  using C = typename Cx<T>::t;
  constexpr int R = kWarp / W;
  constexpr int NB = kWarp;   // weights of 32 nodes per batch (one lane each)
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int4 cur;
  C* tile = reinterpret_cast<C*>(smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  T* wb = reinterpret_cast<T*>(smem + tl.smem_tile) + warp * (NB * W);
  const int r = lane / W, l = lane - r * W;
  const bool lane_on = r < R;
  const T* sfrac = reinterpret_cast<const T*>(bins.sfrac);
  const T norm = (T)geo.norm;

  while (next_item(bins, SPREAD ? 1 : 0, &cur)) {
    const int4 item = cur;
    const TileOrigin o = decode_tile(geo, tl, item.x);
    if (SPREAD) {
      C z;
      z.x = (T)0;
      z.y = (T)0;
      for (int e = threadIdx.x; e < tl.S; e += blockDim.x) tile[e] = z;
    } else {
      load_tile<1, C>(tile, in + o.inst * geo.ntot, geo, tl, o, warp, nwarps, lane);
    }
    __syncthreads();
    for (int64_t bs = item.y + (int64_t)warp * NB; bs < item.z; bs += (int64_t)nwarps * NB) {
      const int nb = (int)min((int64_t)NB, item.z - bs);
      compute_batch_weights<1, W, T>(wb, sfrac, bs, nb, geo, lane);
      __syncwarp();
      for (int q0 = 0; q0 < nb; q0 += R) {
        const int q = q0 + r;
        const bool on = lane_on && q < nb;
        const int64_t k = bs + (on ? q : q0);
        const int idx = bins.sidx[k];
        const int o0 = bins.soff[k] & 1023;
        const T w = on ? wb[q * W + l] : (T)0;
        if (!SPREAD) {
          C acc = on ? cscale(tile[o0 + l], w) : C{(T)0, (T)0};
          // segmented reduction over the W lanes of node r
#pragma unroll
          for (int s = 1; s < W; s <<= 1) {
            C o2;
            o2.x = __shfl_down_sync(0xffffffffu, acc.x, s);
            o2.y = __shfl_down_sync(0xffffffffu, acc.y, s);
            if (l + s < W) {
              acc.x += o2.x;
              acc.y += o2.y;
            }
          }
          if (on && l == 0) out[idx] = cscale(acc, norm);
        } else if (on) {
          const C v = cscale(in[idx], norm * w);
          atomicAdd(&tile[o0 + l].x, v.x);
          atomicAdd(&tile[o0 + l].y, v.y);
        }
      }
      __syncwarp();
    }
    __syncthreads();
    if (SPREAD) {
      flush_tile<1, C>(tile, out + o.inst * geo.ntot, geo, tl, o, warp, nwarps, lane);
      __syncthreads();
    }
  }
}

}  // namespace cg
