// kernels_spread_reg.cuh -- 3D FP32 spreading with the output tile held in registers.
//
// Same work items, tiles and weights as k_spread (kernels_grid.cuh), different data
// flow: the CTA has one warp per plane p0 of the padded tile (E0 = T0 + W - 1
// warps) and lane p2 of warp p0 holds the column (p0, :, p2) of the tile, E1
// complex accumulators in registers.  A node j with window start (o0, o1, o2)
// adds
//     (f_j w0_j[p0 - o0] w2_j[p2 - o2]) * w1_j[p1 - o1],   p1 = o1 .. o1 + W - 1,
// with one packed f32x2 FMA per row; a branch tree on o1 (T1 leaves) keeps every
// register index static.  Per-node weights and records are staged in shared
// memory in double-buffered batches of kRegBatch nodes; the shared-memory
// read-modify-write of the tile, the bound of the shared-tile kernel, is gone.
// The finished tile is parked in shared memory and added to the global grid with
// 16-byte atomics.
#pragma once

#include "kernels_grid.cuh"

namespace cg {

constexpr int kRegMaxT0 = 8;    // largest outer tile extent: E0 <= 8 + W - 1 warps per CTA
constexpr int kRegBatch = 32;   // nodes per staged batch

// Whether the register kernel covers a plan: FP32, d = 3, W <= 16 (E2 = 16 + W - 1
// columns fit in a warp), T0 <= kRegMaxT0.
__host__ __device__ constexpr bool spread_reg_ok(int d, int W, int T0) {
  return d == 3 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kRegMaxT0;
}

template <int W>
struct RegNode {
  float2 w1p[W];  // (w1, w1) pairs, the packed-FMA weight operand
  float w0[W];
  float w2[W];
  float2 c;       // f_j * norm
  int off;        // packed tile-local window start, 10 bits per dim
  int pad;
};

template <int W>
__host__ __device__ constexpr int spread_reg_threads_max() { return 32 * (kRegMaxT0 + W - 1); }

// dynamic shared memory: the batch buffers, aliased by the tile (tile_bytes) for the flush
template <int W>
__host__ __device__ constexpr size_t spread_reg_smem(size_t tile_bytes) {
  return 2 * kRegBatch * sizeof(RegNode<W>) > tile_bytes ? 2 * kRegBatch * sizeof(RegNode<W>) : tile_bytes;
}

template <int W, int E1, int K>
__device__ __forceinline__ void reg_rows(float2 (&acc)[E1], const float2* __restrict__ w1p, float2 cb) {
#pragma unroll
  for (int l1 = 0; l1 < W; ++l1) acc[K + l1] = __ffma2_rn(w1p[l1], cb, acc[K + l1]);
}

// rows o1 .. o1 + W - 1 for o1 in [LO, HI), by bisection
template <int W, int E1, int LO, int HI>
__device__ __forceinline__ void reg_tree(float2 (&acc)[E1], int o1, const float2* __restrict__ w1p, float2 cb) {
  if constexpr (HI - LO == 1) {
    reg_rows<W, E1, LO>(acc, w1p, cb);
  } else {
    constexpr int MID = (LO + HI) / 2;
    if (o1 < MID) reg_tree<W, E1, LO, MID>(acc, o1, w1p, cb);
    else reg_tree<W, E1, MID, HI>(acc, o1, w1p, cb);
  }
}

template <int W>
__global__ void __launch_bounds__(spread_reg_threads_max<W>()) k_spread_reg(const float2* __restrict__ f,
                                                                          float2* __restrict__ g, Geom geo,
                                                                          Tiling tl, Bins bins) {
  constexpr int T1 = fixed_t_mid(3, W), T2 = fixed_t_last(3, W);
  constexpr int E1 = T1 + W - 1;
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  static_assert(T2 + W - 1 <= 32, "columns must fit in a warp");
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int4 cur;
  RegNode<W>* stage = reinterpret_cast<RegNode<W>*>(smem);  // [2][kRegBatch]
  const int lane = threadIdx.x & 31, p0 = threadIdx.x >> 5;  // warp p0 owns plane p0
  const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
  const float norm = (float)geo.norm;
  // staging role: (node sq, dim st) for the weights, node threadIdx.x for the record
  const int sq = threadIdx.x / 3, st = threadIdx.x - sq * 3;
  const TapK tks = tap_k(geo, st);
  const bool es = geo.window == kWinES;
  const float mf = (float)geo.m;

  while (next_item(bins, 1, &cur)) {
    const int4 item = cur;
    float2 acc[E1];
#pragma unroll
    for (int i = 0; i < E1; ++i) acc[i] = make_float2(0.f, 0.f);
    float pf_fr = 0.f;
    int pf_off = 0;
    float2 pf_val = make_float2(0.f, 0.f);
    {
      const int nb0 = min(kRegBatch, item.z - item.y);
      if (sq < nb0) pf_fr = sfrac[(int64_t)(item.y + sq) * 3 + st];
      if ((int)threadIdx.x < nb0) {
        pf_off = bins.soff[item.y + threadIdx.x];
        pf_val = f[bins.sidx[item.y + threadIdx.x]];
      }
    }
    int buf = 0;
    for (int bs = item.y; bs < item.z; bs += kRegBatch, buf ^= 1) {
      const int nb = min(kRegBatch, item.z - bs);
      RegNode<W>* sb = stage + buf * kRegBatch;
      if (sq < nb) {
        // tap l of dim st at y = fr + m - l, as WeightMath<float>::taps
        RegNode<W>& nd = sb[sq];
        float wt[W];
        if (es) {
#pragma unroll
          for (int l = 0; l < W; ++l) wt[l] = win_tap<kWinES>(pf_fr + (mf - (float)l), tks);
        } else {
#pragma unroll
          for (int l = 0; l < W; ++l) wt[l] = win_tap<kWinGauss>(pf_fr + (mf - (float)l), tks);
        }
#pragma unroll
        for (int l = 0; l < W; ++l) {
          if (st == 0) nd.w0[l] = wt[l];
          else if (st == 1) nd.w1p[l] = make_float2(wt[l], wt[l]);
          else nd.w2[l] = wt[l];
        }
      }
      if ((int)threadIdx.x < nb) {
        sb[threadIdx.x].off = pf_off;
        sb[threadIdx.x].c = cscale(pf_val, norm);
      }
      const int bn = bs + kRegBatch;
      if (bn < item.z) {
        const int nbn = min(kRegBatch, item.z - bn);
        if (sq < nbn) pf_fr = sfrac[(int64_t)(bn + sq) * 3 + st];
        if ((int)threadIdx.x < nbn) {
          pf_off = bins.soff[bn + threadIdx.x];
          pf_val = f[bins.sidx[bn + threadIdx.x]];
        }
      }
      // One barrier per batch suffices: a warp restages buffer buf ^ 1 only after
      // every warp has passed this barrier, i.e. finished the batch held there.
      __syncthreads();
      for (int q = 0; q < nb; ++q) {
        const RegNode<W>& nd = sb[q];
        const uint32_t off = (uint32_t)nd.off;
        const int l0 = p0 - (int)(off & MASK);
        if ((unsigned)l0 >= (unsigned)W) continue;  // plane outside the node's window (warp-uniform)
        const int o1 = (off >> SH) & MASK, l2 = lane - (int)(off >> (2 * SH));
        const float wb = (unsigned)l2 < (unsigned)W ? nd.w2[l2] : 0.f;
        const float2 cb = cscale(nd.c, nd.w0[l0] * wb);
        reg_tree<W, E1, 0, T1>(acc, o1, nd.w1p, cb);
      }
    }
    // Park the columns in a shared-memory tile (aliasing the batch buffers, which
    // every warp has left once it reaches the barrier) and flush it as k_spread does.
    constexpr int S = fixed_row_stride(3, W), PS = fixed_plane_stride(3, W);
    float2* tile = reinterpret_cast<float2*>(smem);
    __syncthreads();
    if (lane < tl.E[2]) {
      float2* col = tile + p0 * PS + lane;
#pragma unroll
      for (int p1 = 0; p1 < E1; ++p1) col[p1 * S] = acc[p1];
    }
    __syncthreads();
    const TileOrigin o = decode_tile<3>(geo, tl, item.x);
    flush_tile<3, W, float2>(tile, g + o.inst * geo.ntot, geo, tl, o);
    __syncthreads();  // every warp is done with `cur` and the batch buffers
  }
}

}  // namespace cg
