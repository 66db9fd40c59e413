// kernels_spread_tc.cuh -- 3D FP32 spreading on the tensor cores (tcgen05, 3xTF32).
//
// Same work items, tiles and weights as k_spread (kernels_grid.cuh).  For a tile
// with padded extents E0 x E1 x E2 and a batch of K nodes, the update
//     G[p0, p1, p2] += sum_j w0_j[p0 - o0_j] w1_j[p1 - o1_j] w2_j[p2 - o2_j] f_j
// is the product D += A B^T of
//     A[(p0, p1), j]     = w0_j[p0 - o0_j] w1_j[p1 - o1_j]      (E0 E1 rows, real)
//     B[(p2, re|im), j]  = w2_j[p2 - o2_j] (Re f_j | Im f_j)    (2 E2 <= 64 rows)
// (weights are zero outside a node's window).  D lives in tensor memory: row
// (p0, p1) is TMEM lane (row mod 128) of M-tile row / 128, column 2 p2 + (re|im).
//
// Per batch of kTcK = 16 nodes the CTA (1) stages the node records, (2) evaluates
// w0 and w1 over the padded planes/rows and builds B, (3) builds A; operands are
// split into TF32 hi + lo parts (hi = tf32(v), lo = v - hi), and the thread
// mappings write 128 contiguous bytes per 8-lane store phase (no bank
// conflicts).  One thread then issues, per M-tile
// and k-step of 8 nodes, the three MMAs hi*hi + hi*lo + lo*hi (FP32 accuracy,
// error ~2^-22 relative per product) and commits them to the stage's mbarrier.
// Operands are double-buffered: batch b + 1 is built while the MMAs of batch b run.
// At the end of a work item the accumulators go TMEM -> registers -> a shared-
// memory tile (aliasing the operand buffers) and are added to the global grid
// by the 16-byte-atomic flush shared with the other spreading kernels.
//
// Every mbarrier wait is bounded; a wait that gives up sets the plan's device
// status flag, the kernel still drains (bounded), frees its tensor memory and
// returns.  Tensor-memory allocation cannot contend: the launcher sizes shared
// memory so that the CTAs resident on one SM never ask for more than 512 columns.
#pragma once

#include "kernels_grid.cuh"
#include "tc_sm100.cuh"

namespace cg {

constexpr int kTcMaxT0 = 16;     // outer tile extent limit (E0 <= 31 planes)
constexpr int kTcK = 16;         // nodes per staged batch: two TF32 k-steps of 8
constexpr int kTcThreads = 512;
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcN = 64;         // MMA N: 2 E2 <= 62 columns (p2, re/im), padded
constexpr int kTcWxStride = 20;  // floats per expanded-weight row: 8 consecutive rows hit distinct banks
// one node-record buffer, in int4 units: [kTcK] int4 window starts, [kTcK] float2
// values (kTcK / 2 int4), [kTcK][4] float fractions (kTcK int4)
constexpr int kTcRecInt4 = kTcK + kTcK / 2 + kTcK;
constexpr uint32_t kTcLBO = 128;                // core matrices along K
constexpr uint32_t kTcSBO = (kTcK / 4) * 128;   // 8-row groups
constexpr uint32_t kTcPolls = 1u << 22;         // mbarrier polls before giving up

__host__ __device__ constexpr bool spread_tc_ok(int d, int W, int T0) {
  return d == 3 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kTcMaxT0;
}

// Shared-memory layout of k_spread_tc (byte offsets; host and device agree).
struct TcLayout {
  int mt;                 // M-tiles of 128 rows covering E0 E1 rows
  uint32_t a_bytes;       // one A part (hi or lo) of one stage
  uint32_t stage_bytes;   // A hi, A lo, B hi, B lo
  uint32_t rec_off;       // 2 x ([kTcK] int4 window starts, [kTcK] float2 values, [kTcK][4] fractions)
  uint32_t wx0_off;       // [E0][kTcWxStride] w0 expanded over planes
  uint32_t wx1_off;       // [E1][kTcWxStride] w1 expanded over rows
  uint32_t bar_off;       // 2 mbarriers, tensor-memory base
  uint32_t total;
  uint32_t tmem_cols;     // power of two >= 32
};

__host__ __device__ inline TcLayout tc_layout(int W, int E0, size_t tile_bytes) {
  TcLayout L{};
  const int E1 = fixed_t_mid(3, W) + W - 1;
  const int rows = E0 * E1;
  L.mt = (rows + 127) / 128;
  L.a_bytes = (uint32_t)L.mt * 128u * kTcK * 4u;
  const uint32_t b_bytes = kTcN * kTcK * 4u;
  L.stage_bytes = 2u * L.a_bytes + 2u * b_bytes;
  uint32_t ops = 2u * L.stage_bytes;
  if (tile_bytes > ops) ops = (uint32_t)tile_bytes;
  ops = (ops + 1023u) & ~1023u;
  L.rec_off = ops;
  L.wx0_off = L.rec_off + 2u * kTcRecInt4 * 16u;
  L.wx1_off = L.wx0_off + (uint32_t)E0 * kTcWxStride * 4u;
  L.bar_off = (L.wx1_off + (uint32_t)E1 * kTcWxStride * 4u + 15u) & ~15u;
  L.total = L.bar_off + 32u;
  uint32_t c = 32;
  while (c < (uint32_t)L.mt * kTcN) c <<= 1;
  L.tmem_cols = c;
  return L;
}

// byte offset of element (row 8 rg + ri, node group kg) in a K-major no-swizzle operand
__device__ __forceinline__ uint32_t tc_elem_off(int rg, int ri, int kg) {
  return (uint32_t)rg * kTcSBO + (uint32_t)kg * kTcLBO + (uint32_t)ri * 16u;
}

__device__ __forceinline__ void tc_split4(float4 v, float4& hi, float4& lo) {
  hi.x = tc::tf32_round(v.x);
  hi.y = tc::tf32_round(v.y);
  hi.z = tc::tf32_round(v.z);
  hi.w = tc::tf32_round(v.w);
  lo.x = v.x - hi.x;
  lo.y = v.y - hi.y;
  lo.z = v.z - hi.z;
  lo.w = v.w - hi.w;
}

// tap weight exp(-(fr + m - l)^2 / b) (as WeightMath<float>::taps), zero outside the window
__device__ __forceinline__ float tc_tap(float fr, float mf, int l, int W, float cb) {
  const float y = fr + (mf - (float)l);
  return (unsigned)l < (unsigned)W ? exp2f(-(y * y) * cb) : 0.f;
}

// Flush of the shared-memory tile (layout of k_spread: row (p0, p1) at p0 PS + p1 S)
// to the global grid: warp w takes rows 2 w, 2 w + 1, then + 2 kTcWarps; lane
// (half, k) adds the column pair (2k, 2k + 1) of row 2 w + half with one 16-byte
// atomic (the pair never straddles the power-of-two wrap: tile origins and 2k are
// even).  All extents but E0 are compile-time, so no runtime division.
template <int W>
__device__ __forceinline__ void tc_flush(const float2* tile, float2* __restrict__ gi, const Geom& geo,
                                         const Tiling& tl, const TileOrigin& o) {
  constexpr int E1 = fixed_t_mid(3, W) + W - 1;
  constexpr int S = fixed_row_stride(3, W), PS = fixed_plane_stride(3, W);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane >> 4, k = lane & 15;
  const int E0a = tl.E[0], E1a = tl.E[1], E2a = tl.E[2];
  const int64_t n0 = geo.n[0], n1 = geo.n[1], n2 = geo.n[2];
  const int p2 = 2 * k;
  const bool on = p2 < E2a;
  const int64_t col = wrap_pow2(o.a[2] + p2, n2);
  const int rows = E0a * E1;
  for (int r = 2 * warp + half; r < rows; r += 2 * kTcWarps) {
    const int p0 = r / E1, p1 = r - p0 * E1;
    if (!on || p1 >= E1a) continue;
    const float2* src = tile + p0 * PS + p1 * S + p2;
    const float4 v = *reinterpret_cast<const float4*>(src);
    float2* dst = gi + (wrap_pow2(o.a[0] + p0, n0) * n1 + wrap_pow2(o.a[1] + p1, n1)) * n2 + col;
    if (p2 + 1 < E2a) {
      if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) atomicAdd(reinterpret_cast<float4*>(dst), v);
    } else if (v.x != 0.f || v.y != 0.f) {
      atomicAdd(dst, make_float2(v.x, v.y));
    }
  }
}

template <int W>
__global__ void __launch_bounds__(kTcThreads, 1) k_spread_tc(const float2* __restrict__ f, float2* __restrict__ g,
                                                             Geom geo, Tiling tl, Bins bins) {
  constexpr int T1 = fixed_t_mid(3, W), T2 = fixed_t_last(3, W);
  constexpr int E1 = T1 + W - 1, E2 = T2 + W - 1;
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr int S = fixed_row_stride(3, W), PS = fixed_plane_stride(3, W);
  constexpr int kMaxMt = (kTcMaxT0 + W - 1) * E1 / 128 + 1;  // M-tiles at the largest E0
  constexpr int kIssuer = kTcThreads - 32;                     // lane 0 of the last warp issues the MMAs
  static_assert(2 * E2 <= kTcN, "complex columns must fit the MMA N");
  static_assert(S > E2 && S % 2 == 0 && PS % 2 == 0, "pair stores need a padding column and even strides");
  static_assert(kTcWarps * 8 >= kTcN && kTcK == 16, "staging roles assume 16 nodes and 8 B-row warps");
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int4 cur;
  const int E0 = tl.E[0];
  const TcLayout L = tc_layout(W, E0, tl.smem_tile);
  // two record buffers: [kTcK] int4 window starts, [kTcK] float2 values, [kTcK][4] fractions
  int4* rec_buf = reinterpret_cast<int4*>(smem + L.rec_off);
  float* wx0 = reinterpret_cast<float*>(smem + L.wx0_off);
  float* wx1 = reinterpret_cast<float*>(smem + L.wx1_off);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L.bar_off);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ri = lane & 7, kg = lane >> 3;  // operand builds: row in group, node group of 4
  const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
  const float norm = (float)geo.norm;
  const float mf = (float)geo.m;
  const float cb0 = geo.cbf[0], cb1 = geo.cbf[1], cb2 = geo.cbf[2];
  const int rows = E0 * E1;

  // this thread's A rows (row groups warp + kTcWarps i): float offsets into wx0 / wx1, -1 past the tile
  int a_off0[(kMaxMt * 16 + kTcWarps - 1) / kTcWarps], a_off1[(kMaxMt * 16 + kTcWarps - 1) / kTcWarps];
#pragma unroll
  for (int i = 0; i < (kMaxMt * 16 + kTcWarps - 1) / kTcWarps; ++i) {
    const int r = (warp + kTcWarps * i) * 8 + ri;
    const int p0 = r / E1, p1 = r - p0 * E1;
    a_off0[i] = r < rows ? p0 * kTcWxStride + kg * 4 : -1;
    a_off1[i] = p1 * kTcWxStride + kg * 4;
  }

  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_fence_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, L.tmem_cols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  // descriptors of the stage operands at k-step 0, M-tile 0; other (M-tile, k-step)
  // pairs add their byte offset >> 4 to the 14-bit start-address field (no carry:
  // shared memory ends below 2^18 bytes)
  const uint32_t sa0 = tc::smem_u32(smem), sb0 = sa0 + 2 * L.a_bytes;
  const uint64_t d_ah = tc::smem_desc(sa0, kTcLBO, kTcSBO);
  const uint64_t d_al = tc::smem_desc(sa0 + L.a_bytes, kTcLBO, kTcSBO);
  const uint64_t d_bh = tc::smem_desc(sb0, kTcLBO, kTcSBO);
  const uint64_t d_bl = tc::smem_desc(sb0 + kTcN * kTcK * 4, kTcLBO, kTcSBO);
  const uint64_t d_stage = (uint64_t)(L.stage_bytes >> 4);  // stage 1 = stage 0 + d_stage
  uint32_t commits0 = 0, commits1 = 0, waits0 = 0, waits1 = 0;  // CTA-uniform
  bool healthy = true;

  // record roles: thread j < kTcK loads node j; threads kTcK .. 4 kTcK - 1 load fraction (j, t)
  const int fq = (tid - kTcK) / 3, ft = (tid - kTcK) - 3 * ((tid - kTcK) / 3);
  const bool is_frac = tid >= kTcK && tid < 4 * kTcK;
  float pf_fr = 0.f;
  int pf_off = 0;
  float2 pf_val = make_float2(0.f, 0.f);
  auto fetch = [&](int base, int end) {  // registers <- records of nodes base .. min(base + kTcK, end)
    const int nbn = min(kTcK, end - base);
    if (is_frac && fq < nbn) pf_fr = sfrac[(int64_t)(base + fq) * 3 + ft];
    if (tid < nbn) {
      pf_off = bins.soff[base + tid];
      pf_val = f[bins.sidx[base + tid]];
    }
  };
  auto stash = [&](int rb, int nbn) {  // record buffer rb <- registers
    int4* rec = rec_buf + rb * kTcRecInt4;
    if (tid < kTcK) {
      const uint32_t off = (uint32_t)pf_off;
      rec[tid] = tid < nbn ? make_int4((int)(off & MASK), (int)((off >> SH) & MASK), (int)(off >> (2 * SH)), 0)
                           : make_int4(1 << 20, 1 << 20, 1 << 20, 0);  // empty slot: no window
      reinterpret_cast<float2*>(rec + kTcK)[tid] = cscale(pf_val, norm);
    }
    if (is_frac) reinterpret_cast<float*>(rec + kTcK + kTcK / 2)[fq * 4 + ft] = pf_fr;
  };

  while (next_item(bins, 1, &cur)) {
    const int4 item = cur;
    if (item.z <= item.y) continue;  // next_item's barrier keeps `cur` safe
    fetch(item.y, item.z);
    stash(0, min(kTcK, item.z - item.y));
    __syncthreads();
    int b = 0;
    for (int bs = item.y; bs < item.z; bs += kTcK, ++b) {
      const int s = b & 1;
      const int bn = bs + kTcK;
      if (bn < item.z) fetch(bn, item.z);  // consumed at the end of this batch
      const int4* rec = rec_buf + s * kTcRecInt4;
      const float2* cval = reinterpret_cast<const float2*>(rec + kTcK);
      const float* frac = reinterpret_cast<const float*>(rec + kTcK + kTcK / 2);
      // stage s is free once the MMAs of batch b - 2 are complete
      if (s == 0 && commits0 > waits0) {
        healthy &= tc::mbar_wait_bounded(&bar[0], waits0 & 1u, kTcPolls);
        ++waits0;
      } else if (s == 1 && commits1 > waits1) {
        healthy &= tc::mbar_wait_bounded(&bar[1], waits1 & 1u, kTcPolls);
        ++waits1;
      }
      unsigned char* stage = smem + (size_t)s * L.stage_bytes;
      unsigned char* a_hi = stage;
      unsigned char* a_lo = stage + L.a_bytes;
      unsigned char* b_hi = stage + 2 * L.a_bytes;
      unsigned char* b_lo = b_hi + kTcN * kTcK * 4;
      // (2) warps 0..7: B rows 8 w .. 8 w + 7; warps 8..: w0 and w1 expanded over planes and rows
      if (warp < kTcN / 8) {
        const int n = warp * 8 + ri, p2 = n >> 1, part = n & 1;
        float vv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = kg * 4 + u;
          const float w2 = tc_tap(frac[j * 4 + 2], mf, p2 - rec[j].z, W, cb2);
          const float2 c = cval[j];
          vv[u] = w2 * (part ? c.y : c.x);
        }
        float4 hi, lo;
        tc_split4(make_float4(vv[0], vv[1], vv[2], vv[3]), hi, lo);
        const uint32_t o = tc_elem_off(warp, ri, kg);
        *reinterpret_cast<float4*>(b_hi + o) = hi;
        *reinterpret_cast<float4*>(b_lo + o) = lo;
      } else {
        for (int i = tid - (kTcN / 8) * 32; i < (E0 + E1) * kTcK; i += kTcThreads - (kTcN / 8) * 32) {
          const int j = i & (kTcK - 1), p = i / kTcK;
          const int4 r = rec[j];
          if (p < E0) wx0[p * kTcWxStride + j] = tc_tap(frac[j * 4 + 0], mf, p - r.x, W, cb0);
          else wx1[(p - E0) * kTcWxStride + j] = tc_tap(frac[j * 4 + 1], mf, (p - E0) - r.y, W, cb1);
        }
      }
      __syncthreads();
      // (3) A: warp w builds row groups w, w + 16, ...; rows past E0 E1 are zero
#pragma unroll
      for (int i = 0; i < (kMaxMt * 16 + kTcWarps - 1) / kTcWarps; ++i) {
        const int rg = warp + kTcWarps * i;
        if (rg < L.mt * 16) {
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (a_off0[i] >= 0) {
            const float4 a = *reinterpret_cast<const float4*>(wx0 + a_off0[i]);
            const float4 c = *reinterpret_cast<const float4*>(wx1 + a_off1[i]);
            v = make_float4(a.x * c.x, a.y * c.y, a.z * c.z, a.w * c.w);
          }
          float4 hi, lo;
          tc_split4(v, hi, lo);
          const uint32_t o = tc_elem_off(rg, ri, kg);
          *reinterpret_cast<float4*>(a_hi + o) = hi;
          *reinterpret_cast<float4*>(a_lo + o) = lo;
        }
      }
      if (bn < item.z) stash(s ^ 1, min(kTcK, item.z - bn));  // records of batch b + 1
      tc::fence_proxy_async_smem();  // generic-proxy operand writes -> tensor core
      __syncthreads();
      if (tid == kIssuer) {
        tc::fence_after_sync();
        const uint32_t idesc = tc::idesc_tf32(128, kTcN);
        const uint64_t so = s ? d_stage : 0ull;
        for (int mt = 0; mt < L.mt; ++mt) {
          const uint32_t d = tmem + (uint32_t)(mt * kTcN);
          const uint64_t am = so + (uint64_t)((mt * 16 * kTcSBO) >> 4);
#pragma unroll
          for (int ks = 0; ks < kTcK / 8; ++ks) {
            const uint64_t ko = (uint64_t)((ks * 2 * kTcLBO) >> 4);
            tc::mma_tf32(d, d_ah + am + ko, d_bh + so + ko, idesc, (b > 0 || ks > 0) ? 1u : 0u);
            tc::mma_tf32(d, d_ah + am + ko, d_bl + so + ko, idesc, 1u);
            tc::mma_tf32(d, d_al + am + ko, d_bh + so + ko, idesc, 1u);
          }
        }
        tc::mma_commit(&bar[s]);
      }
      if (s == 0) ++commits0;
      else ++commits1;
    }
    // drain: every commit of this item completes before the accumulators are read
    if (commits0 > waits0) {
      healthy &= tc::mbar_wait_bounded(&bar[0], waits0 & 1u, kTcPolls);
      ++waits0;
    }
    if (commits1 > waits1) {
      healthy &= tc::mbar_wait_bounded(&bar[1], waits1 & 1u, kTcPolls);
      ++waits1;
    }
    tc::fence_after_sync();
    // TMEM -> shared tile: warp w reads lanes 32 (w % 4) .. + 31 and the 16 columns
    // (8 complex values) 16 (w / 4) .. + 15; 16-byte stores of (p2, p2 + 1) pairs
    // (the padding column S - 1 >= E2 takes the odd tail)
    float2* tile = reinterpret_cast<float2*>(smem);
    {
      const int q = warp & 3, h = warp >> 2;
      for (int mt = 0; mt < L.mt; ++mt) {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(mt * kTcN + h * 16), v);
        tc::tmem_ld_wait();
        const int r = mt * 128 + 32 * q + lane;
        if (r < rows) {
          const int p0 = r / E1, p1 = r - p0 * E1;
          float2* dst = tile + p0 * PS + p1 * S + h * 8;
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (h * 8 + 2 * u < E2)
              *reinterpret_cast<float4*>(dst + 2 * u) = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    const TileOrigin o = decode_tile<3>(geo, tl, item.x);
    tc_flush<W>(tile, g + o.inst * geo.ntot, geo, tl, o);
    __syncthreads();  // the tile aliases the operand buffers of the next item
  }
  // teardown: nothing of ours is in flight unless a wait gave up; give it one more bounded chance
  if (commits0 > waits0) healthy &= tc::mbar_wait_bounded(&bar[0], waits0 & 1u, kTcPolls);
  if (commits1 > waits1) healthy &= tc::mbar_wait_bounded(&bar[1], waits1 & 1u, kTcPolls);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, L.tmem_cols);
  if (!healthy && lane == 0) atomicExch(bins.status, 2);
}

}  // namespace cg
