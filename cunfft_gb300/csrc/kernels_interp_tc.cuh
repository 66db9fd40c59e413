// kernels_interp_tc.cuh -- 3D FP32 interpolation on the tensor cores (tcgen05, 3 x FP16),
// tile chunks streamed by TMA.
//
// Same work items, tiles and weights as k_interp (kernels_grid.cuh).  For a tile
// with padded extents E0 x E1 x E2 and a batch of up to 128 of its nodes,
//     f_j = norm sum_{p0, p1} w0_j[p0 - o0_j] w1_j[p1 - o1_j] H[j, (p0, p1)],
//     H[j, (p0, p1, re|im)] = sum_{p2} w2_j[p2 - o2_j] G[(p0, p1), p2] (re|im)
// and H is the product D = A B^T of
//     A[j, p2]              = w2_j[p2 - o2_j]                  (128 nodes x 32 columns)
//     B[(re|im, p0, p1), p2] = Re|Im G[p0, p1, p2]             (the tile, K = p2)
// computed in chunks of CH planes (the chunk's CH E1 <= 64 (plane, row) pairs are B
// rows 0.. of the real part and 64.. of the imaginary part: N = 128), four chunk
// accumulators in tensor memory.  D lives in tensor memory with node j in lane j, so
// the thread that owns node j finishes the w0 (x) w1 sum over its window from its own
// lane, chunk by chunk, in registers.
//
// Operands are FP16 hi + lo splits (11 + 11 significant bits, the precision of a TF32
// split) multiplied as hi*hi + hi*lo + lo*hi with FP32 accumulation, K = 16 per MMA.
// FP16's range is kept by exact powers of two: A (weights in [0, 1]) by 2^10, each
// padded plane p0 of the grid by 2^(14 - e_p0), 2^e_p0 >= its largest |Re|, |Im|;
// the node threads fold the inverse plane scales into their w0 weights.
//
// The grid is first split (k_split_planes) into those FP16 hi + lo parts of its real and
// imaginary parts, each an array over the periodically padded index range
// [0, n_t + W - 1) per dimension.  Every tile's padded box then lies inside the
// arrays (no wrap), and one thread loads each chunk with four TMA boxes (hi re, hi im,
// lo re, lo im; 32 halves x E1 rows x CH planes) straight into the 64-byte swizzled
// K-major layout the MMAs read.  Warp roles: warp 0 lane 0 issues the TMA loads
// (eight chunk stages), warp 1 lane 0 the MMAs, warps 2-13 (three per lane quarter)
// prepare their nodes' weights and A and reduce D.  Hand-offs are mbarriers (the chunk stages'
// with TMA transaction counts); every wait is bounded and a wait that gives up sets
// the plan's device status flag.
#pragma once

#include <cuda.h>
#include <type_traits>
#include <cuda_fp16.h>

#include "kernels_grid.cuh"
#include "tc_sm100.cuh"

namespace cg {

constexpr int kItMaxT0 = 16;       // outer tile extent limit (E0 <= 31 planes)
constexpr int kItK = 32;           // K: innermost tile columns p2 (E2 <= 31), padded; one 64-byte row
constexpr int kItNodes = 128;      // nodes per batch (MMA M)
constexpr int kItTmaWarp = 0;
constexpr int kItMmaWarp = 1;
constexpr int kItNodeWarp0 = 2;    // 12 node warps: lane quarter = warp % 4, part = (warp - 2) / 4
constexpr int kItNodeWarps = 12;
constexpr int kItParts = kItNodeWarps / 4;     // node warps per lane quarter
constexpr int kItThreads = (2 + kItNodeWarps) * 32;
constexpr int kItHalf = 64;                    // B rows per part: real parts 0..63, imaginary 64..127
constexpr int kItN = 2 * kItHalf;              // MMA N
constexpr int kItStages = 8;                   // chunk stages (TMA ring)
constexpr int kItAcc = 4;                      // tensor-memory accumulators of kItN columns
constexpr uint32_t kItLBO = 128;               // A: core matrices (8 rows x 8 halves) along K
constexpr uint32_t kItSBOA = 512;              // A: 8-row groups (32 K values = 4 core matrices)
constexpr uint32_t kItAPart = 128u * 64u;      // one A part (hi or lo): 128 rows x 64 bytes
constexpr uint32_t kItPart = kItHalf * 64;     // one B part (hi re, hi im, lo re, lo im): 64 rows x 64 bytes
constexpr uint32_t kItStage = 4 * kItPart;     // one chunk stage: B hi = parts 0-1, B lo = parts 2-3
constexpr float kItScaleA = 1024.f;            // A = w2 in [0, 1] -> [0, 2^10]
constexpr int kItWtStride = 55;                // floats per node in the weight table (odd: no bank conflicts)
constexpr int kItLogB = 14;                    // |B| scaled to below 2^14 per plane
constexpr uint32_t kItPolls = 1u << 20;        // mbarrier polls (<= 1 us each) before giving up

__host__ __device__ constexpr int it_e1(int W) { return fixed_t_mid(3, W) + W - 1; }
__host__ __device__ constexpr int it_ch(int W) { return kItHalf / it_e1(W); }                 // planes per chunk
__host__ __device__ constexpr int it_pairs(int W) { return it_ch(W) * it_e1(W); }            // (plane, row) pairs <= 64

// The innermost tile extent (a power of two <= 16, at most n2) must give TMA boxes a
// 16-byte aligned start: at least 8 halves.
__host__ __device__ constexpr bool interp_tc_ok(int d, int W, int T0, int64_t n2) {
  return d == 3 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kItMaxT0 && n2 >= 8 && n2 % 8 == 0;
}

// Shared-memory layout (byte offsets from a 1024-byte aligned base; host and device agree).
struct ItLayout {
  uint32_t b_off;      // kItStages chunk stages of kItStage
  uint32_t a_off;      // 2 buffers x (A hi, A lo)
  uint32_t bar_off;    // afull[2], bfull[8], bempty[8], tfull[4], tempty[4]; tensor-memory base
  uint32_t red_off;    // 2 x 2 x 128 float2: parts 1 and 2's partial sums per node
  uint32_t wt_off;     // [128][kItWtStride] floats: each node's w0 (planes) and w1 (rows) of the batch
  uint32_t total;      // bytes past the aligned base
  uint32_t dyn;        // dynamic shared memory to request (alignment slack included)
};

__host__ __device__ constexpr ItLayout it_layout() {
  return ItLayout{0u,
                  kItStages * kItStage,
                  kItStages * kItStage + 4u * kItAPart,
                  kItStages * kItStage + 4u * kItAPart + 256u,
                  kItStages * kItStage + 4u * kItAPart + 256u + 4096u,
                  kItStages * kItStage + 4u * kItAPart + 256u + 4096u + 128u * kItWtStride * 4u,
                  kItStages * kItStage + 4u * kItAPart + 256u + 4096u + 128u * kItWtStride * 4u + 1024u};
}

// Padded split planes of the grid: half [batch][4][P0][P1][P2s], component 0 hi re,
// 1 hi im, 2 lo re, 3 lo im; P_t = n_t + W - 1 holds grid index i mod n_t, P2s = P2
// rounded up to a multiple of 8 (16-byte rows).  Plane scales: float [batch][P0],
// the inverse 2^(e - 14) of each padded plane's scale, 2^e above the largest |Re|,
// |Im| of its grid plane (uint32 [batch][n0] maxima, float bits).
struct ItSplit {
  int64_t P0, P1, P2, P2s;
};
__host__ __device__ inline ItSplit it_split_dims(const Geom& g) {
  ItSplit s;
  s.P0 = g.n[0] + g.W - 1;
  s.P1 = g.n[1] + g.W - 1;
  s.P2 = g.n[2] + g.W - 1;
  s.P2s = (s.P2 + 7) / 8 * 8;
  return s;
}

// 4 FP32 values -> FP16 hi and lo = fp16(v - hi), 4 halves each
__device__ __forceinline__ void it_split4_f16(float4 v, uint2& hi, uint2& lo) {
  const __half2 h0 = __floats2half2_rn(v.x, v.y), h1 = __floats2half2_rn(v.z, v.w);
  const float2 f0 = __half22float2(h0), f1 = __half22float2(h1);
  const __half2 l0 = __floats2half2_rn(v.x - f0.x, v.y - f0.y), l1 = __floats2half2_rn(v.z - f1.x, v.w - f1.y);
  hi = make_uint2(*reinterpret_cast<const uint32_t*>(&h0), *reinterpret_cast<const uint32_t*>(&h1));
  lo = make_uint2(*reinterpret_cast<const uint32_t*>(&l0), *reinterpret_cast<const uint32_t*>(&l1));
}

// Four consecutive complex values as two float4 (one 16-byte load each when the
// address is 16-byte aligned, else four 8-byte loads: a caller's grid may be only
// 8-byte aligned)
__device__ __forceinline__ void ld_quad(const float2* src, bool al16, float4& a, float4& b) {
  if (al16) {
    a = reinterpret_cast<const float4*>(src)[0];
    b = reinterpret_cast<const float4*>(src)[1];
  } else {
    const float2 v0 = src[0], v1 = src[1], v2 = src[2], v3 = src[3];
    a = make_float4(v0.x, v0.y, v1.x, v1.y);
    b = make_float4(v2.x, v2.y, v3.x, v3.y);
  }
}

// 2^(14 - e) with 2^e > mx, as the exponent e
__device__ __forceinline__ int it_plane_exp(float mx) {
  int ex = 0;
  frexpf(mx, &ex);
  return ex;
}

constexpr int kItSplitThreads = 1024;

// The grid's padded FP16 hi/lo planes in one pass over the grid.  CTA c takes padded
// planes (instance, i0) c, c + G, ...: it reads grid plane i0 mod n0 once for its largest
// |Re|, |Im| (a block reduction), then again (from L2: the CTAs' planes in flight stay well
// below its size) to write the plane's P1 x P2s quads of FP16 hi + lo parts of the real
// and imaginary parts, scaled by the plane's 2^(14 - e), and the plane's inverse scale.
// A quad (4 consecutive p2 of one padded row) never straddles the grid's wrap (n2 % 8 == 0).
static __global__ void __launch_bounds__(kItSplitThreads) k_split_planes(const float2* __restrict__ g,
                                                                   __half* __restrict__ out,
                                                                   float* __restrict__ inv_scale, Geom geo,
                                                                   ItSplit sd) {
  __shared__ uint32_t wmax[kItSplitThreads / 32];
  const int64_t plane_elems = geo.n[1] * geo.n[2], q4 = sd.P2s / 4, comp = sd.P0 * sd.P1 * sd.P2s;
  const bool al16 = (reinterpret_cast<uintptr_t>(g) & 15u) == 0;  // n1 n2 is a multiple of 8
  for (int64_t pl = blockIdx.x; pl < sd.P0 * geo.batch; pl += gridDim.x) {
    const int64_t inst = pl / sd.P0, i0 = pl - inst * sd.P0;
    const float2* src = g + (inst * geo.n[0] + wrap_up(i0, geo.n[0])) * plane_elems;
    float mx = 0.f;
    for (int64_t e = threadIdx.x; e < plane_elems / 4; e += blockDim.x) {
      float4 a, b;
      ld_quad(src + 4 * e, al16, a, b);
      mx = fmaxf(mx, fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(a.w))),
                           fmaxf(fmaxf(fabsf(b.x), fabsf(b.y)), fmaxf(fabsf(b.z), fabsf(b.w)))));
    }
    const uint32_t wm = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = wm;
    __syncthreads();
    uint32_t m = 0;
#pragma unroll 8
    for (int w = 0; w < kItSplitThreads / 32; ++w) m = max(m, wmax[w]);
    __syncthreads();  // wmax is rewritten by the next plane
    const int ex = it_plane_exp(__uint_as_float(m));
    const float scale = ldexpf(1.f, kItLogB - ex);
    if (threadIdx.x == 0) inv_scale[inst * sd.P0 + i0] = ldexpf(1.f, ex - kItLogB);
    __half* const o_plane = out + inst * 4 * comp + i0 * sd.P1 * sd.P2s;
    // the second pass runs backwards: the plane's last lines, read most recently, are the
    // likeliest still in L2
    for (int64_t e = sd.P1 * q4 - 1 - threadIdx.x; e >= 0; e -= blockDim.x) {
      const int64_t i1 = e / q4, i2 = (e - i1 * q4) * 4;
      float4 a, b;
      ld_quad(src + wrap_up(i1, geo.n[1]) * geo.n[2] + wrap_up(i2, geo.n[2]), al16, a, b);
      __half* o = o_plane + i1 * sd.P2s + i2;
      uint2 h, l;
      it_split4_f16(make_float4(a.x * scale, a.z * scale, b.x * scale, b.z * scale), h, l);
      *reinterpret_cast<uint2*>(o) = h;
      *reinterpret_cast<uint2*>(o + 2 * comp) = l;
      it_split4_f16(make_float4(a.y * scale, a.w * scale, b.y * scale, b.w * scale), h, l);
      *reinterpret_cast<uint2*>(o + comp) = h;
      *reinterpret_cast<uint2*>(o + 3 * comp) = l;
    }
  }
}

// Position in this CTA's batch sequence: items c, c + G, ... (CTA c of G; items are
// never empty) and the batch of up to 128 nodes within the item; the following
// item's descriptor is loaded one item ahead.
struct ItCursor {
  int it, b;
  int4 item, next;
};
__device__ __forceinline__ void it_cursor_init(ItCursor& c, const Bins& bins, int num_items) {
  const int G = (int)gridDim.x;
  c.it = (int)blockIdx.x;
  c.b = 0;
  c.item = c.it < num_items ? bins.items[c.it] : make_int4(0, 0, 0, 0);
  c.next = c.it + G < num_items ? bins.items[c.it + G] : make_int4(0, 0, 0, 0);
}
__device__ __forceinline__ void it_cursor_step(ItCursor& c, const Bins& bins, int num_items) {
  const int G = (int)gridDim.x;
  if (c.it >= num_items) return;
  if (c.item.y + (++c.b) * kItNodes < c.item.z) return;
  c.it += G;
  c.b = 0;
  c.item = c.next;
  c.next = c.it + G < num_items ? bins.items[c.it + G] : make_int4(0, 0, 0, 0);
}

// One node's record, loaded from the bins into registers ahead of use.
struct ItRec {
  uint32_t off;  // packed window start (all ones: no node)
  float fr0, fr1, fr2;
  int idx;       // output index, -1: no node
};
__device__ __forceinline__ ItRec it_load_rec(const ItCursor& c, int num_items, int slot, const Bins& bins) {
  ItRec r{0xFFFFFFFFu, 0.f, 0.f, 0.f, -1};
  if (c.it >= num_items) return r;
  const int j = c.item.y + c.b * kItNodes + slot;
  if (j < c.item.z) {
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    r.off = (uint32_t)bins.soff[j];
    r.fr0 = sfrac[(int64_t)j * 3];
    r.fr1 = sfrac[(int64_t)j * 3 + 1];
    r.fr2 = sfrac[(int64_t)j * 3 + 2];
    r.idx = bins.sidx[j];
  }
  return r;
}

template <int W, int WIN>
__global__ void __launch_bounds__(kItThreads, 1) k_interp_tc(const __grid_constant__ CUtensorMap tmap,
                                                             const float* __restrict__ plane_inv,
                                                             float2* __restrict__ f, Geom geo, Tiling tl, Bins bins) {
  constexpr int E1 = it_e1(W), CH = it_ch(W), NP = it_pairs(W);
  constexpr int E0MAX = kItMaxT0 + W - 1;
  constexpr int MAXCH = (E0MAX + CH - 1) / CH;
  constexpr int GI = (NP + 15) / 16;  // 16-pair groups of the tensor-memory read-out
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr uint32_t kBoxBytes = (uint32_t)(kItK * 2 * E1 * CH);
  static_assert(NP <= kItHalf && NP > 0, "a chunk's (plane, row) pairs must fit one B part");
  static_assert(kItAcc * kItN <= 512, "the accumulators must fit tensor memory");
  static_assert(fixed_t_last(3, W) + W - 1 <= kItK, "innermost padded extent must fit K");
  static_assert(E0MAX + E1 <= kItWtStride, "a node's w0 and w1 must fit its weight-table row");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const ItLayout L = it_layout();
  uint64_t* afull = reinterpret_cast<uint64_t*>(smem + L.bar_off);  // [2] A of the batch built
  uint64_t* bfull = afull + 2;                                       // [8] tile chunk landed (TMA)
  uint64_t* bempty = afull + 2 + kItStages;                          // [8] MMAs of the chunk complete
  uint64_t* tfull = afull + 2 + 2 * kItStages;                       // [4] accumulator complete
  uint64_t* tempty = tfull + kItAcc;                                 // [4] accumulator read out
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + kItAcc);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int E0 = tl.E[0];
  const int nch = (E0 + CH - 1) / CH;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) tc::mbar_init(&afull[i], 4);  // one arrival per A-building (part 2) warp
    for (int i = 0; i < kItStages; ++i) {
      tc::mbar_init(&bfull[i], 1);    // the TMA thread's arrival (+ the boxes' bytes)
      tc::mbar_init(&bempty[i], 1);
    }
    for (int i = 0; i < kItAcc; ++i) {
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], kItNodeWarps);  // one arrival per node warp
    }
    tc::mbar_fence_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  bool healthy = true;

  // Every role walks items c, c + G, ... (CTA c), batches of 128 nodes within an
  // item and nch chunks within a batch; chunk gc (counted across the CTA's whole
  // sequence) uses chunk stage gc & 7 in its cycle gc >> 3 and accumulator gc & 3
  // in its cycle gc >> 2.
  if (warp == kItTmaWarp) {
    // ======================= TMA: tile chunks =======================
    if (lane == 0) {
      uint32_t gc = 0;
      for (int it = blockIdx.x; it < num_items; it += G) {
        const int4 item = bins.items[it];
        const TileOrigin o = decode_tile<3>(geo, tl, item.x);
        const int nbatch = (item.z - item.y + kItNodes - 1) / kItNodes;
        for (int bt = 0; bt < nbatch; ++bt) {
          for (int c = 0; c < nch; ++c, ++gc) {
            const uint32_t buf = gc % kItStages;
            if (gc >= kItStages)
              healthy &= tc::mbar_wait_bounded(&bempty[buf], ((gc / kItStages) - 1u) & 1u, kItPolls);
            unsigned char* st = smem + L.b_off + buf * kItStage;
            tc::mbar_arrive_expect_tx(&bfull[buf], 4u * kBoxBytes);
            // x = o.a[2] is a multiple of the innermost tile extent (>= 8 halves: 16 bytes)
            for (int comp = 0; comp < 4; ++comp)
              tc::tma_load_5d(st + comp * kItPart, &tmap, (int)o.a[2], (int)o.a[1], (int)o.a[0] + c * CH, comp,
                              (int)o.inst, &bfull[buf]);
          }
        }
      }
      // the boxes of the last chunks have landed before this CTA can exit
      for (uint32_t k = 1; k <= (uint32_t)kItStages && k <= gc; ++k)
        healthy &= tc::mbar_wait_bounded(&bfull[(gc - k) % kItStages], ((gc - k) / kItStages) & 1u, kItPolls);
    }
    __syncwarp();
  } else if (warp == kItMmaWarp) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sa = tc::smem_u32(smem + L.a_off), sb = tc::smem_u32(smem + L.b_off);
      const uint64_t d_abuf = (uint64_t)((2u * kItAPart) >> 4);  // A buffer 1 = buffer 0 + d_abuf
      const uint64_t d_ah = tc::smem_desc(sa, kItLBO, kItSBOA);
      const uint64_t d_al = tc::smem_desc(sa + kItAPart, kItLBO, kItSBOA);
      const uint64_t d_bh = tc::smem_desc_sw64(sb);
      const uint64_t d_bl = tc::smem_desc_sw64(sb + 2u * kItPart);
      const uint64_t d_buf = (uint64_t)(kItStage >> 4);  // stage k = stage 0 + k d_buf
      const uint32_t idesc = tc::idesc_f16(128, kItN);
      uint32_t gc = 0, gbt = 0;
      for (int it = blockIdx.x; it < num_items; it += G) {
        const int4 item = bins.items[it];
        const int nbatch = (item.z - item.y + kItNodes - 1) / kItNodes;
        for (int bt = 0; bt < nbatch; ++bt, ++gbt) {
          const uint32_t ab = gbt & 1u;
          healthy &= tc::mbar_wait_bounded(&afull[ab], (gbt >> 1) & 1u, kItPolls);
          const uint64_t ao = ab ? d_abuf : 0ull;
          for (int c = 0; c < nch; ++c, ++gc) {
            const uint32_t buf = gc % kItStages, acc = gc % kItAcc;
            healthy &= tc::mbar_wait_bounded(&bfull[buf], (gc / kItStages) & 1u, kItPolls);
            if (gc >= kItAcc) healthy &= tc::mbar_wait_bounded(&tempty[acc], ((gc / kItAcc) - 1u) & 1u, kItPolls);
            tc::fence_after_sync();
            const uint32_t d = tmem + acc * (uint32_t)kItN;
            const uint64_t bo = (uint64_t)buf * d_buf;
#pragma unroll
            for (int ks = 0; ks < kItK / 16; ++ks) {
              const uint64_t ka = (uint64_t)((ks * 2 * kItLBO) >> 4);  // A: two core matrices per k-step
              const uint64_t kb = (uint64_t)((ks * 32) >> 4);          // B: 32 bytes into the swizzled row
              tc::mma_f16(d, d_ah + ao + ka, d_bh + bo + kb, idesc, ks > 0 ? 1u : 0u);
              tc::mma_f16(d, d_ah + ao + ka, d_bl + bo + kb, idesc, 1u);
              tc::mma_f16(d, d_al + ao + ka, d_bh + bo + kb, idesc, 1u);
            }
            tc::mma_commit(&bempty[buf]);
            tc::mma_commit(&tfull[acc]);
          }
        }
      }
      // the last chunk commits are waited by the node warps; the last bempty arrivals here
      for (uint32_t k = 1; k <= (uint32_t)kItStages && k <= gc; ++k)
        healthy &= tc::mbar_wait_bounded(&bempty[(gc - k) % kItStages], ((gc - k) / kItStages) & 1u, kItPolls);
    }
    __syncwarp();
  } else {
    // ======================= node warps: A, then the w0 (x) w1 reduction =======================
    // Three warps per tensor-memory lane quarter.  Per batch, part 0 writes its nodes' w0
    // over the tile's planes (times each plane's inverse scale and 2^-10) and part 1 their
    // w1 over the rows into a per-node weight table, and part 2 builds A of the next
    // batch; per chunk, part h reduces the chunk's planes h, h + 3, ...; parts 1 and 2
    // hand their sums to part 0 through shared memory once per batch.  Records are
    // loaded two batches ahead; A of batch gbt + 1 is built at the start of batch gbt
    // (its buffer's previous batch, gbt - 1, is complete: every part waited for all of
    // its accumulators), so the MMAs never wait for A.
    const int q = warp & 3;             // tensor-memory lane quarter
    const int h = (warp - kItNodeWarp0) >> 2;
    const int slot = 32 * q + lane;     // node slot in the batch = TMEM lane = A row
    float2* red = reinterpret_cast<float2*>(smem + L.red_off);
    const float norm = (float)geo.norm;
    const float mf = (float)geo.m;
    const int64_t P0 = it_split_dims(geo).P0;
    const TapK k0 = tap_k<WIN>(geo, 0), k1 = tap_k<WIN>(geo, 1), k2 = tap_k<WIN>(geo, 2);
    auto build_a = [&](const ItRec& r, uint32_t ab) {
      unsigned char* ah = smem + L.a_off + ab * 2u * kItAPart;
      unsigned char* al = ah + kItAPart;
      const int o2 = (int)(r.off >> (2 * SH));
#pragma unroll
      for (int k8 = 0; k8 < kItK / 8; ++k8) {
        float t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = tc_tap<WIN>(r.fr2, mf, 8 * k8 + u - o2, W, k2) * kItScaleA;
        uint2 h0, l0, h1, l1;
        it_split4_f16(make_float4(t[0], t[1], t[2], t[3]), h0, l0);
        it_split4_f16(make_float4(t[4], t[5], t[6], t[7]), h1, l1);
        const uint32_t oa = (uint32_t)(slot >> 3) * kItSBOA + (uint32_t)k8 * kItLBO + (uint32_t)(slot & 7) * 16u;
        *reinterpret_cast<uint4*>(ah + oa) = make_uint4(h0.x, h0.y, h1.x, h1.y);
        *reinterpret_cast<uint4*>(al + oa) = make_uint4(l0.x, l0.y, l1.x, l1.y);
      }
      tc::fence_proxy_async_smem();
      tc::mbar_arrive_warp(&afull[ab]);
    };
    // part H's share of one chunk: the accumulator's columns of planes H, H + 3, ...
    // (16-column groups gmin .. gmax), every load issued before one wait; the columns
    // are released before the arithmetic
    auto reduce_part = [&](auto HC, uint32_t t0, uint32_t acc, int c, const float* w1x, const float* wt,
                           float& ax, float& ay) {
      constexpr int H = decltype(HC)::value;
      constexpr int LASTPL = H < CH ? H + ((CH - 1 - H) / 3) * 3 : H;
      constexpr int GMIN = (H * E1) / 16, GMAX = H < CH ? (LASTPL * E1 + E1 - 1) / 16 : GMIN;
      constexpr int NG = GMAX - GMIN + 1;
      float vr[NG][16], vi[NG][16];
      if (H < CH) {
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          tc::tmem_ld16(t0 + (uint32_t)((GMIN + g) * 16), vr[g]);                    // real parts
          tc::tmem_ld16(t0 + (uint32_t)kItHalf + (uint32_t)((GMIN + g) * 16), vi[g]);  // imaginary parts
        }
        tc::tmem_ld_wait();
      }
      tc::fence_before_sync();
      tc::mbar_arrive_warp(&tempty[acc]);
      if (H < CH) {
#pragma unroll
        for (int pl = H; pl < CH; pl += 3) {
          float sx = 0.f, sy = 0.f;
#pragma unroll
          for (int p1 = 0; p1 < E1; ++p1) {
            const int col = pl * E1 + p1, g = col / 16 - GMIN, u = col % 16;
            sx = fmaf(w1x[p1], vr[g][u], sx);
            sy = fmaf(w1x[p1], vi[g][u], sy);
          }
          const int p0 = c * CH + pl;
          if (p0 < E0) {
            const float w0 = wt[p0];
            ax = fmaf(w0, sx, ax);
            ay = fmaf(w0, sy, ay);
          }
        }
      }
    };
    ItCursor c0, c1, c2;  // batches gbt, gbt + 1, gbt + 2
    it_cursor_init(c0, bins, num_items);
    c1 = c0;
    it_cursor_step(c1, bins, num_items);
    c2 = c1;
    it_cursor_step(c2, bins, num_items);
    ItRec rc = it_load_rec(c0, num_items, slot, bins), rn = it_load_rec(c1, num_items, slot, bins);
    if (c0.it < num_items && h == 2) build_a(rc, 0u);
    uint32_t gc = 0, gbt = 0;
    float* wt = reinterpret_cast<float*>(smem + L.wt_off) + slot * kItWtStride;  // w0 [0, E0MAX), w1 after
    for (; c0.it < num_items; ++gbt) {
      const ItRec rnn = it_load_rec(c2, num_items, slot, bins);
      // weight table (parts 0 and 1) and the next batch's A (part 2); the previous
      // batch's readers of the table are past its final barrier
      if (h == 0) {
        const TileOrigin to = decode_tile<3>(geo, tl, c0.item.x);
        const float* pinv = plane_inv + to.inst * P0 + to.a[0];  // this tile's plane scales
        const int pmax = (int)(P0 - to.a[0]);  // padded planes from the tile's first; no window reaches past them
        const int o0 = (int)(rc.off & MASK);
#pragma unroll 4
        for (int p = 0; p < E0; ++p)
          wt[p] = p < pmax ? tc_tap<WIN>(rc.fr0, mf, p - o0, W, k0) * (pinv[p] * (1.f / kItScaleA)) : 0.f;
      } else if (h == 1) {
        const int o1 = (int)((rc.off >> SH) & MASK);
#pragma unroll
        for (int p = 0; p < E1; ++p) wt[E0MAX + p] = tc_tap<WIN>(rc.fr1, mf, p - o1, W, k1);
      } else if (c1.it < num_items) {
        build_a(rn, (gbt + 1u) & 1u);
      }
      tc::named_sync(1, kItNodeWarps * 32);
      float w1x[E1];
#pragma unroll
      for (int p = 0; p < E1; ++p) w1x[p] = wt[E0MAX + p];
      float accx = 0.f, accy = 0.f;
#pragma unroll 1
      for (int c = 0; c < nch; ++c) {
        const uint32_t acc = gc % kItAcc;
        healthy &= tc::mbar_wait_warp(&tfull[acc], (gc / kItAcc) & 1u, kItPolls);
        tc::fence_after_sync();
        const uint32_t t0 = tmem + ((uint32_t)(32 * q) << 16) + acc * (uint32_t)kItN;
        if (h == 0) reduce_part(std::integral_constant<int, 0>{}, t0, acc, c, w1x, wt, accx, accy);
        else if (h == 1) reduce_part(std::integral_constant<int, 1>{}, t0, acc, c, w1x, wt, accx, accy);
        else reduce_part(std::integral_constant<int, 2>{}, t0, acc, c, w1x, wt, accx, accy);
        ++gc;
      }
      // parts 1 and 2's sums to part 0 (buffer gbt & 1: part 0 read the other one before
      // this batch's table barrier), which writes the sample
      float2* rb = red + (gbt & 1u) * 256u;
      if (h > 0) rb[(h - 1) * 128 + slot] = make_float2(accx, accy);
      tc::named_sync(1, kItNodeWarps * 32);
      if (h == 0) {
        const float2 o1 = rb[slot], o2 = rb[128 + slot];
        if (rc.idx >= 0) f[rc.idx] = make_float2((accx + o1.x + o2.x) * norm, (accy + o1.y + o2.y) * norm);
      }
      rc = rn;
      rn = rnn;
      c0 = c1;
      c1 = c2;
      it_cursor_step(c2, bins, num_items);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  __syncwarp();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (!healthy) atomicExch(bins.status, 2);
}

}  // namespace cg
