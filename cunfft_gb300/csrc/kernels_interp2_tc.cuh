// kernels_interp2_tc.cuh -- 2D FP32 interpolation on the tensor cores (tcgen05, FP16 hi/lo x 3),
// sub-tiles streamed by TMA.
//
// The reference's 2D forward gridding (kernelConvWithGauss_2d, FGG form
// src/cunfft_kernel.cu:667-712: every node sums its (2m+2)^2 window of the oversampled grid
// with the weights psi_0 psi_1), with the same window-start rule and taps.  The binning
// orders every tile's nodes by sub-tile of 16 x 16 window starts (Tiling::ns sub-bins), and
// a work item is up to kSubItem = 128 nodes of one sub-tile.  For such a batch,
//     f_j = norm sum_{r} w0_j[r - l0_j] H[j, r],
//     H[j, (re|im, r)] = sum_{k} w1_j[k - l1_j] G[r, k] (re|im)
// with r over the sub-tile's 16 + W - 1 <= 31 rows and k over its 16 + W - 1 <= 31 columns
// (l0, l1: the node's window start inside the sub-tile).  H is the product D = A B^T of
//     A[j, k]               = w1_j[k - l1_j]           (128 nodes x K = 32, FP16 hi + lo, x 2^10)
//     B[(re|im, r), k]      = Re|Im G[r, k]            (N = 64 rows: real parts 0..31, imaginary 32..63)
// and the three products hi*hi + hi*lo + lo*hi accumulate in FP32 in tensor memory, node j
// in lane j.  The thread of node j finishes the sum over its W rows from its own lane.
//
// The grid is first split (k_split_rows) into FP16 hi + lo parts of its real and imaginary
// parts, each an array over the periodically padded index range [0, n_t + W - 1) per
// dimension, every padded row scaled by its own power of two 2^(14 - e_r) (2^e_r above its
// largest |Re|, |Im|); the node threads fold the inverse row scales into their w0 weights.
// A sub-tile's B then is four TMA boxes (hi re, hi im, lo re, lo im; 32 halves x (16 + W - 1)
// rows) straight into the 64-byte swizzled K-major layout the MMAs read.
//
// Warp roles: warp 0 lane 0 issues the TMA loads (kI2Stages stages), warp 1 lane 0 the MMAs,
// warps 2-9 are two A sets of four warps on alternate items (A of item li into buffer
// li % kI2ABufs, once the MMAs of item li - kI2ABufs have read it), warps 10-17 two
// reducing sets of four warps on alternate items (the accumulator of item li, one of
// kI2Acc in tensor memory, reduced over each node's rows).  So no warp waits for an MMA
// round trip between its own two jobs: the A sets run up to four items ahead of the MMAs,
// the reducing sets behind them.  Node records are loaded one item ahead.  Hand-offs are
// mbarriers; every wait is bounded, and a wait that gives up raises the CTA's abort flag
// and the plan's device status flag, after which every role leaves its loop at its next
// wait and the kernel drains (bounded), frees its tensor memory and returns.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>

#include "kernels_interp_tc.cuh"
#include "kernels_spread_tc.cuh"

namespace cg {

constexpr int kI2Sub = 16;                    // sub-tile extent of window starts per dimension
constexpr int kI2K = 32;                      // K: a sub-tile's 16 + W - 1 <= 31 columns, padded (one 64-byte row)
constexpr int kI2Rows = 32;                   // B rows per part: a sub-tile's 16 + W - 1 <= 31 rows, padded
constexpr int kI2N = 2 * kI2Rows;             // MMA N: real parts 0..31, imaginary parts 32..63
constexpr int kI2Sets = 2;                    // A-building sets and reducing sets, each on alternate items
constexpr int kI2AWarp0 = 2;                  // warps 2-9: two A sets of four warps
constexpr int kI2RWarp0 = kI2AWarp0 + 4 * kI2Sets;  // warps 10-17: two reducing sets of four warps
constexpr int kI2Threads = (kI2RWarp0 + 4 * kI2Sets) * 32;
constexpr int kI2ABufs = 4;                   // A buffers (item li uses li % 4)
constexpr int kI2Stages = 8;                  // B stages (TMA ring)
constexpr int kI2Acc = 8;                     // tensor-memory accumulators of kI2N columns (512 in all)
constexpr uint32_t kI2Part = kI2Rows * 64u;   // one B part (hi re, hi im, lo re, lo im): 32 rows x 64 bytes
constexpr uint32_t kI2Stage = 4u * kI2Part;   // B hi = parts 0-1, B lo = parts 2-3
constexpr uint32_t kI2Polls = 1u << 20;       // mbarrier polls (<= 1 us each) before giving up

// 2D, 2m+2 in [4, 16], inner tile extent >= 16 (16-column sub-tiles whose TMA boxes start on
// 32-byte boundaries) and a row length divisible by 8 (16-byte rows of the split arrays; the
// split's quads never straddle the row's wrap)
__host__ __device__ constexpr bool interp2_tc_ok(int d, int W, int T1, int64_t n1) {
  return d == 2 && W >= 4 && W <= 16 && T1 >= kI2Sub && n1 >= 8 && n1 % 8 == 0;
}

// Shared-memory layout (byte offsets from a 1024-byte aligned base; host and device agree).
struct I2Layout {
  uint32_t b_off;      // kI2Stages B stages of kI2Stage
  uint32_t a_off;      // kI2ABufs A buffers x (A hi, A lo)
  uint32_t bar_off;    // afull[4], aempty[4], bfull[8], bempty[8], tfull[8], tempty[8]; tensor-memory base; abort flag
  uint32_t total;      // bytes past the aligned base
  uint32_t dyn;        // dynamic shared memory to request (alignment slack included)
};

__host__ __device__ constexpr I2Layout i2_layout() {
  return I2Layout{0u,
                  kI2Stages * kI2Stage,
                  kI2Stages * kI2Stage + (uint32_t)kI2ABufs * 2u * kItAPart,
                  kI2Stages * kI2Stage + (uint32_t)kI2ABufs * 2u * kItAPart + 512u,
                  kI2Stages * kI2Stage + (uint32_t)kI2ABufs * 2u * kItAPart + 512u + 1024u};
}

// Two Gaussian taps at integer offsets l and l + 1 of a node's window (fraction fr, cut-off
// mf = m), times 2^s: packed FP32x2 arithmetic for the exponents, one ex2 each, zero
// outside [0, W).  The same values as tc_tap<kWinGauss> times 2^s up to the last bits of ex2.
__device__ __forceinline__ float2 tap2_gauss(float fr, float mf, int l, int W, TapK k, float s) {
  const float c = fr + mf;
  const float2 y = __fadd2_rn(make_float2(c, c), make_float2(-(float)l, -(float)(l + 1)));
  const float2 e = __ffma2_rn(__fmul2_rn(y, y), make_float2(-k.a, -k.a), make_float2(s, s));
  return make_float2((unsigned)l < (unsigned)W ? tap_exp2(e.x) : 0.f, (unsigned)(l + 1) < (unsigned)W ? tap_exp2(e.y) : 0.f);
}
// the same for either window (the ES window takes the scalar form)
template <int WIN>
__device__ __forceinline__ float2 tap2(float fr, float mf, int l, int W, TapK k, float s, float scale) {
  if (WIN == kWinGauss) return tap2_gauss(fr, mf, l, W, k, s);
  return make_float2(tc_tap<WIN>(fr, mf, l, W, k) * scale, tc_tap<WIN>(fr, mf, l + 1, W, k) * scale);
}

// Padded split rows of a 2D grid, in the 3D split layout with one row per plane: half
// [batch][4][P0][P2s] with P0 = n0 + W - 1 padded rows, P1 = 1, P2 = n1 + W - 1 padded
// columns and P2s its multiple of 8.  Row scales: float [batch][P0], the inverse
// 2^(e - 14) of each padded row.
__host__ __device__ inline ItSplit i2_split_dims(const Geom& g) {
  ItSplit s;
  s.P0 = g.n[0] + g.W - 1;
  s.P1 = 1;
  s.P2 = g.n[1] + g.W - 1;
  s.P2s = (s.P2 + 7) / 8 * 8;
  return s;
}

constexpr int kI2SplitThreads = 256;

// The grid's padded FP16 hi/lo rows in one pass: warp w takes padded rows (instance, i0)
// w, w + nwarps, ...: it reads grid row i0 mod n0 once for its largest |Re|, |Im| (a warp
// reduction) and again (from L1: a row is n1 complex values) to write the row's P2s / 4
// quads of FP16 hi + lo parts of the real and imaginary parts, scaled by the row's
// 2^(14 - e), and the row's inverse scale.  A quad never straddles the row's wrap
// (n1 % 8 == 0).
static __global__ void __launch_bounds__(kI2SplitThreads) k_split_rows(const float2* __restrict__ g,
                                                                 __half* __restrict__ out,
                                                                 float* __restrict__ inv_scale, Geom geo, ItSplit sd) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t n0 = geo.n[0], n1 = geo.n[1], q4 = sd.P2s / 4, comp = sd.P0 * sd.P2s;
  const bool al16 = (reinterpret_cast<uintptr_t>(g) & 15u) == 0;  // n1 is a multiple of 8
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < sd.P0 * geo.batch; r += nwarps) {
    const int64_t inst = r / sd.P0, i0 = r - inst * sd.P0;
    const float2* src = g + (inst * n0 + wrap_up(i0, n0)) * n1;
    float mx = 0.f;
    for (int64_t e = lane; e < n1 / 4; e += 32) {
      float4 a, b;
      ld_quad(src + 4 * e, al16, a, b);
      mx = fmaxf(mx, fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(a.w))),
                           fmaxf(fmaxf(fabsf(b.x), fabsf(b.y)), fmaxf(fabsf(b.z), fabsf(b.w)))));
    }
    const uint32_t m = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
    const int ex = it_plane_exp(__uint_as_float(m));
    const float scale = ldexpf(1.f, kItLogB - ex);
    if (lane == 0) inv_scale[inst * sd.P0 + i0] = ldexpf(1.f, ex - kItLogB);
    __half* const o_row = out + inst * 4 * comp + i0 * sd.P2s;
    for (int64_t e = lane; e < q4; e += 32) {
      const int64_t i1 = 4 * e;
      float4 a, b;
      ld_quad(src + wrap_up(i1, n1), al16, a, b);
      __half* o = o_row + i1;
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

// Sub-tile of an interpolation item: its tile's origin and instance, and the sub-tile's
// first row and column (tile origin + sub-tile offset).
struct I2Sub {
  TileOrigin o;
  int r0, c0;   // grid row and column of the sub-tile's first window start
  int s0, s1;   // sub-tile offsets inside the tile (rows, columns)
};
__device__ __forceinline__ I2Sub i2_decode(const Geom& geo, const Tiling& tl, int key) {
  I2Sub u;
  const int tile = key / tl.ns, sub = key - tile * tl.ns;
  u.o = decode_tile<2>(geo, tl, tile);
  const int sb0 = sub / tl.snb1, sb1 = sub - sb0 * tl.snb1;
  u.s0 = sb0 << tl.ssh[0];
  u.s1 = sb1 << tl.ssh[1];
  u.r0 = (int)u.o.a[0] + u.s0;
  u.c0 = (int)u.o.a[1] + u.s1;
  return u;
}

template <int W, int WIN>
__global__ void __launch_bounds__(kI2Threads, 1) k_interp2_tc(const __grid_constant__ CUtensorMap tmap,
                                                              const float* __restrict__ row_inv,
                                                              float2* __restrict__ f, Geom geo, Tiling tl, Bins bins) {
  constexpr int SH = off_bits(2);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  static_assert(kI2Sub + W - 1 <= kI2K, "a sub-tile's columns must fit K");
  static_assert(kI2Sub + W - 1 <= kI2Rows, "a sub-tile's rows must fit one B part");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const I2Layout L = i2_layout();
  uint64_t* afull = reinterpret_cast<uint64_t*>(smem + L.bar_off);  // [4] A of the buffer's item built
  uint64_t* aempty = afull + kI2ABufs;                               // [4] MMAs of the buffer's item complete
  uint64_t* bfull = aempty + kI2ABufs;                               // [8] sub-tile landed (TMA)
  uint64_t* bempty = bfull + kI2Stages;                              // [8] MMAs of the stage complete
  uint64_t* tfull = bempty + kI2Stages;                              // [8] accumulator complete
  uint64_t* tempty = tfull + kI2Acc;                                 // [8] accumulator read out
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + kI2Acc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int num_items = *bins.num_iitems;
  const int G = (int)gridDim.x;
  // B rows of a sub-tile: the windows of 16 rows of window starts (16 + W - 1 <= 31); a
  // sub-tile of fewer rows (tiles of fewer than 16 rows) loads real grid rows past its own,
  // so that every B row the reduction weights is finite
  constexpr int kRows = kI2Sub + W - 1;

  if (tid == 0) {
    for (int i = 0; i < kI2ABufs; ++i) {
      tc::mbar_init(&afull[i], 4);    // one arrival per warp of the A set
      tc::mbar_init(&aempty[i], 1);
    }
    for (int i = 0; i < kI2Stages; ++i) {
      tc::mbar_init(&bfull[i], 1);    // the TMA thread's arrival (+ the boxes' bytes)
      tc::mbar_init(&bempty[i], 1);
    }
    for (int i = 0; i < kI2Acc; ++i) {
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], 4);   // one arrival per warp of the reducing set
    }
    *abort_flag = 0;
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

  // Item li of this CTA (li = 0, 1, ...) is bins.iitems[blockIdx.x + li G]; it uses B
  // stage li % kI2Stages in its cycle li / kI2Stages, accumulator li % kI2Acc in its cycle
  // li / kI2Acc, and A buffer li % kI2ABufs in its cycle li / kI2ABufs; A set and reducing
  // set li % kI2Sets.
  if (warp == 0) {
    // ======================= TMA: sub-tiles =======================
    if (lane == 0) {
      const uint32_t box = (uint32_t)(kI2K * 2 * kRows);
      uint32_t li = 0;
      for (int it = blockIdx.x; it < num_items; it += G, ++li) {
        const int4 item = bins.iitems[it];
        const I2Sub u = i2_decode(geo, tl, item.x);
        const uint32_t st = li % kI2Stages;
        if (li >= (uint32_t)kI2Stages && !tc::mbar_wait_bounded(&bempty[st], ((li / kI2Stages) - 1u) & 1u, kI2Polls))
          healthy = false;
        if (!healthy || *abort_flag != 0) {
          healthy = false;
          break;
        }
        unsigned char* dst = smem + L.b_off + st * kI2Stage;
        tc::mbar_arrive_expect_tx(&bfull[st], 4u * box);
        // x = c0 is a multiple of 16 halves (tile and sub-tile origins): 32-byte aligned
        for (int comp = 0; comp < 4; ++comp)
          tc::tma_load_5d(dst + comp * kI2Part, &tmap, u.c0, u.r0, 0, comp, (int)u.o.inst, &bfull[st]);
      }
      // the boxes in flight have landed before this CTA can exit
      for (uint32_t k = 1; k <= (uint32_t)kI2Stages && k <= li; ++k)
        healthy &= tc::mbar_wait_bounded(&bfull[(li - k) % kI2Stages], ((li - k) / kI2Stages) & 1u, kI2Polls);
      if (!healthy) *abort_flag = 1;
    }
    __syncwarp();
  } else if (warp == 1) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sa = tc::smem_u32(smem + L.a_off), sb = tc::smem_u32(smem + L.b_off);
      const uint32_t idesc = tc::idesc_f16(128, kI2N);
      uint32_t li = 0;
      for (int it = blockIdx.x; it < num_items; it += G, ++li) {
        const uint32_t ab = li % kI2ABufs, st = li % kI2Stages, acc = li % kI2Acc;
        bool ok = tc::mbar_wait_bounded(&afull[ab], (li / kI2ABufs) & 1u, kI2Polls);
        ok = ok && tc::mbar_wait_bounded(&bfull[st], (li / kI2Stages) & 1u, kI2Polls);
        if (ok && li >= (uint32_t)kI2Acc) ok = tc::mbar_wait_bounded(&tempty[acc], ((li / kI2Acc) - 1u) & 1u, kI2Polls);
        if (!ok || *abort_flag != 0) {
          healthy = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t d = tmem + acc * (uint32_t)kI2N;
        const uint64_t d_ah = tc::smem_desc(sa + ab * 2u * kItAPart, kItLBO, kItSBOA);
        const uint64_t d_al = tc::smem_desc(sa + ab * 2u * kItAPart + kItAPart, kItLBO, kItSBOA);
        const uint64_t d_bh = tc::smem_desc_sw64(sb + st * kI2Stage);
        const uint64_t d_bl = tc::smem_desc_sw64(sb + st * kI2Stage + 2u * kI2Part);
#pragma unroll
        for (int ks = 0; ks < kI2K / 16; ++ks) {
          const uint64_t ka = (uint64_t)((ks * 2 * kItLBO) >> 4);  // A: two core matrices per k-step
          const uint64_t kb = (uint64_t)((ks * 32) >> 4);          // B: 32 bytes into the swizzled row
          tc::mma_f16(d, d_ah + ka, d_bh + kb, idesc, ks > 0 ? 1u : 0u);
          tc::mma_f16(d, d_ah + ka, d_bl + kb, idesc, 1u);
          tc::mma_f16(d, d_al + ka, d_bh + kb, idesc, 1u);
        }
        tc::mma_commit(&bempty[st]);
        tc::mma_commit(&aempty[ab]);
        tc::mma_commit(&tfull[acc]);
      }
      // the last commits of each stage: no arrival may land after exit (the commits of one
      // item complete together, so its bempty covers its aempty and tfull)
      for (uint32_t k = 1; k <= (uint32_t)kI2Stages && k <= li; ++k)
        healthy &= tc::mbar_wait_bounded(&bempty[(li - k) % kI2Stages], ((li - k) / kI2Stages) & 1u, kI2Polls);
      if (!healthy) *abort_flag = 1;
    }
    __syncwarp();
  } else if (warp < kI2RWarp0) {
    // ======================= A sets: w1 over the sub-tile's 32 columns =======================
    // Set `set` takes the CTA's items set, set + 2, ...; warp (lane quarter q) builds the A
    // rows of nodes 32 q .. 32 q + 31 (slot = A row).  A quarter past the item's last node
    // skips its arithmetic but takes part in every hand-off.
    const int set = (warp - kI2AWarp0) >> 2, q = warp & 3, slot = 32 * q + lane;
    const float mf = (float)geo.m;
    const TapK k1 = tap_k<WIN>(geo, 1);
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    uint32_t li = (uint32_t)set;
    int it = blockIdx.x + set * G;
    // records of the next item, loaded one item ahead
    int4 nitem = it < num_items ? bins.iitems[it] : make_int4(0, 0, 1, 0);
    uint32_t noff = 0;
    float nfr = 0.f;
    if (it < num_items && slot < nitem.z - nitem.y) {
      noff = (uint32_t)bins.soff[nitem.y + slot];
      nfr = sfrac[(int64_t)(nitem.y + slot) * 2 + 1];
    }
    for (; it < num_items; it += kI2Sets * G, li += kI2Sets) {
      const int4 cur = nitem;
      const uint32_t off = noff;
      const float fr1 = nfr;
      const int itn = it + kI2Sets * G;
      if (itn < num_items) {
        nitem = bins.iitems[itn];
        if (slot < nitem.z - nitem.y) {
          noff = (uint32_t)bins.soff[nitem.y + slot];
          nfr = sfrac[(int64_t)(nitem.y + slot) * 2 + 1];
        }
      }
      const int n = cur.z - cur.y;
      const bool on = n > 32 * q;  // warp-uniform
      const uint32_t ab = li % kI2ABufs;
      if (li >= (uint32_t)kI2ABufs) {  // the MMAs of item li - kI2ABufs have read the buffer
        const bool ok = tc::mbar_wait_warp(&aempty[ab], ((li / kI2ABufs) - 1u) & 1u, kI2Polls);
        if (__any_sync(0xffffffffu, !ok || *abort_flag != 0)) {  // the whole warp leaves together
          healthy = false;
          break;
        }
      } else if (__any_sync(0xffffffffu, *abort_flag != 0)) {
        healthy = false;
        break;
      }
      if (on) {
        const int s1 = (int)(i2_decode(geo, tl, cur.x).s1);
        const int l1 = slot < n ? (int)((off >> SH) & MASK) - s1 : 1 << 20;  // no node: every tap zero
        unsigned char* const ah = smem + L.a_off + ab * 2u * kItAPart;
        unsigned char* const al = ah + kItAPart;
#pragma unroll
        for (int k8 = 0; k8 < kI2K / 8; ++k8) {
          uint32_t hi[4], lo[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int k = 8 * k8 + 2 * v;
            const float2 t = k < kI2Sub + W - 1 ? tap2<WIN>(fr1, mf, k - l1, W, k1, 10.f, kItScaleA)
                                                : make_float2(0.f, 0.f);
            tc_split2_f16(t, hi[v], lo[v]);
          }
          const uint32_t oa = (uint32_t)(slot >> 3) * kItSBOA + (uint32_t)k8 * kItLBO + (uint32_t)(slot & 7) * 16u;
          *reinterpret_cast<uint4*>(ah + oa) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
          *reinterpret_cast<uint4*>(al + oa) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
      }
      tc::fence_proxy_async_smem();
      tc::mbar_arrive_warp(&afull[ab]);
    }
    if (!healthy) *abort_flag = 1;
  } else {
    // ======================= reducing sets: the accumulators =======================
    // Set `set` takes the CTA's items set, set + 2, ...; warp (lane quarter q) reduces TMEM
    // lanes 32 q .. 32 q + 31: node slot 32 q + lane sums its W rows of the accumulator with
    // its w0 weights and the rows' inverse scales.
    const int set = (warp - kI2RWarp0) >> 2, q = warp & 3, slot = 32 * q + lane;
    const float mf = (float)geo.m;
    const float norm = (float)geo.norm * (1.f / kItScaleA);
    const int64_t P0 = i2_split_dims(geo).P0;
    const TapK k0 = tap_k<WIN>(geo, 0);
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    uint32_t li = (uint32_t)set;
    int it = blockIdx.x + set * G;
    int4 nitem = it < num_items ? bins.iitems[it] : make_int4(0, 0, 1, 0);
    uint32_t noff = 0;
    float nfr = 0.f;
    int nidx = -1;
    if (it < num_items && slot < nitem.z - nitem.y) {
      noff = (uint32_t)bins.soff[nitem.y + slot];
      nfr = sfrac[(int64_t)(nitem.y + slot) * 2];
      nidx = bins.sidx[nitem.y + slot];
    }
    for (; it < num_items; it += kI2Sets * G, li += kI2Sets) {
      const int4 cur = nitem;
      const uint32_t off = noff;
      const float fr0 = nfr;
      const int idx = nidx;
      const int itn = it + kI2Sets * G;
      if (itn < num_items) {
        nitem = bins.iitems[itn];
        nidx = -1;
        if (slot < nitem.z - nitem.y) {
          noff = (uint32_t)bins.soff[nitem.y + slot];
          nfr = sfrac[(int64_t)(nitem.y + slot) * 2];
          nidx = bins.sidx[nitem.y + slot];
        }
      }
      const int n = cur.z - cur.y;
      const bool on = n > 32 * q;  // warp-uniform
      const I2Sub u = i2_decode(geo, tl, cur.x);
      // the sub-tile's row scales: lane r holds row r's (rows past the padded range: 0)
      const float rs = lane < kRows && u.r0 + lane < P0 ? __ldg(row_inv + u.o.inst * P0 + u.r0 + lane) : 0.f;
      const int l0 = slot < n ? (int)(off & MASK) - u.s0 : 1 << 20;
      const uint32_t acc = li % kI2Acc;
      const bool ok = tc::mbar_wait_warp(&tfull[acc], (li / kI2Acc) & 1u, kI2Polls);
      if (__any_sync(0xffffffffu, !ok || *abort_flag != 0)) {  // the whole warp leaves together
        healthy = false;
        break;
      }
      tc::fence_after_sync();
      float2 fs = make_float2(0.f, 0.f);
      if (on) {
        const uint32_t t0 = tmem + ((uint32_t)(32 * q) << 16) + acc * (uint32_t)kI2N;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (16 * h < kRows) {
            float vr[16], vi[16];
            tc::tmem_ld16(t0 + (uint32_t)(16 * h), vr);
            tc::tmem_ld16(t0 + (uint32_t)(kI2Rows + 16 * h), vi);
            tc::tmem_ld_wait();
#pragma unroll
            for (int c = 0; c < 16; c += 2) {
              const int r = 16 * h + c;
              if (r < kRows) {  // rows past kRows hold stale shared memory: never touched
                const float2 w = tap2<WIN>(fr0, mf, r - l0, W, k0, 0.f, 1.f);
                const float w0 = w.x * __shfl_sync(0xffffffffu, rs, r);
                fs = __ffma2_rn(make_float2(w0, w0), make_float2(vr[c], vi[c]), fs);
                if (r + 1 < kRows) {
                  const float w1 = w.y * __shfl_sync(0xffffffffu, rs, r + 1);
                  fs = __ffma2_rn(make_float2(w1, w1), make_float2(vr[c + 1], vi[c + 1]), fs);
                }
              }
            }
          }
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive_warp(&tempty[acc]);
      if (idx >= 0) f[idx] = make_float2(fs.x * norm, fs.y * norm);
    }
    if (!healthy) *abort_flag = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (!healthy) atomicExch(bins.status, 2);
}

}  // namespace cg
