// kernels_spread_tc.cuh -- 3D FP32 spreading on the tensor cores (tcgen05, 3 x FP16).
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
// Warp roles: 15 builder warps and one MMA warp.  Per batch of kTcK = 16 nodes the
// builders (1) evaluate w0 and w1 over the padded planes/rows and build B, then,
// after one named barrier among themselves, (2) build A; operands are split into
// FP16 hi + lo parts (hi = fp16(v), lo = fp16(v - hi): 11 + 11 significant bits,
// the precision of a TF32 hi + lo split), and the thread mappings write 128
// contiguous bytes per 8-lane store phase (no bank conflicts).  FP16's range is
// kept by powers of two: A (weights in [0, 1]) is scaled by 2^10, B by 2^(14 - e)
// where 2^e bounds |w2 f norm| over the call's samples (their largest |Re|, |Im|,
// found by k_permute_samples), and the epilogue scales the sums back exactly.
// Each builder thread then arrives on the stage's `full` mbarrier; lane 0 of the
// MMA warp waits on it and issues, per M-tile, the three kind::f16 MMAs (K = 16
// nodes) hi*hi + hi*lo + lo*hi with FP32 accumulation (error ~2^-22 relative per
// product), then commits them to the stage's `empty` mbarrier.  Operands have 3 stages where
// shared memory allows, else 2 (builders wait on `empty` before reusing a stage);
// node records are loaded two batches ahead and staged one batch ahead.
// At the end of a work item the accumulators go TMEM -> registers -> a shared-
// memory tile (aliasing the operand buffers) and are added to the global grid
// by the 16-byte-atomic flush shared with the other spreading kernels.
//
// Every mbarrier wait is bounded; a wait that gives up sets the plan's device
// status flag, the kernel still drains (bounded), frees its tensor memory and
// returns.  Tensor-memory allocation cannot contend: the launcher sizes shared
// memory so that the CTAs resident on one SM never ask for more than 512 columns.
#pragma once

#include <cuda_fp16.h>

#include "kernels_grid.cuh"
#include "tc_sm100.cuh"

namespace cg {

constexpr int kTcMaxT0 = 16;     // outer tile extent limit (E0 <= 31 planes)
constexpr int kTcK = 16;         // nodes per staged batch: one FP16 MMA k-step of 16
constexpr int kTcBuilders = 15;                  // warps that build operands
constexpr int kTcMmaWarp = kTcBuilders;           // lane 0 issues the MMAs
constexpr int kTcEpiWarp0 = kTcBuilders + 1;      // 4 epilogue warps: TMEM lane quarters 0..3
constexpr int kTcThreads = (kTcBuilders + 1 + 4) * 32;
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcN = 64;         // MMA N: 2 E2 <= 62 columns (p2, re/im), padded
constexpr int kTcWxStride = 20;  // floats per expanded-weight row: 8 consecutive rows hit distinct banks
constexpr int kTcWbStride = 24;  // floats per B-table row: rows two apart start 16 banks apart
// Node records stream into a ring of kTcRing slots, kTcAhead batches ahead of use.
// A slot holds [kTcK] packed window starts (int), [kTcK][3] fractions (float) and
// [kTcK] samples (float2, in sorted order); unused node slots hold a window start
// of all ones (no plane, row or column inside the tile) and zeros.
constexpr int kTcRing = 4;
constexpr int kTcAhead = kTcRing - 1;
constexpr uint32_t kTcSlotOff = 0, kTcSlotFrac = kTcK * 4, kTcSlotVal = kTcK * 16, kTcSlotBytes = kTcK * 24;
constexpr uint32_t kTcLBO = 128;                // core matrices (8 rows x 8 FP16) along K
constexpr uint32_t kTcSBO = (kTcK / 8) * 128;   // 8-row groups
constexpr float kTcScaleA = 1024.f;             // A = w0 w1 in [0, 1] -> [0, 2^10]
constexpr int kTcLogB = 14;                     // |B| scaled to below 2^14
constexpr uint32_t kTcPolls = 1u << 20;         // mbarrier polls (<= 1 us each) before giving up

__host__ __device__ constexpr bool spread_tc_ok(int d, int W, int T0) {
  return d == 3 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kTcMaxT0;
}

// Shared-memory layout of k_spread_tc (byte offsets; host and device agree).
struct TcLayout {
  int mt;                 // M-tiles of 128 rows covering E0 E1 rows
  uint32_t a_bytes;       // one A part (hi or lo) of one stage
  uint32_t stage_bytes;   // A hi, A lo, B hi, B lo
  int ns;                 // operand stages: 3 where they fit in shared memory, else 2
  uint32_t rec_off;       // kTcRing record slots of kTcSlotBytes
  uint32_t wx_off;        // 2 x ([E0][kTcWxStride] w0 over planes, [E1][kTcWxStride] w1 over rows)
  uint32_t wx_stage;      // bytes of one expanded-weight buffer
  uint32_t wb_off;        // 2 x [kTcN][kTcWbStride] B values w2 f (rows (p2, re|im), 16 nodes), FP32
  uint32_t wb_stage;      // bytes of one B-table buffer
  uint32_t bar_off;       // mbarriers full[3], empty[3], acc_full[2], acc_empty[2]; tensor-memory base
  uint32_t total;
  int nacc;               // accumulator buffers in tensor memory (2 when they fit in 512 columns)
  uint32_t tmem_cols;     // power of two >= 32
};

__host__ __device__ inline TcLayout tc_layout(int W, int E0) {
  TcLayout L{};
  const int E1 = fixed_t_mid(3, W) + W - 1;
  const int rows = E0 * E1;
  L.mt = (rows + 127) / 128;
  L.a_bytes = (uint32_t)L.mt * 128u * kTcK * 2u;
  const uint32_t b_bytes = kTcN * kTcK * 2u;
  L.stage_bytes = 2u * L.a_bytes + 2u * b_bytes;
  for (L.ns = 3; L.ns >= 2; --L.ns) {  // 3 operand stages when they fit in 227 KB
    const uint32_t ops = ((uint32_t)L.ns * L.stage_bytes + 1023u) & ~1023u;
    L.rec_off = ops;
    L.wx_off = L.rec_off + kTcRing * kTcSlotBytes;
    L.wx_stage = (uint32_t)(E0 + E1) * kTcWxStride * 4u;
    L.wb_off = (L.wx_off + 2u * L.wx_stage + 15u) & ~15u;
    L.wb_stage = (uint32_t)kTcN * kTcWbStride * 4u;
    L.bar_off = L.wb_off + 2u * L.wb_stage;
    L.total = L.bar_off + 96u;
    if (L.total <= 227u * 1024u) break;
  }
  L.nacc = 2u * (uint32_t)L.mt * kTcN <= 512u ? 2 : 1;
  uint32_t c = 32;
  while (c < (uint32_t)(L.nacc * L.mt * kTcN)) c <<= 1;
  L.tmem_cols = c;
  return L;
}

// byte offset of the 8 FP16 values (row 8 rg + ri, nodes 8 kg .. 8 kg + 7) in a K-major
// no-swizzle operand
__device__ __forceinline__ uint32_t tc_elem_off(int rg, int ri, int kg) {
  return (uint32_t)rg * kTcSBO + (uint32_t)kg * kTcLBO + (uint32_t)ri * 16u;
}

// 8 FP32 values -> FP16 hi (8 halves) and lo = fp16(v - hi) (8 halves)
__device__ __forceinline__ void tc_split8_f16(const float* v, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __half2 hh = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
    const float2 hf = __half22float2(hh);
    const __half2 ll = __floats2half2_rn(v[2 * i] - hf.x, v[2 * i + 1] - hf.y);
    h[i] = *reinterpret_cast<const uint32_t*>(&hh);
    l[i] = *reinterpret_cast<const uint32_t*>(&ll);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// 2 FP32 values -> FP16 hi pair and lo = fp16(v - hi) pair (the subtraction as one
// packed FP32 add)
__device__ __forceinline__ void tc_split2_f16(float2 v, uint32_t& hi, uint32_t& lo) {
  const __half2 hh = __float22half2_rn(v);
  const float2 hf = __half22float2(hh);
  const __half2 ll = __float22half2_rn(__fadd2_rn(v, make_float2(-hf.x, -hf.y)));
  hi = *reinterpret_cast<const uint32_t*>(&hh);
  lo = *reinterpret_cast<const uint32_t*>(&ll);
}

// 4 FP32 values -> FP16 hi (4 halves) and lo = fp16(v - hi) (4 halves)
__device__ __forceinline__ void tc_split4_f16(const float* v, uint2& hi, uint2& lo) {
  uint32_t h[2], l[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const __half2 hh = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
    const float2 hf = __half22float2(hh);
    const __half2 ll = __floats2half2_rn(v[2 * i] - hf.x, v[2 * i + 1] - hf.y);
    h[i] = *reinterpret_cast<const uint32_t*>(&hh);
    l[i] = *reinterpret_cast<const uint32_t*>(&ll);
  }
  hi = make_uint2(h[0], h[1]);
  lo = make_uint2(l[0], l[1]);
}

// 2^(kTcLogB - e), 2^e >= the call's largest |w2 f norm| (w2 <= 1): the B scale
__device__ __forceinline__ float tc_scale_b(const Bins& bins, float norm) {
  int e = 0;
  frexpf(__uint_as_float(*bins.fmax) * norm, &e);
  return ldexpf(1.f, kTcLogB - e);
}


// Position in this CTA's batch sequence: work items c, c + G, c + 2G, ... (CTA c,
// G CTAs; items are never empty) and the batch of kTcK nodes within the item.
// The descriptor of the following item is loaded one item ahead.
struct TcCursor {
  int it;       // item index (>= num_items: past the end)
  int b;        // batch within the item
  int4 item;    // (tile, first node, end node, -)
  int4 next;    // item it + G
};

__device__ __forceinline__ void tc_cursor_init(TcCursor& c, const Bins& bins, int num_items) {
  const int G = (int)gridDim.x;
  c.it = (int)blockIdx.x;
  c.b = 0;
  c.item = c.it < num_items ? bins.items[c.it] : make_int4(0, 0, 0, 0);
  c.next = c.it + G < num_items ? bins.items[c.it + G] : make_int4(0, 0, 0, 0);
}

__device__ __forceinline__ void tc_cursor_step(TcCursor& c, const Bins& bins, int num_items) {
  const int G = (int)gridDim.x;
  if (c.item.y + (++c.b) * kTcK < c.item.z) return;
  c.it += G;
  c.b = 0;
  c.item = c.next;
  c.next = c.it + G < num_items ? bins.items[c.it + G] : make_int4(0, 0, 0, 0);
}

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int W, int WIN>
__global__ void __launch_bounds__(kTcThreads, 1) k_spread_tc(const float2* __restrict__ f, float2* __restrict__ g,
                                                             Geom geo, Tiling tl, Bins bins) {
  constexpr int T1 = fixed_t_mid(3, W), T2 = fixed_t_last(3, W);
  constexpr int E1 = T1 + W - 1, E2 = T2 + W - 1;
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr int kBuildThreads = kTcBuilders * 32;
  constexpr int kBWarps = kTcN / 8;                             // builders of B: one 8-row group each
  constexpr int kExpWarps = kTcBuilders - kBWarps;              // builders expanding w0 / w1
  // A tasks: (node group kg, row p1) pairs times planes p0; builder thread t takes pair
  // t % kAPairs and planes t / kAPairs + kAStride i, so its w1 values load once per batch
  constexpr int kAPairs = 2 * E1;
  constexpr int kAStride = kBuildThreads / kAPairs;
  constexpr int kAMaxP = (kTcMaxT0 + W - 1 + kAStride - 1) / kAStride;  // planes per thread at the largest E0
  static_assert(kAStride >= 1, "every (node group, row) pair needs a builder thread");
  static_assert(2 * E2 <= kTcN, "complex columns must fit the MMA N");
  static_assert(kExpWarps >= 1 && kTcK == 16, "staging roles assume 16 nodes and 8 B-row warps");
  extern __shared__ __align__(16) unsigned char smem[];
  const int E0 = tl.E[0];
  const TcLayout L = tc_layout(W, E0);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bar_off);    // [ns] operands of stage s built
  uint64_t* empty = full + 3;                                         // [ns] MMAs of stage s complete
  uint64_t* acc_full = full + 6;                                      // [2] accumulator a complete
  uint64_t* acc_empty = full + 8;                                     // [2] accumulator a read out
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 80);
  const uint32_t ns = (uint32_t)L.ns;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rows = E0 * E1;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  if (tid == 0) {
    for (uint32_t i = 0; i < ns; ++i) {
      tc::mbar_init(&full[i], kBuildThreads);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(&acc_full[0], 1);
    tc::mbar_init(&acc_full[1], 1);
    tc::mbar_init(&acc_empty[0], 128);
    tc::mbar_init(&acc_empty[1], 128);
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
  bool healthy = true;

  // Work items are taken round-robin (CTA c: items c, c + G, ...), so every role
  // walks the same sequence without a CTA-wide barrier.  Batches are numbered
  // across items (gb); batch gb uses operand stage gb % ns in its cycle gb / ns
  // (the phase index of that stage's barriers), and record / expanded-weight
  // buffer gb & 1.
  if (warp < kTcBuilders) {
    // ======================= builder warps =======================
    const int ri = lane & 7;  // B build: row in group
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    const float2* fperm = reinterpret_cast<const float2*>(bins.fperm);
    const float norm = (float)geo.norm;
    const float bscale = norm * tc_scale_b(bins, norm);  // w2 f -> B
    const int apair = tid % kAPairs, ablk = tid / kAPairs;  // A task: pair and first plane
    const int akg = apair / E1, ap1 = apair - akg * E1;
    const bool a_on = ablk < kAStride;
    const float mf = (float)geo.m;
    const TapK k0 = tap_k<WIN>(geo, 0), k1 = tap_k<WIN>(geo, 1), k2 = tap_k<WIN>(geo, 2);
    // loads of one batch's records into ring slot `slot` (threads < 4 kTcK): thread
    // j < kTcK the window start and sample of node j, thread kTcK + i fraction i
    auto load = [&](const TcCursor& c, int slot) {
      unsigned char* sl = smem + L.rec_off + slot * kTcSlotBytes;
      const int base = c.item.y + c.b * kTcK, n = min(kTcK, c.item.z - base);
      if (tid < kTcK) {
        if (tid < n) {
          cp_async4(sl + kTcSlotOff + tid * 4, bins.soff + base + tid);
          cp_async8(sl + kTcSlotVal + tid * 8, fperm + base + tid);
        } else {
          reinterpret_cast<int*>(sl + kTcSlotOff)[tid] = -1;
          reinterpret_cast<float2*>(sl + kTcSlotVal)[tid] = make_float2(0.f, 0.f);
        }
      } else if (tid < 4 * kTcK) {
        const int i = tid - kTcK;
        if (i < 3 * n) cp_async4(sl + kTcSlotFrac + i * 4, sfrac + (int64_t)base * 3 + i);
        else reinterpret_cast<float*>(sl + kTcSlotFrac)[i] = 0.f;
      }
    };
    TcCursor cc, lc;  // the batch being built and the batch being loaded
    tc_cursor_init(cc, bins, num_items);
    lc = cc;
#pragma unroll
    for (int d = 0; d < kTcAhead; ++d) {
      if (lc.it < num_items) {
        load(lc, d);
        tc_cursor_step(lc, bins, num_items);
      }
      cp_async_commit();
    }
    // A rows past the tile's E0 E1 (up to the M-tiles' 128 L.mt) stay zero: written
    // once here, never by the per-batch builds (published by their proxy fences)
    {
      const int nrow = L.mt * 128 - rows;
      for (int i = tid; i < (int)ns * 2 * nrow * 2; i += kBuildThreads) {
        const int g = i & 1, rr = (i >> 1) % nrow, part = (i >> 1) / nrow;  // part: stage x (hi, lo)
        const int r = rows + rr;
        unsigned char* base = smem + (size_t)(part >> 1) * L.stage_bytes + (size_t)(part & 1) * L.a_bytes;
        *reinterpret_cast<uint4*>(base + tc_elem_off(r >> 3, r & 7, g)) = make_uint4(0u, 0u, 0u, 0u);
      }
    }
    cp_async_wait_group<kTcAhead - 1>();
    tc::named_sync(1, kBuildThreads);  // records of batch 0 visible
    uint32_t gb = 0, st = 0, cyc = 0;  // batch, its stage and cycle
    for (; cc.it < num_items; tc_cursor_step(cc, bins, num_items), ++gb) {
      // records of batch gb + kTcAhead into the slot batch gb - 1 used
      if (lc.it < num_items) {
        load(lc, (int)((gb + kTcAhead) % kTcRing));
        tc_cursor_step(lc, bins, num_items);
      }
      cp_async_commit();
      // stage st is free once the MMAs of batch gb - ns (its previous cycle) are complete:
      // one thread waits, and the builders' barrier after phase (1) publishes it (the
      // stage is written only in phase (2); a wait by every thread would poll one
      // mbarrier word from 32 lanes per warp)
      if (cyc > 0 && tid == kBuildThreads - 32)
        healthy &= tc::mbar_wait_bounded(&empty[st], (cyc - 1u) & 1u, kTcPolls);
      const unsigned char* sl = smem + L.rec_off + (gb % kTcRing) * kTcSlotBytes;
      const uint32_t* roff = reinterpret_cast<const uint32_t*>(sl + kTcSlotOff);
      const float* frac = reinterpret_cast<const float*>(sl + kTcSlotFrac);
      const float2* val = reinterpret_cast<const float2*>(sl + kTcSlotVal);
      float* wx = reinterpret_cast<float*>(smem + L.wx_off + (size_t)(gb & 1u) * L.wx_stage);
      float* wb = reinterpret_cast<float*>(smem + L.wb_off + (size_t)(gb & 1u) * L.wb_stage);
      unsigned char* stage = smem + (size_t)st * L.stage_bytes;
      unsigned char* a_hi = stage;
      unsigned char* a_lo = stage + L.a_bytes;
      unsigned char* b_hi = stage + 2 * L.a_bytes;
      unsigned char* b_lo = b_hi + kTcN * kTcK * 2;
      // (1) warps 0..7: lane (node j, half h) of warp w writes the B values w2 f of
      // columns p2 = 2 w + h and 2 w + h + 16 (rows 2 p2 + re|im of the B table; p2 >= E2
      // gives zero taps); the other builders: w0 and w1 over planes and rows
      if (warp < kBWarps) {
        const int j = lane & (kTcK - 1), p2a = 2 * warp + (lane >> 4);
        const int o = (int)(roff[j] >> (2 * SH));
        const float fr = frac[j * 3 + 2];
        const float2 c = val[j];
        float* const col = wb + j;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int p2 = p2a + 16 * i;
          const float w2 = tc_tap<WIN>(fr, mf, p2 - o, W, k2) * bscale;
          col[(2 * p2) * kTcWbStride] = w2 * c.x;
          col[(2 * p2 + 1) * kTcWbStride] = w2 * c.y;
        }
      } else {
        // lane (node j, dimension dd) of expansion warp xw: one load of the node's record,
        // then the taps of planes (dd = 0) or rows (dd = 1) xw, xw + kExpWarps, ...
        const int xw = warp - kBWarps, j = lane & (kTcK - 1), dd = lane >> 4;
        const uint32_t off = roff[j];
        const float fr = frac[j * 3 + dd];
        const int o = dd ? (int)((off >> SH) & MASK) : (int)(off & MASK);
        const int Ed = dd ? E1 : E0;
        const TapK kd = dd ? k1 : k0;
        float* const col = wx + (dd ? E0 : 0) * kTcWxStride + j;
        for (int p = xw; p < Ed; p += kExpWarps) col[p * kTcWxStride] = tc_tap<WIN>(fr, mf, p - o, W, kd);
      }
      cp_async_wait_group<kTcAhead - 1>();  // this thread's loads of batch gb + 1 have landed
      tc::named_sync(1, kBuildThreads);     // (1) done; stage st free, w0 / w1 and batch gb + 1's records visible
      // (2) B from registers; A: this thread's (node group, row) pair over its planes
      if (warp < kBWarps) {  // row 8 w + ri, nodes 4 q4 .. 4 q4 + 3
        const int q4 = lane >> 3;
        const float4 t = *reinterpret_cast<const float4*>(wb + (warp * 8 + ri) * kTcWbStride + 4 * q4);
        const float vv[4] = {t.x, t.y, t.z, t.w};
        uint2 hi, lo;
        tc_split4_f16(vv, hi, lo);
        const uint32_t o = tc_elem_off(warp, ri, q4 >> 1) + (uint32_t)(q4 & 1) * 8u;
        *reinterpret_cast<uint2*>(b_hi + o) = hi;
        *reinterpret_cast<uint2*>(b_lo + o) = lo;
      }
      if (a_on) {
        const float4 c0 = *reinterpret_cast<const float4*>(wx + (E0 + ap1) * kTcWxStride + akg * 8);
        const float4 c1 = *reinterpret_cast<const float4*>(wx + (E0 + ap1) * kTcWxStride + akg * 8 + 4);
        const float cw[8] = {c0.x * kTcScaleA, c0.y * kTcScaleA, c0.z * kTcScaleA, c0.w * kTcScaleA,
                             c1.x * kTcScaleA, c1.y * kTcScaleA, c1.z * kTcScaleA, c1.w * kTcScaleA};
#pragma unroll
        for (int i = 0; i < kAMaxP; ++i) {
          const int p0 = ablk + kAStride * i;
          if (p0 < E0) {
            const float4 a0 = *reinterpret_cast<const float4*>(wx + p0 * kTcWxStride + akg * 8);
            const float4 a1 = *reinterpret_cast<const float4*>(wx + p0 * kTcWxStride + akg * 8 + 4);
            const float v[8] = {a0.x * cw[0], a0.y * cw[1], a0.z * cw[2], a0.w * cw[3],
                                a1.x * cw[4], a1.y * cw[5], a1.z * cw[6], a1.w * cw[7]};
            uint4 hi, lo;
            tc_split8_f16(v, hi, lo);
            const int r = p0 * E1 + ap1;
            const uint32_t o = tc_elem_off(r >> 3, r & 7, akg);
            *reinterpret_cast<uint4*>(a_hi + o) = hi;
            *reinterpret_cast<uint4*>(a_lo + o) = lo;
          }
        }
      }
      tc::fence_proxy_async_smem();  // generic-proxy operand writes -> tensor core
      tc::mbar_arrive(&full[st]);
      if (++st == ns) {
        st = 0;
        ++cyc;
      }
    }
    cp_async_wait_group<0>();
  } else if (warp == kTcMmaWarp) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sa0 = tc::smem_u32(smem), sb0 = sa0 + 2 * L.a_bytes;
      const uint64_t d_ah = tc::smem_desc(sa0, kTcLBO, kTcSBO);
      const uint64_t d_al = tc::smem_desc(sa0 + L.a_bytes, kTcLBO, kTcSBO);
      const uint64_t d_bh = tc::smem_desc(sb0, kTcLBO, kTcSBO);
      const uint64_t d_bl = tc::smem_desc(sb0 + kTcN * kTcK * 2, kTcLBO, kTcSBO);
      const uint64_t d_stage = (uint64_t)(L.stage_bytes >> 4);  // stage s = stage 0 + s d_stage
      const uint32_t idesc = tc::idesc_f16(128, kTcN);
      uint32_t gb = 0, st = 0, cyc = 0, k = 0;
      int4 nxt = (int)blockIdx.x < num_items ? bins.items[blockIdx.x] : make_int4(0, 0, 0, 0);
      for (int it = blockIdx.x; it < num_items; it += G) {
        const int4 item = nxt;
        if (it + G < num_items) nxt = bins.items[it + G];  // one item ahead
        const int nbatch = (item.z - item.y + kTcK - 1) / kTcK;
        const uint32_t a = k % (uint32_t)L.nacc, use = k / (uint32_t)L.nacc;
        // accumulator a is free once the epilogue has read item k - nacc out of it
        if (use > 0) healthy &= tc::mbar_wait_bounded(&acc_empty[a], (use - 1) & 1u, kTcPolls);
        tc::fence_after_sync();
        const uint32_t acc = tmem + a * (uint32_t)(L.mt * kTcN);
        for (int b = 0; b < nbatch; ++b, ++gb) {
          healthy &= tc::mbar_wait_bounded(&full[st], cyc & 1u, kTcPolls);
          tc::fence_after_sync();
          const uint64_t so = (uint64_t)st * d_stage;
          for (int mt = 0; mt < L.mt; ++mt) {
            const uint32_t d = acc + (uint32_t)(mt * kTcN);
            const uint64_t am = so + (uint64_t)((mt * 16 * kTcSBO) >> 4);
            tc::mma_f16(d, d_ah + am, d_bh + so, idesc, b > 0 ? 1u : 0u);  // K = 16: the whole batch
            tc::mma_f16(d, d_ah + am, d_bl + so, idesc, 1u);
            tc::mma_f16(d, d_al + am, d_bh + so, idesc, 1u);
          }
          tc::mma_commit(&empty[st]);
          if (++st == ns) {
            st = 0;
            ++cyc;
          }
        }
        tc::mma_commit(&acc_full[a]);
        ++k;
      }
      // the last commit of each stage is waited by nobody else; no arrival may land after exit
      for (uint32_t i = 1; i <= ns && i <= gb; ++i) {
        const uint32_t bb = gb - i;
        healthy &= tc::mbar_wait_bounded(&empty[bb % ns], (bb / ns) & 1u, kTcPolls);
      }
    }
    __syncwarp();
  } else {
    // ======================= epilogue warps =======================
    // warp kTcEpiWarp0 + q reads TMEM lanes 32 q .. 32 q + 31, i.e. rows mt*128 + 32 q + lane,
    // and adds each row's (p2, p2 + 1) pairs to the grid with 16-byte atomics
    const int q = warp - kTcEpiWarp0;
    const int64_t n0 = geo.n[0], n1 = geo.n[1], n2 = geo.n[2];
    const int E1a = tl.E[1], E2a = tl.E[2];
    const bool one_wrap = n2 >= E2a;
    const float unscale = 1.f / (kTcScaleA * tc_scale_b(bins, (float)geo.norm));  // a power of two: exact
    // 16-byte pair atomics need an even row length and a 16-byte aligned grid
    const bool pairs = (n2 & 1) == 0 && (reinterpret_cast<uintptr_t>(g) & 15u) == 0 && (geo.ntot & 1) == 0;
    uint32_t k = 0;
    int4 nxt = (int)blockIdx.x < num_items ? bins.items[blockIdx.x] : make_int4(0, 0, 0, 0);
    for (int it = blockIdx.x; it < num_items; it += G) {
      const int4 item = nxt;
      if (it + G < num_items) nxt = bins.items[it + G];  // one item ahead
      const uint32_t a = k % (uint32_t)L.nacc, use = k / (uint32_t)L.nacc;
      const TileOrigin o = decode_tile<3>(geo, tl, item.x);
      float2* gi = g + o.inst * geo.ntot;
      healthy &= tc::mbar_wait_bounded(&acc_full[a], use & 1u, kTcPolls);
      __syncwarp();
      tc::fence_after_sync();
      const uint32_t acc = tmem + a * (uint32_t)(L.mt * kTcN) + ((uint32_t)(32 * q) << 16);
      // columns: a2 + p2 wraps at most once when the row is at least as long as the
      // padded tile (then p2 >= kw wraps); shorter rows take the general wrap
      const int kw = (int)(n2 - o.a[2] < 64 ? n2 - o.a[2] : 64);
      for (int mt = 0; mt < L.mt; ++mt) {
        const int r = mt * 128 + 32 * q + lane;
        const int p0 = r / E1, p1 = r - p0 * E1;
        const bool row_on = r < rows && p1 < E1a;
        const int64_t rbase = (wrap_up(o.a[0] + p0, n0) * n1 + wrap_up(o.a[1] + p1, n1)) * n2;
        float2* const rowa = gi + rbase + o.a[2];
        float2* const roww = rowa - n2;
#pragma unroll 1
        for (int c = 0; c < kTcN / 16; ++c) {
          float v[16];
          tc::tmem_ld16(acc + (uint32_t)(mt * kTcN + c * 16), v);
          tc::tmem_ld_wait();
          if (row_on) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int p2 = c * 8 + 2 * u;  // pair (p2, p2 + 1): columns 4u .. 4u + 3 of this load
              if (p2 < E2a) {
                float2* dst = one_wrap ? (p2 >= kw ? roww : rowa) + p2 : gi + rbase + wrap_up(o.a[2] + p2, n2);
                const float4 w = make_float4(v[4 * u] * unscale, v[4 * u + 1] * unscale, v[4 * u + 2] * unscale,
                                             v[4 * u + 3] * unscale);
                if (p2 + 1 < E2a && pairs) {  // the pair is 16-byte aligned
                  if (w.x != 0.f || w.y != 0.f || w.z != 0.f || w.w != 0.f)
                    atomicAdd(reinterpret_cast<float4*>(dst), w);
                } else {
                  if (w.x != 0.f || w.y != 0.f) atomicAdd(dst, make_float2(w.x, w.y));
                  if (p2 + 1 < E2a && (w.z != 0.f || w.w != 0.f))
                    atomicAdd(one_wrap ? (p2 + 1 >= kw ? roww : rowa) + (p2 + 1)
                                       : gi + rbase + wrap_up(o.a[2] + p2 + 1, n2),
                              make_float2(w.z, w.w));
                }
              }
            }
          }
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&acc_empty[a]);
      ++k;
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  __syncwarp();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, L.tmem_cols);
  if (!healthy) atomicExch(bins.status, 2);
}

}  // namespace cg
