// kernels_spread_tm.cuh -- 3D FP32 spreading on the tensor cores with the A operand in
// tensor memory (tcgen05.mma reading A from TMEM, B from shared memory).
//
// The reference's adjoint gridding (kernelConvWithGauss_adjoint_*, src/cunfft_kernel.cu:
// 608-1197), with the same window-start rule and taps, as the same product as k_spread_tc
// (kernels_spread_tc.cuh): per batch of kTmK = 32 nodes of a tile, D += A B^T with
//     A[(p0, p1), j]     = w0_j[p0 - o0_j] w1_j[p1 - o1_j]      (FP16 hi + lo, x 2^10)
//     B[(p2, re|im), j]  = w2_j[p2 - o2_j] (Re f_j | Im f_j)    (FP16 hi + lo, x 2^(14 - e))
// and the three products hi*hi + hi*lo + lo*hi accumulated in FP32.  Here the builder
// threads write A from registers straight into tensor memory (tcgen05.st), so shared
// memory carries only B, the node records and the expanded weights: A's shared-memory
// stores and the tensor core's shared-memory reads of A, most of k_spread_tc's
// shared-memory traffic, are gone.
//
// Rows of A and D: M-tile mt, TMEM lane L = p1 + E1 a (a < AP = floor(128 / E1)) is
// row (p0, p1) with p0 = a + AP mt; lanes with a >= AP or p0 >= E0 hold zero rows of
// A.  The thread owning lane L keeps its w1 row in registers over its M-tiles.
// Tensor memory (512 columns): the work item's accumulators in columns [0, 256)
// (M-tile mt at 64 mt, column 2 p2 + re|im) and kTmStages = 2 A stages in [256, 512)
// (stage s, M-tile mt: hi in 256 + 128 s + 32 mt .. + 15, lo in the next 16 columns; each
// batch is two MMA k-steps of 16 nodes, columns 8 ks of each part).
// There is one accumulator set: the MMAs of a work item's first batch wait, M-tile by
// M-tile, until the epilogue has read that M-tile of the previous item out.
//
// Warp roles (20 warps): 15 builders, one MMA issuer (lane 0), 4 epilogue warps.  Per
// batch the builders (1) evaluate w0 / w1 over the tile's planes and rows (lane = node
// and dimension) and the B values w2 f (lane = node and column) into shared tables
// (warps 8-14; w1 pre-scaled by the A scale 2^10), then after a named barrier among
// themselves (2) write A
// (warps 0-7: warp w owns lane quarter w % 4 of M-tiles w / 4 and w / 4 + 2) and split
// B into its shared-memory stage (warps 8-14).  The epilogue copies each M-tile into
// shared staging rows and releases it before its atomics.  Hand-offs are mbarriers; every wait
// is bounded, and a wait that gives up sets the plan's device status flag, after
// which the kernel still drains (bounded), frees its tensor memory and returns.
#pragma once

#include <cuda_fp16.h>

#include "kernels_spread_tc.cuh"

namespace cg {

constexpr int kTmBuilders = 15;                 // warps 0-7 write A; warps 8-14 the tables and B
constexpr int kTmAWarps = 8;
constexpr int kTmBWarps = kTmBuilders - kTmAWarps;  // 20 warps in all: 96 registers per thread
constexpr int kTmMmaWarp = kTmBuilders;         // lane 0 issues the MMAs
constexpr int kTmEpiWarp0 = kTmBuilders + 1;    // 4 epilogue warps: lane quarter warp % 4
constexpr int kTmThreads = (kTmBuilders + 1 + 4) * 32;
constexpr int kTmK = 32;                        // nodes per batch: two FP16 MMA k-steps of 16
constexpr int kTmStages = 2;                    // operand stages (A in TMEM, B in shared memory)
constexpr int kTmMaxMt = 4;                     // M-tiles: 4 x 64 accumulator columns
constexpr uint32_t kTmACol0 = 256;              // first A-stage column
constexpr uint32_t kTmAStageCols = 128;         // 4 M-tiles x (16 hi + 16 lo) columns
constexpr uint32_t kTmBPart = kTcN * kTmK * 2u; // B hi (or lo) of one stage
constexpr uint32_t kTmBStage = 2u * kTmBPart;
constexpr uint32_t kTmSBO = (kTmK / 8) * 128u;  // B: 8-row groups of kTmK / 8 core matrices
constexpr int kTmWxStride = 36;                 // floats per weight-table row: 8 consecutive rows, distinct banks
constexpr int kTmWbStride = 40;                 // floats per B-table row: rows two apart 16 banks apart
constexpr int kTmRing = 4;                      // record slots, loaded kTmRing - 1 batches ahead
constexpr uint32_t kTmSlotOff = 0, kTmSlotFrac = kTmK * 4, kTmSlotVal = kTmK * 16, kTmSlotBytes = kTmK * 24;
constexpr int kTmStgStride = kTcN + 4;          // floats per staging row: 8 consecutive rows, distinct banks

__host__ __device__ constexpr int tm_e1(int W) { return fixed_t_mid(3, W) + W - 1; }
__host__ __device__ constexpr int tm_ap(int W) { return 128 / tm_e1(W); }  // planes per M-tile
__host__ __device__ constexpr int tm_mt(int W, int E0) { return (E0 + tm_ap(W) - 1) / tm_ap(W); }

// 3D, and the tile's planes fit 4 M-tiles at AP planes each
__host__ __device__ constexpr bool spread_tm_ok(int d, int W, int T0, int E0) {
  return spread_tc_ok(d, W, T0) && tm_mt(W, E0) <= kTmMaxMt;
}

// Shared-memory layout of k_spread_tm (byte offsets; host and device agree).
struct TmLayout {
  int mt;               // M-tiles covering the tile's E0 planes
  uint32_t rec_off;     // kTmRing record slots (B stages at offset 0)
  uint32_t wx_off;      // 2 x ([E0][kTmWxStride] w0 over planes, [E1][kTmWxStride] w1 over rows)
  uint32_t wx_stage;
  uint32_t wb_off;      // 2 x [kTcN][kTmWbStride] B values w2 f (rows 2 p2 + re|im, kTmK nodes)
  uint32_t wb_stage;
  uint32_t bar_off;     // full[4], empty[4], acc_full[4], acc_empty[4]; tensor-memory base
  uint32_t stg_off;     // [4 x 128][kTmStgStride] accumulator rows staged for the atomics
  uint32_t total;
};

__host__ __device__ inline TmLayout tm_layout(int W, int E0) {
  TmLayout L{};
  L.mt = tm_mt(W, E0);
  L.rec_off = kTmStages * kTmBStage;
  L.wx_off = L.rec_off + kTmRing * kTmSlotBytes;
  L.wx_stage = (uint32_t)(E0 + tm_e1(W)) * kTmWxStride * 4u;
  L.wb_off = (L.wx_off + 2u * L.wx_stage + 15u) & ~15u;
  L.wb_stage = (uint32_t)kTcN * kTmWbStride * 4u;
  L.bar_off = L.wb_off + 2u * L.wb_stage;
  L.stg_off = L.bar_off + 16u * 8u + 16u;
  L.total = L.stg_off + (uint32_t)kTmMaxMt * 128u * kTmStgStride * 4u;
  return L;
}

// TcCursor step over batches of kTmK nodes
__device__ __forceinline__ void tm_cursor_step(TcCursor& c, const Bins& bins, int num_items) {
  const int G = (int)gridDim.x;
  if (c.item.y + (++c.b) * kTmK < c.item.z) return;
  c.it += G;
  c.b = 0;
  c.item = c.next;
  c.next = c.it + G < num_items ? bins.items[c.it + G] : make_int4(0, 0, 0, 0);
}

template <int W, int WIN>
__global__ void __launch_bounds__(kTmThreads, 1) k_spread_tm(const float2* __restrict__ f, float2* __restrict__ g,
                                                             Geom geo, Tiling tl, Bins bins) {
  constexpr int E1 = tm_e1(W), AP = tm_ap(W);
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr int kBuildThreads = kTmBuilders * 32;
  static_assert(2 * (fixed_t_last(3, W) + W - 1) <= kTcN, "complex columns must fit the MMA N");
  static_assert(kTmK == 32 && kTcN == 64, "staging roles assume 32 nodes and 64 B rows");
  static_assert(AP >= 1, "a plane's rows must fit one M-tile");
  extern __shared__ __align__(16) unsigned char smem[];
  const int E0 = tl.E[0];
  const TmLayout L = tm_layout(W, E0);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bar_off);  // [4] operands of stage s written
  uint64_t* empty = full + 4;                                       // [4] MMAs of stage s complete
  uint64_t* acc_full = full + 8;                                    // [4] M-tile mt of the item complete
  uint64_t* acc_empty = full + 12;                                  // [4] M-tile mt read out
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 128);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + L.bar_off + 132);  // a wait gave up
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  if (tid == 0) {
    for (int i = 0; i < 4; ++i) {
      tc::mbar_init(&full[i], kBuildThreads);
      tc::mbar_init(&empty[i], 1);
      tc::mbar_init(&acc_full[i], 1);
      tc::mbar_init(&acc_empty[i], 128);
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

  // Every role walks items c, c + G, ... (CTA c); batch gb (counted across the CTA's
  // items) uses stage gb % 4 in its cycle gb / 4 and record / table buffers gb & 1.
  // A role whose bounded wait gives up raises abort_flag and leaves its loop; the
  // builders leave together after their barrier, the others at their next wait, so a
  // broken hand-off ends the kernel after a few bounded waits instead of one per batch.
  if (warp < kTmBuilders) {
    // ======================= builder warps =======================
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    const float2* fperm = reinterpret_cast<const float2*>(bins.fperm);
    const float norm = (float)geo.norm;
    const float bscale = norm * tc_scale_b(bins, norm);  // w2 f -> B
    const float mf = (float)geo.m;
    const TapK k0 = tap_k<WIN>(geo, 0), k1 = tap_k<WIN>(geo, 1), k2 = tap_k<WIN>(geo, 2);
    // A writer (warps 0-7): TMEM lane aL of M-tiles amt, amt + 2
    const int aq = warp & 3, amt = (warp >> 2) & 1, aL = 32 * aq + lane;
    const int aa = aL / E1, ap1 = aL - aa * E1;
    const bool a_row = aa < AP;
    // loads of one batch's records into ring slot `slot` (threads < 4 kTmK)
    auto load = [&](const TcCursor& c, int slot) {
      unsigned char* sl = smem + L.rec_off + slot * kTmSlotBytes;
      const int base = c.item.y + c.b * kTmK, n = min(kTmK, c.item.z - base);
      if (tid < kTmK) {
        if (tid < n) {
          cp_async4(sl + kTmSlotOff + tid * 4, bins.soff + base + tid);
          cp_async8(sl + kTmSlotVal + tid * 8, fperm + base + tid);
        } else {
          reinterpret_cast<int*>(sl + kTmSlotOff)[tid] = -1;
          reinterpret_cast<float2*>(sl + kTmSlotVal)[tid] = make_float2(0.f, 0.f);
        }
      } else if (tid < 4 * kTmK) {
        const int i = tid - kTmK;
        if (i < 3 * n) cp_async4(sl + kTmSlotFrac + i * 4, sfrac + (int64_t)base * 3 + i);
        else reinterpret_cast<float*>(sl + kTmSlotFrac)[i] = 0.f;
      }
    };
    TcCursor cc, lc;  // the batch being built and the batch being loaded
    tc_cursor_init(cc, bins, num_items);
    lc = cc;
#pragma unroll
    for (int d = 0; d < kTmRing - 1; ++d) {
      if (lc.it < num_items) {
        load(lc, d);
        tm_cursor_step(lc, bins, num_items);
      }
      cp_async_commit();
    }
    cp_async_wait_group<kTmRing - 2>();
    tc::named_sync(1, kBuildThreads);  // records of batch 0 visible
    uint32_t gb = 0, st = 0, cyc = 0;
    for (; cc.it < num_items; tm_cursor_step(cc, bins, num_items), ++gb) {
      if (lc.it < num_items) {
        load(lc, (int)((gb + kTmRing - 1) % kTmRing));
        tm_cursor_step(lc, bins, num_items);
      }
      cp_async_commit();
      // stage st (its B buffer and its A columns) is free once the MMAs of batch gb - 4
      // are complete: one thread waits, the barrier after phase (1) publishes it
      bool fail = false;
      if (cyc > 0 && tid == kBuildThreads - 32) fail = !tc::mbar_wait_bounded(&empty[st], (cyc - 1u) & 1u, kTcPolls);
      healthy &= !fail;
      const unsigned char* sl = smem + L.rec_off + (gb % kTmRing) * kTmSlotBytes;
      const uint32_t* roff = reinterpret_cast<const uint32_t*>(sl + kTmSlotOff);
      const float* frac = reinterpret_cast<const float*>(sl + kTmSlotFrac);
      const float2* val = reinterpret_cast<const float2*>(sl + kTmSlotVal);
      float* wx = reinterpret_cast<float*>(smem + L.wx_off + (size_t)(gb & 1u) * L.wx_stage);
      float* wb = reinterpret_cast<float*>(smem + L.wb_off + (size_t)(gb & 1u) * L.wb_stage);
      // a batch of at most 16 nodes (most of an item's last batch) needs only the first
      // node half: its second k-step is neither built nor multiplied
      const int halves = cc.item.z - (cc.item.y + cc.b * kTmK) > 16 ? 2 : 1;
      if (warp >= kTmAWarps) {
        // (1) the B warps evaluate every table of the batch (the A warps' phase (2) is
        // the long one): lane (node j, dimension dd) of warp kTmAWarps + w the taps of
        // planes (dd = 0) or rows (dd = 1) w, w + kTmBWarps, ...; lane (node j, half h)
        // the B values w2 f of columns p2 = 2 w + h + 2 kTmBWarps i < 32 (p2 >= E2 gives
        // zero taps)
        const int bw = warp - kTmAWarps, hd = lane >> 4;
#pragma unroll
        for (int jh = 0; jh < kTmK / 16; ++jh) {  // the batch's node halves
          if (jh >= halves) break;
          const int j = 16 * jh + (lane & 15);
          const uint32_t off = roff[j];
          {
            const float fr = frac[j * 3 + hd];
            const int o = hd ? (int)((off >> SH) & MASK) : (int)(off & MASK);
            const int Ed = hd ? E1 : E0;
            const TapK kd = hd ? k1 : k0;
            const float sc = hd ? kTcScaleA : 1.f;  // w1 carries the A scale 2^10
            float* const col = wx + (hd ? E0 : 0) * kTmWxStride + j;
            for (int p = bw; p < Ed; p += kTmBWarps) col[p * kTmWxStride] = tc_tap<WIN>(fr, mf, p - o, W, kd) * sc;
          }
          const int o2 = (int)(off >> (2 * SH));
          const float fr2 = frac[j * 3 + 2];
          const float2 c = val[j];
          float* const col = wb + j;
#pragma unroll
          for (int i = 0; i < (kTcN / 2 + 2 * kTmBWarps - 1) / (2 * kTmBWarps); ++i) {
            const int p2 = 2 * bw + hd + 2 * kTmBWarps * i;
            if (p2 >= kTcN / 2) break;
            const float w2 = tc_tap<WIN>(fr2, mf, p2 - o2, W, k2) * bscale;
            col[(2 * p2) * kTmWbStride] = w2 * c.x;
            col[(2 * p2 + 1) * kTmWbStride] = w2 * c.y;
          }
        }
      }
      cp_async_wait_group<kTmRing - 2>();  // this thread's loads of batch gb + 1 have landed
      // (1) done; stage st free, tables and next records visible; the builders leave
      // together when any of them saw a wait give up or the abort flag raised
      if (tc::named_sync_or(1, kBuildThreads, fail || *abort_flag != 0)) {
        healthy = false;
        break;
      }
      if (warp < kTmAWarps) {
        // (2) A rows of lane aL, M-tiles amt and amt + 2: w0 (w1 2^10) -> FP16 hi, lo
        tc::fence_after_sync();
        const uint32_t tq = tmem + ((uint32_t)(32 * aq) << 16) + kTmACol0 + st * kTmAStageCols;
#pragma unroll
        for (int kh = 0; kh < kTmK / 16; ++kh) {  // nodes 16 kh .. 16 kh + 15: columns 8 kh of each part
          if (kh >= halves) break;
          float2 w1r[8];
          if (a_row) {
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
              const float4 t = *reinterpret_cast<const float4*>(wx + (E0 + ap1) * kTmWxStride + 16 * kh + 4 * c4);
              w1r[2 * c4] = make_float2(t.x, t.y);
              w1r[2 * c4 + 1] = make_float2(t.z, t.w);
            }
          } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) w1r[k] = make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int mt = amt + 2 * i;
            if (mt < L.mt) {
              const int p0 = aa + AP * mt;
              uint32_t hi[8], lo[8];
              if (a_row && p0 < E0) {
#pragma unroll
                for (int c4 = 0; c4 < 4; ++c4) {
                  const float4 t = *reinterpret_cast<const float4*>(wx + p0 * kTmWxStride + 16 * kh + 4 * c4);
                  tc_split2_f16(__fmul2_rn(make_float2(t.x, t.y), w1r[2 * c4]), hi[2 * c4], lo[2 * c4]);
                  tc_split2_f16(__fmul2_rn(make_float2(t.z, t.w), w1r[2 * c4 + 1]), hi[2 * c4 + 1], lo[2 * c4 + 1]);
                }
              } else {
#pragma unroll
                for (int c = 0; c < 8; ++c) hi[c] = lo[c] = 0u;
              }
              tc::tmem_st8(tq + (uint32_t)(32 * mt + 8 * kh), hi);
              tc::tmem_st8(tq + (uint32_t)(32 * mt + 16 + 8 * kh), lo);
            }
          }
        }
        tc::tmem_st_wait();
        tc::fence_before_sync();
      } else {
        // (2) B rows 8 rg + ri (lane ri = lane & 7) of row groups rg = w, w + kTmBWarps < 8,
        // nodes 4 q .. 4 q + 3 (q = q4, q4 + 4) -> FP16 hi, lo
        const int ri = lane & 7, q4 = lane >> 3;
        unsigned char* b_hi = smem + (size_t)st * kTmBStage;
        for (int rg = warp - kTmAWarps; rg < kTcN / 8; rg += kTmBWarps) {
#pragma unroll
          for (int kh = 0; kh < kTmK / 16; ++kh) {
            if (kh >= halves) break;
            const int q = q4 + 4 * kh;
            const float4 t = *reinterpret_cast<const float4*>(wb + (rg * 8 + ri) * kTmWbStride + 4 * q);
            const float vv[4] = {t.x, t.y, t.z, t.w};
            uint2 hi, lo;
            tc_split4_f16(vv, hi, lo);
            const uint32_t o = (uint32_t)rg * kTmSBO + (uint32_t)(q >> 1) * kTcLBO + (uint32_t)ri * 16u +
                               (uint32_t)(q & 1) * 8u;
            *reinterpret_cast<uint2*>(b_hi + o) = hi;
            *reinterpret_cast<uint2*>(b_hi + kTmBPart + o) = lo;
          }
        }
        tc::fence_proxy_async_smem();  // generic-proxy operand writes -> tensor core
      }
      tc::mbar_arrive(&full[st]);
      if (++st == kTmStages) {
        st = 0;
        ++cyc;
      }
    }
    cp_async_wait_group<0>();
  } else if (warp == kTmMmaWarp) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sb0 = tc::smem_u32(smem);
      const uint64_t d_bh = tc::smem_desc(sb0, kTcLBO, kTmSBO);
      const uint64_t d_bl = tc::smem_desc(sb0 + kTmBPart, kTcLBO, kTmSBO);
      const uint64_t d_stage = (uint64_t)(kTmBStage >> 4);  // stage s = stage 0 + s d_stage
      const uint32_t idesc = tc::idesc_f16(128, kTcN);
      uint32_t gb = 0, st = 0, cyc = 0, k = 0;
      int4 nxt = (int)blockIdx.x < num_items ? bins.items[blockIdx.x] : make_int4(0, 0, 0, 0);
      for (int it = blockIdx.x; it < num_items; it += G, ++k) {
        const int4 item = nxt;
        if (it + G < num_items) nxt = bins.items[it + G];  // one item ahead
        const int nbatch = (item.z - item.y + kTmK - 1) / kTmK;
        for (int b = 0; b < nbatch && healthy; ++b, ++gb) {
          const int halves = item.z - (item.y + b * kTmK) > 16 ? 2 : 1;  // k-steps built (as the builders)
          healthy = tc::mbar_wait_bounded(&full[st], cyc & 1u, kTcPolls);
          if (!healthy) break;
          tc::fence_after_sync();
          const uint64_t so = (uint64_t)st * d_stage;
          const uint32_t ta = tmem + kTmACol0 + st * kTmAStageCols;
          for (int mt = 0; mt < L.mt; ++mt) {
            if (b == 0 && k > 0) {  // M-tile mt of item k - 1 read out
              healthy &= tc::mbar_wait_bounded(&acc_empty[mt], (k - 1u) & 1u, kTcPolls);
              tc::fence_after_sync();
            }
            const uint32_t d = tmem + (uint32_t)(mt * kTcN), am = ta + (uint32_t)(32 * mt);
#pragma unroll
            for (int ks = 0; ks < kTmK / 16; ++ks) {  // k-steps of 16 nodes: A columns 8 ks, B 256 ks bytes
              if (ks >= halves) break;
              const uint64_t kb = (uint64_t)(ks * 2 * kTcLBO) >> 4;
              const uint32_t ak = am + (uint32_t)(8 * ks);
              tc::mma_f16_ta(d, ak, d_bh + so + kb, idesc, (b > 0 || ks > 0) ? 1u : 0u);
              tc::mma_f16_ta(d, ak, d_bl + so + kb, idesc, 1u);
              tc::mma_f16_ta(d, ak + 16u, d_bh + so + kb, idesc, 1u);
            }
            if (b == nbatch - 1) tc::mma_commit(&acc_full[mt]);
          }
          tc::mma_commit(&empty[st]);
          if (++st == kTmStages) {
            st = 0;
            ++cyc;
          }
        }
        if (!healthy) {
          *abort_flag = 1;
          break;
        }
      }
      // the last commit of each stage is waited by nobody else; no arrival may land after exit
      for (uint32_t i = 1; i <= (uint32_t)kTmStages && i <= gb; ++i) {
        const uint32_t bb = gb - i;
        healthy &= tc::mbar_wait_bounded(&empty[bb % kTmStages], (bb / kTmStages) & 1u, kTcPolls);
      }
    }
    __syncwarp();
  } else {
    // ======================= epilogue warps =======================
    // Per work item: warp kTmEpiWarp0 + i copies TMEM lanes 32 q .. 32 q + 31 (q = warp % 4)
    // of each M-tile into its own shared staging rows and releases the M-tile at once, so
    // the next item's MMAs need not wait for the reductions; then each thread adds its
    // rows to the grid.  With an even row length and at most one wrap of the tile's
    // columns, a row is one or two contiguous runs of the grid row: each run goes as one
    // bulk FP32 reduction (cp.reduce.async.bulk, performed in L2; runs rounded up to
    // 16 bytes with the zero column past the tile); otherwise 16- or 8-byte atomics.
    // A thread reads back only the rows it wrote, so the staging needs no barrier; it
    // waits for its bulk reductions to have read a row before rewriting it.
    const int q = warp & 3;
    const int64_t n0 = geo.n[0], n1 = geo.n[1], n2 = geo.n[2];
    const int E1a = tl.E[1], E2a = tl.E[2];
    const bool one_wrap = n2 >= E2a;
    const float unscale = 1.f / (kTcScaleA * tc_scale_b(bins, (float)geo.norm));  // a power of two: exact
    // 16-byte pair atomics need an even row length and a 16-byte aligned grid
    const bool pairs = (n2 & 1) == 0 && (reinterpret_cast<uintptr_t>(g) & 15u) == 0 && (geo.ntot & 1) == 0;
    const int eL = 32 * q + lane, ea = eL / E1, ep1 = eL - ea * E1;
    float* const stg = reinterpret_cast<float*>(smem + L.stg_off) + eL * kTmStgStride;  // + 128 mt rows
    uint32_t k = 0;
    int4 nxt = (int)blockIdx.x < num_items ? bins.items[blockIdx.x] : make_int4(0, 0, 0, 0);
    for (int it = blockIdx.x; it < num_items; it += G, ++k) {
      const int4 item = nxt;
      if (it + G < num_items) nxt = bins.items[it + G];  // one item ahead
      tc::bulk_wait_read();  // the previous item's reductions have read the staging rows
      for (int mt = 0; mt < L.mt && healthy; ++mt) {
        healthy = __all_sync(0xffffffffu, tc::mbar_wait_bounded(&acc_full[mt], k & 1u, kTcPolls));
        if (!healthy) break;
        tc::fence_after_sync();
        const uint32_t acc = tmem + (uint32_t)(mt * kTcN) + ((uint32_t)(32 * q) << 16);
        float* const srow = stg + mt * 128 * kTmStgStride;
#pragma unroll
        for (int c = 0; c < kTcN / 16; ++c) {
          float v[16];
          tc::tmem_ld16(acc + (uint32_t)(c * 16), v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int u = 0; u < 4; ++u)
            *reinterpret_cast<float4*>(srow + 16 * c + 4 * u) =
                make_float4(v[4 * u] * unscale, v[4 * u + 1] * unscale, v[4 * u + 2] * unscale, v[4 * u + 3] * unscale);
        }
        tc::fence_before_sync();
        tc::mbar_arrive(&acc_empty[mt]);
      }
      if (!healthy) {
        *abort_flag = 1;
        break;
      }
      const TileOrigin o = decode_tile<3>(geo, tl, item.x);
      float2* gi = g + o.inst * geo.ntot;
      // columns: a2 + p2 wraps at most once when the row is at least as long as the
      // padded tile (then p2 >= kw wraps); shorter rows take the general wrap
      const int kw = (int)(n2 - o.a[2] < 64 ? n2 - o.a[2] : 64);
      const bool bulk = one_wrap && (n2 & 1) == 0;
      if (bulk) tc::fence_proxy_async_smem();  // staged rows -> bulk-copy engine
#pragma unroll 1
      for (int mt = 0; mt < L.mt; ++mt) {
        const int p0 = ea + AP * mt;
        if (!(ea < AP && p0 < E0 && ep1 < E1a)) continue;
        const float* const srow = stg + mt * 128 * kTmStgStride;
        const int64_t rbase = (wrap_up(o.a[0] + p0, n0) * n1 + wrap_up(o.a[1] + ep1, n1)) * n2;
        float2* const rowa = gi + rbase + o.a[2];
        float2* const roww = rowa - n2;
        if (bulk) {
          // run 1: columns [0, c1) at a2 + p2; run 2: columns [kw, E2a) at p2 - kw (wrapped)
          const uint32_t s0 = tc::smem_u32(srow);
          const int c1 = E2a < kw ? E2a : kw;
          const uint32_t b1 = (uint32_t)((c1 + 1) & ~1) * 8u;
          const uint32_t b2 = kw < E2a ? (uint32_t)((E2a - kw + 1) & ~1) * 8u : 0u;
          const bool aligned = ((reinterpret_cast<uintptr_t>(rowa) | s0) & 15u) == 0u &&
                               ((reinterpret_cast<uintptr_t>(roww + kw) | (s0 + (uint32_t)kw * 8u)) & 15u) == 0u;
          if (aligned) {
            tc::bulk_reduce_add_f32(rowa, s0, b1);
            if (b2) tc::bulk_reduce_add_f32(roww + kw, s0 + (uint32_t)kw * 8u, b2);
            continue;
          }
        }
#pragma unroll 4
        for (int u = 0; u < kTcN / 4; ++u) {
          const int p2 = 2 * u;  // pair (p2, p2 + 1): staged columns 4u .. 4u + 3
          if (p2 < E2a) {
            const float4 w = *reinterpret_cast<const float4*>(srow + 4 * u);  // scaled when staged
            float2* dst = one_wrap ? (p2 >= kw ? roww : rowa) + p2 : gi + rbase + wrap_up(o.a[2] + p2, n2);
            if (p2 + 1 < E2a && pairs) {  // the pair is 16-byte aligned
              if (w.x != 0.f || w.y != 0.f || w.z != 0.f || w.w != 0.f) atomicAdd(reinterpret_cast<float4*>(dst), w);
            } else {
              if (w.x != 0.f || w.y != 0.f) atomicAdd(dst, make_float2(w.x, w.y));
              if (p2 + 1 < E2a && (w.z != 0.f || w.w != 0.f))
                atomicAdd(one_wrap ? (p2 + 1 >= kw ? roww : rowa) + (p2 + 1) : gi + rbase + wrap_up(o.a[2] + p2 + 1, n2),
                          make_float2(w.z, w.w));
            }
          }
        }
      }
      tc::bulk_commit();
    }
    tc::bulk_wait_all();  // every reduction complete before the CTA's shared memory goes
  }
  tc::fence_before_sync();
  __syncthreads();
  __syncwarp();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (!healthy) atomicExch(bins.status, 2);
}

}  // namespace cg
