// kernels_spread2_tm.cuh -- 2D FP32 spreading on the tensor cores (tcgen05, FP16 hi/lo x 3).
//
// The reference's 2D adjoint gridding (kernelConvWithGauss_adjoint_2d, FGG form
// src/cunfft_kernel.cu:842-878: every node adds f_j psi_0 psi_1 to a (2m+2)^2 window of the
// oversampled grid through CAS-loop atomics), with the same window-start rule and taps,
// computed per tile of the binned nodes as a matrix product.  For a tile of T0 x T1 grid
// points (T0, T1 <= 64; padded extents E0 = T0 + W - 1 <= 128, E1 = T1 + W - 1 <= 79) and
// a batch of kTcK = 16 nodes,
//     D[p0, 2 p1 + c] += sum_j A[p0, j] B[2 p1 + c, j]
//     A[p0, j]         = w0_j[p0 - o0_j] 2^10                     (M = 128 rows)
//     B[2 p1 + c, j]   = w1_j[p1 - o1_j] (Re f_j | Im f_j) s_B    (N = 160 columns)
// with taps zero outside a node's window, s_B = norm 2^(14 - e) (2^e bounds the samples, as
// in the 3D kernels), both operands split into FP16 hi + lo and the three products
// hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory.
//
// Unlike 3D, both operands are one tap wide: a node costs 128 A entries and 160 B entries
// (against W^2 <= 256 taps), and the tensor core does the W^2 multiply-adds.  Each operand
// thread evaluates the taps of its own row (A: row p0, w0 of the 16 nodes) or column pair
// (B: column p1, w1 of 8 nodes) straight from the node records, so no stage sits between
// the records and the operands.
//
// Warp roles (25 warps): two sets of operand warps that take alternate batches (set s the
// batches gb with gb % 2 = s), A warps 0-3 and 16-19 (warp w writes TMEM lanes
// 32 (w % 4) .. + 31 of the operand stage, one row p0 per thread, hi and lo halves with
// tcgen05.st), B warps 4-8 and 20-24 (thread t of 160: rows 2 p1 and 2 p1 + 1 of B, nodes
// 8 h .. 8 h + 7, p1 = t / 2, h = t % 2, into the shared-memory operand stage); the record
// warp 9 (node records into a ring of kT2Ring slots by cp.async, kT2Ahead batches ahead);
// the MMA warp 10 (lane 0); epilogue warps 12-15 (TMEM lane quarter warp % 4); warp 11
// idles.  Operands are four stages deep (full / empty), records kT2Ring deep (rec_full /
// rec_empty), and the accumulators double-buffered in tensor memory (acc_full /
// acc_empty): while the epilogue reads one work item's tile out and adds it to the grid as
// bulk FP32 reductions (cp.reduce.async.bulk, one or two per row), the MMAs of the next
// item accumulate into the other set.  Every mbarrier wait is bounded; a wait that gives up
// sets the plan's device status flag, after which the kernel drains (bounded), frees its
// tensor memory and returns.
#pragma once

#include <cuda_fp16.h>

#include "kernels_spread_tc.cuh"

namespace cg {

constexpr int kT2MaxT0 = 64;               // E0 = T0 + W - 1 <= 128 rows (M = 128)
constexpr int kT2N = 160;                  // MMA N: 2 E1 <= 158 columns (p1, re|im), padded
constexpr int kT2AWarps = 4;
constexpr int kT2BWarps = 5;               // 160 threads: (p1 < 80, node half)
constexpr int kT2OpWarps = kT2AWarps + kT2BWarps;
constexpr int kT2RecWarp = kT2OpWarps;     // warp 9
constexpr int kT2MmaWarp = kT2RecWarp + 1; // warp 10
constexpr int kT2EpiWarp0 = 12;            // warps 12-15: lane quarters 0-3
constexpr int kT2OpSet1 = 16;              // warps 16-24: the operand warps of odd batches
constexpr int kT2Threads = (kT2OpSet1 + kT2OpWarps) * 32;
constexpr int kT2Stages = 4;
constexpr int kT2Ring = 8;                 // record slots
constexpr int kT2Ahead = 4;                // record loads in flight (batches)
constexpr uint32_t kT2Spin = 8;            // non-blocking polls before a hand-off wait suspends
constexpr uint32_t kT2BBytes = (uint32_t)kT2N * kTcK * 2u;   // one FP16 part of one B stage
constexpr uint32_t kT2ACol0 = 2u * kT2N;   // A stages after the two accumulator sets
constexpr int kT2StgStride = kT2N + 4;     // floats per staging row
constexpr uint32_t kT2SlotOff = 0, kT2SlotFrac = kTcK * 4, kT2SlotVal = kTcK * 12, kT2SlotBytes = kTcK * 20;

__host__ __device__ constexpr bool spread2_tm_ok(int d, int W, int T0, int T1) {
  return d == 2 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kT2MaxT0 && T1 >= 1 && T1 <= 64;
}

// Shared-memory layout of k_spread2_tm (byte offsets; host and device agree).
struct T2Layout {
  uint32_t b_off;     // kT2Stages x (B hi, B lo)
  uint32_t rec_off;   // kT2Ring record slots: window starts [16], fractions [16][2], samples [16]
  uint32_t bar_off;   // full[4], empty[4], acc_full[2], acc_empty[2], rec_full[8], rec_empty[8];
                      // tensor-memory base, abort flag
  uint32_t stg_off;   // [128][kT2StgStride] accumulator rows staged for the reductions
  uint32_t total;
};

__host__ __device__ constexpr T2Layout t2_layout() {
  T2Layout L{};
  L.b_off = 0;
  L.rec_off = kT2Stages * 2u * kT2BBytes;
  L.bar_off = (L.rec_off + kT2Ring * kT2SlotBytes + 15u) & ~15u;
  L.stg_off = L.bar_off + (12u + 2u * kT2Ring) * 8u + 16u;
  L.total = L.stg_off + 128u * kT2StgStride * 4u;
  return L;
}

template <int W, int WIN>
__global__ void __launch_bounds__(kT2Threads, 1) k_spread2_tm(const float2* __restrict__ f, float2* __restrict__ g,
                                                              Geom geo, Tiling tl, Bins bins) {
  constexpr int SH = off_bits(2);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr T2Layout L = t2_layout();
  static_assert(2 * (63 + W) <= kT2N, "complex columns must fit the MMA N");
  static_assert(kTcK == 16, "roles assume 16 nodes per batch");
  extern __shared__ __align__(16) unsigned char smem[];
  const int E0 = tl.E[0], E1 = tl.E[1];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bar_off);  // [4] operands of stage s written
  uint64_t* empty = full + 4;                                       // [4] MMAs of stage s complete
  uint64_t* acc_full = full + 8;                                    // [2] accumulator set s complete
  uint64_t* acc_empty = full + 10;                                  // [2] accumulator set s read out
  uint64_t* rec_full = full + 12;                                   // [kT2Ring] records of slot r landed
  uint64_t* rec_empty = rec_full + kT2Ring;                         // [kT2Ring] slot r read
  unsigned char* const bar_end = smem + L.bar_off + (12u + 2u * kT2Ring) * 8u;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_end);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bar_end + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  if (tid == 0) {
    for (int i = 0; i < 4; ++i) {
      tc::mbar_init(&full[i], kT2OpWarps);  // one arrival per operand warp of the batch's set
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&acc_full[i], 1);
      tc::mbar_init(&acc_empty[i], 4);      // one arrival per epilogue warp
    }
    for (int i = 0; i < kT2Ring; ++i) {
      tc::mbar_init(&rec_full[i], 1);       // the record warp
      tc::mbar_init(&rec_empty[i], kT2OpWarps);
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

  // Every role walks items c, c + G, ... (CTA c) in batches of kTcK nodes; batch gb
  // (counted across the CTA's items) uses operand stage gb % 4 in its cycle gb / 4, record
  // slot gb % kT2Ring and operand set gb % 2; item k of the CTA accumulates into set k % 2.
  if (warp == kT2RecWarp) {
    // ======================= record warp =======================
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    const float2* fperm = reinterpret_cast<const float2*>(bins.fperm);
    TcCursor lc;
    tc_cursor_init(lc, bins, num_items);
    uint32_t gb = 0;
    for (; lc.it < num_items; tc_cursor_step(lc, bins, num_items), ++gb) {
      const uint32_t r = gb % kT2Ring;
      // slot r free once both operand sets' warps of batch gb - kT2Ring have read it
      if (gb >= (uint32_t)kT2Ring &&
          !tc::mbar_wait_warp(&rec_empty[r], ((gb / kT2Ring) - 1u) & 1u, kTcPolls)) {
        healthy = false;
        break;
      }
      if (*abort_flag != 0) {
        healthy = false;
        break;
      }
      unsigned char* sl = smem + L.rec_off + r * kT2SlotBytes;
      const int base = lc.item.y + lc.b * kTcK, n = min(kTcK, lc.item.z - base);
      if (lane < kTcK) {
        if (lane < n) {
          cp_async4(sl + kT2SlotOff + lane * 4, bins.soff + base + lane);
          cp_async8(sl + kT2SlotVal + lane * 8, fperm + base + lane);
        } else {
          reinterpret_cast<uint32_t*>(sl + kT2SlotOff)[lane] = 0xffffffffu;  // no node: zero taps
          reinterpret_cast<float2*>(sl + kT2SlotVal)[lane] = make_float2(0.f, 0.f);
        }
      }
      if (lane < 2 * n) cp_async4(sl + kT2SlotFrac + lane * 4, sfrac + (int64_t)base * 2 + lane);
      else reinterpret_cast<float*>(sl + kT2SlotFrac)[lane] = 0.f;
      cp_async_commit();
      if (gb >= (uint32_t)kT2Ahead) {  // the records of batch gb - kT2Ahead have landed
        cp_async_wait_group<kT2Ahead>();
        tc::mbar_arrive_warp(&rec_full[(gb - kT2Ahead) % kT2Ring]);
      }
    }
    cp_async_wait_group<0>();
    for (uint32_t b = gb > (uint32_t)kT2Ahead ? gb - kT2Ahead : 0u; b < gb; ++b)
      tc::mbar_arrive_warp(&rec_full[b % kT2Ring]);
    if (!healthy) *abort_flag = 1;
  } else if (warp < kT2OpWarps || warp >= kT2OpSet1) {
    // ======================= operand warps: A (0-3, 16-19) and B (4-8, 20-24) =======================
    const uint32_t set = warp >= kT2OpSet1 ? 1u : 0u;
    const int lw = warp - (set ? kT2OpSet1 : 0);
    const bool is_a = lw < kT2AWarps;
    const int p0 = 32 * lw + lane;                        // A: row (TMEM lane; warp % 4 == lw)
    const int bt = 32 * (lw - kT2AWarps) + lane;         // B: task
    const int p1 = bt >> 1, h = bt & 1;
    const float mf = (float)geo.m;
    const TapK k0 = tap_k<WIN>(geo, 0), k1 = tap_k<WIN>(geo, 1);
    const float norm = (float)geo.norm;
    const float bscale = norm * tc_scale_b(bins, norm);
    uint32_t gb = 0;
    TcCursor cc;
    tc_cursor_init(cc, bins, num_items);
    for (; cc.it < num_items; tc_cursor_step(cc, bins, num_items), ++gb) {
      if ((gb & 1u) != set) continue;
      const uint32_t r = gb % kT2Ring, st = gb & 3u, cyc = gb >> 2;
      bool ok = tc::mbar_wait_warp(&rec_full[r], (gb / kT2Ring) & 1u, kTcPolls, kT2Spin);
      if (ok && cyc > 0) ok = tc::mbar_wait_warp(&empty[st], (cyc - 1u) & 1u, kTcPolls, kT2Spin);
      if (!ok || *abort_flag != 0) {
        healthy = false;
        break;
      }
      const unsigned char* sl = smem + L.rec_off + r * kT2SlotBytes;
      const uint32_t* offs = reinterpret_cast<const uint32_t*>(sl + kT2SlotOff);
      const float2* frs = reinterpret_cast<const float2*>(sl + kT2SlotFrac);
      // Does any node of the batch reach this warp's rows (A: p0 in [32 lw, 32 lw + 32))
      // or columns (B: p1 in [16 b, 16 b + 16), b = lw - 4)?  Node j reaches
      // [o_j, o_j + W).  With the binning's 16 x 16 sub-tile order a batch's window starts
      // lie within a few rows and columns, so most operand warps of a batch write zeros
      // without evaluating taps (every tap of such a warp is zero, so for finite samples
      // the operands are the same).  The test is warp-uniform.
      bool reached;
      {
        const uint32_t mo = offs[lane & (kTcK - 1)];
        const bool has = lane < kTcK && mo != 0xffffffffu;
        const uint32_t o = is_a ? (mo & MASK) : ((mo >> SH) & MASK);
        const uint32_t omin = __reduce_min_sync(0xffffffffu, has ? o : 0xffffffffu);
        const uint32_t oend = __reduce_max_sync(0xffffffffu, has ? o + (uint32_t)W : 0u);  // 0: no node
        const int r0 = is_a ? 32 * lw : 16 * (lw - kT2AWarps), rn = is_a ? 32 : 16;
        reached = oend != 0u && (int)omin < r0 + rn && (int)oend > r0;
      }
      if (is_a) {
        tc::fence_after_sync();
        uint32_t hi[8], lo[8];
        if (reached) {
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            float v[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const int j = 2 * c + u;
              const uint32_t off = offs[j];
              const int l = p0 - (int)(off & MASK);  // no node: l < 0, a zero tap
              v[u] = tc_tap<WIN>(frs[j].x, mf, l, W, k0) * kTcScaleA;
            }
            tc_split2_f16(make_float2(v[0], v[1]), hi[c], lo[c]);
          }
        } else {
#pragma unroll
          for (int c = 0; c < 8; ++c) hi[c] = lo[c] = 0u;
        }
        const uint32_t ta = tmem + ((uint32_t)(32 * lw) << 16) + kT2ACol0 + st * 16u;
        tc::tmem_st8(ta, hi);
        tc::tmem_st8(ta + 8u, lo);
        tc::tmem_st_wait();
        tc::fence_before_sync();
      } else {
        const float2* val = reinterpret_cast<const float2*>(sl + kT2SlotVal);
        uint4 rh, rl, ih, il;
        if (reached) {
          float re[8], im[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int j = 8 * h + u;
            const uint32_t off = offs[j];
            const int l = off == 0xffffffffu ? -1 : p1 - (int)((off >> SH) & MASK);
            const float w = tc_tap<WIN>(frs[j].y, mf, l, W, k1) * bscale;
            const float2 v = val[j];
            re[u] = w * v.x;
            im[u] = w * v.y;
          }
          tc_split8_f16(re, rh, rl);
          tc_split8_f16(im, ih, il);
        } else {
          rh = rl = ih = il = make_uint4(0u, 0u, 0u, 0u);
        }
        unsigned char* bst = smem + L.b_off + st * 2u * kT2BBytes;
        const int r0 = 2 * p1;  // rows r0 (Re) and r0 + 1 (Im): same 8-row group
        const uint32_t o0 = tc_elem_off(r0 >> 3, r0 & 7, h), o1 = tc_elem_off(r0 >> 3, (r0 & 7) + 1, h);
        *reinterpret_cast<uint4*>(bst + o0) = rh;
        *reinterpret_cast<uint4*>(bst + kT2BBytes + o0) = rl;
        *reinterpret_cast<uint4*>(bst + o1) = ih;
        *reinterpret_cast<uint4*>(bst + kT2BBytes + o1) = il;
        tc::fence_proxy_async_smem();  // generic-proxy operand writes -> tensor core
      }
      tc::mbar_arrive_warp(&full[st]);
      tc::mbar_arrive_warp(&rec_empty[r]);
    }
    if (!healthy) *abort_flag = 1;
  } else if (warp == kT2MmaWarp) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sb0 = tc::smem_u32(smem + L.b_off);
      const uint64_t d_bh = tc::smem_desc(sb0, kTcLBO, kTcSBO);
      const uint64_t d_bl = tc::smem_desc(sb0 + kT2BBytes, kTcLBO, kTcSBO);
      const uint64_t d_stage = (uint64_t)((2u * kT2BBytes) >> 4);
      const uint32_t idesc = tc::idesc_f16(128, kT2N);
      uint32_t gb = 0, st = 0, cyc = 0, k = 0;
      int4 nxt = (int)blockIdx.x < num_items ? bins.items[blockIdx.x] : make_int4(0, 0, 0, 0);
      for (int it = blockIdx.x; it < num_items && healthy; it += G, ++k) {
        const int4 item = nxt;
        if (it + G < num_items) nxt = bins.items[it + G];
        const uint32_t set = k & 1u;
        if (k >= 2) {  // accumulator set `set` read out (item k - 2)
          healthy = tc::mbar_wait_bounded(&acc_empty[set], ((k - 2u) >> 1) & 1u, kTcPolls);
          tc::fence_after_sync();
        }
        const uint32_t d = tmem + set * kT2N;
        const int nbatch = (item.z - item.y + kTcK - 1) / kTcK;
        for (int b = 0; b < nbatch && healthy; ++b, ++gb) {
          healthy = tc::mbar_wait_spin(&full[st], cyc & 1u, kTcPolls, kT2Spin);
          if (!healthy) break;
          tc::fence_after_sync();
          const uint64_t so = (uint64_t)st * d_stage;
          const uint32_t ta = tmem + kT2ACol0 + st * 16u;
          tc::mma_f16_ta(d, ta, d_bh + so, idesc, b > 0 ? 1u : 0u);  // K = 16: the whole batch
          tc::mma_f16_ta(d, ta, d_bl + so, idesc, 1u);
          tc::mma_f16_ta(d, ta + 8u, d_bh + so, idesc, 1u);
          tc::mma_commit(&empty[st]);
          if (b == nbatch - 1) tc::mma_commit(&acc_full[set]);
          if (++st == kT2Stages) {
            st = 0;
            ++cyc;
          }
        }
        if (!healthy) *abort_flag = 1;
      }
      // the last commit of each stage is waited by nobody else; no arrival may land after exit
      for (uint32_t i = 1; i <= (uint32_t)kT2Stages && i <= gb; ++i) {
        const uint32_t bb = gb - i;
        healthy &= tc::mbar_wait_bounded(&empty[bb % kT2Stages], (bb / kT2Stages) & 1u, kTcPolls);
      }
    }
    __syncwarp();
  } else if (warp >= kT2EpiWarp0 && warp < kT2EpiWarp0 + 4) {
    // ======================= epilogue warps =======================
    // Per work item: thread (lane quarter q, lane) reads TMEM row p0 = 32 q + lane of the
    // item's accumulator set into its own staging row, releases the set, and adds the row
    // to grid row a0 + p0: columns a1 .. a1 + E1 - 1, one contiguous run or two when they
    // wrap the row end, each as one bulk FP32 reduction (runs rounded up to 16 bytes with
    // the zero column past the padded tile); odd row lengths, rows shorter than the tile
    // and 8-byte aligned grids take 8- or 16-byte atomics.
    const int q = warp & 3, ep0 = 32 * q + lane;
    const int64_t n0 = geo.n[0], n1 = geo.n[1];
    const bool one_wrap = n1 >= E1;
    const float unscale = 1.f / (kTcScaleA * tc_scale_b(bins, (float)geo.norm));  // a power of two: exact
    const bool pairs = (n1 & 1) == 0 && (reinterpret_cast<uintptr_t>(g) & 15u) == 0 && (geo.ntot & 1) == 0;
    float* const srow = reinterpret_cast<float*>(smem + L.stg_off) + ep0 * kT2StgStride;
    uint32_t k = 0;
    int4 nxt = (int)blockIdx.x < num_items ? bins.items[blockIdx.x] : make_int4(0, 0, 0, 0);
    for (int it = blockIdx.x; it < num_items; it += G, ++k) {
      const int4 item = nxt;
      if (it + G < num_items) nxt = bins.items[it + G];
      const uint32_t set = k & 1u;
      healthy = tc::mbar_wait_warp(&acc_full[set], (k >> 1) & 1u, kTcPolls);
      if (!healthy) {
        *abort_flag = 1;
        break;
      }
      tc::bulk_wait_read();  // the previous item's reductions have read this thread's row
      tc::fence_after_sync();
      // tcgen05.ld is warp-collective: a warp with any tile row reads all 32 of its lanes
      // (the rows past E0 are zeros, staged and never reduced)
      if (32 * q < E0) {
        const uint32_t acc = tmem + set * kT2N + ((uint32_t)(32 * q) << 16);
#pragma unroll
        for (int c = 0; c < kT2N / 16; ++c) {
          float v[16];
          tc::tmem_ld16(acc + (uint32_t)(c * 16), v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int u = 0; u < 4; ++u)
            *reinterpret_cast<float4*>(srow + 16 * c + 4 * u) =
                make_float4(v[4 * u] * unscale, v[4 * u + 1] * unscale, v[4 * u + 2] * unscale, v[4 * u + 3] * unscale);
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive_warp(&acc_empty[set]);
      if (ep0 < E0) {
        const TileOrigin o = decode_tile<2>(geo, tl, item.x);
        float2* const rowa = g + o.inst * geo.ntot + wrap_up(o.a[0] + ep0, n0) * n1;  // grid row start
        const int kw = (int)(n1 - o.a[1] < 128 ? n1 - o.a[1] : 128);  // columns before the row end (capped > E1)
        bool done = false;
        if (one_wrap && (n1 & 1) == 0) {
          // run 1: columns [0, c1) at a1 + p1; run 2: columns [kw, E1) at p1 - kw (wrapped)
          tc::fence_proxy_async_smem();  // staged row -> bulk-copy engine
          const uint32_t s0 = tc::smem_u32(srow);
          const int c1 = E1 < kw ? E1 : kw;
          const uint32_t b1 = (uint32_t)((c1 + 1) & ~1) * 8u;
          const uint32_t b2 = kw < E1 ? (uint32_t)((E1 - kw + 1) & ~1) * 8u : 0u;
          float2* const dst1 = rowa + o.a[1];
          done = ((reinterpret_cast<uintptr_t>(dst1) | s0) & 15u) == 0u &&
                 ((reinterpret_cast<uintptr_t>(rowa) | (s0 + (uint32_t)kw * 8u)) & 15u) == 0u;
          if (done) {
            tc::bulk_reduce_add_f32(dst1, s0, b1);
            if (b2) tc::bulk_reduce_add_f32(rowa, s0 + (uint32_t)kw * 8u, b2);
            tc::bulk_commit();
          }
        }
        for (int p = 0; p < E1 && !done; p += 2) {
          const float4 w = *reinterpret_cast<const float4*>(srow + 2 * p);
          const int64_t c0 = wrap_up(o.a[1] + p, n1);
          if (p + 1 < E1 && pairs && c0 + 1 < n1) {  // pair (p, p + 1) 16-byte aligned and not split by the wrap
            if (w.x != 0.f || w.y != 0.f || w.z != 0.f || w.w != 0.f)
              atomicAdd(reinterpret_cast<float4*>(rowa + c0), w);
          } else {
            if (w.x != 0.f || w.y != 0.f) atomicAdd(rowa + c0, make_float2(w.x, w.y));
            if (p + 1 < E1 && (w.z != 0.f || w.w != 0.f))
              atomicAdd(rowa + wrap_up(o.a[1] + p + 1, n1), make_float2(w.z, w.w));
          }
        }
      }
      __syncwarp();  // the warp reconverges before the next item's collective TMEM reads
    }
    tc::bulk_wait_all();  // every reduction complete before the CTA's shared memory goes
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (!healthy) atomicExch(bins.status, 2);
}

}  // namespace cg
