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
// Unlike 3D, both operands are one tap table wide: a node costs 128 A entries and 160 B
// entries (against W^2 <= 256 taps), and the tensor core does the W^2 multiply-adds.  The
// taps come from per-node tables in which tap l of a node sits at index kT2Zero + l of a
// row of kT2Pad floats that is zero elsewhere, so the A thread of row p0 reads
// w0[j][kT2Zero + p0 - o0_j] and the B thread of column p1 reads w1[j][kT2Zero + p1 - o1_j]
// without a bounds test (rows and columns outside the window read zeros).
//
// Warp roles (16 warps): A warps 0-3 (warp w writes TMEM lanes 32 w .. 32 w + 31, one row
// p0 per thread, its hi and lo halves with tcgen05.st), B warps 4-8 (thread t of 160:
// rows 2 p1 and 2 p1 + 1 of B, nodes 8 h .. 8 h + 7, p1 = t / 2, h = t % 2, into the
// shared-memory operand stage), table warps 9-10 (node records through a cp.async ring,
// then the taps of half the window each, lane = node and dimension), the MMA warp 11
// (lane 0) and epilogue warps 12-15 (TMEM lane quarter warp % 4).  The table buffers are
// double-buffered (tab_full / tab_empty), the operands four stages deep (full / empty),
// the accumulators double-buffered in tensor memory (acc_full / acc_empty): while the
// epilogue reads one work item's tile out and adds it to the grid as bulk FP32 reductions
// (cp.reduce.async.bulk, one or two per row), the MMAs of the next item accumulate into
// the other set.  Every mbarrier wait is bounded; a wait that gives up sets the plan's
// device status flag, after which the kernel drains (bounded), frees its tensor memory and
// returns.
#pragma once

#include <cuda_fp16.h>

#include "kernels_spread_tc.cuh"

namespace cg {

constexpr int kT2MaxT0 = 64;               // E0 = T0 + W - 1 <= 128 rows (M = 128)
constexpr int kT2N = 160;                  // MMA N: 2 E1 <= 158 columns (p1, re|im), padded
constexpr int kT2AWarps = 4;
constexpr int kT2BWarps = 5;               // 160 threads: (p1 < 80, node half)
constexpr int kT2TabWarp0 = kT2AWarps + kT2BWarps;  // warps 9, 10
constexpr int kT2MmaWarp = kT2TabWarp0 + 2;         // warp 11
constexpr int kT2EpiWarp0 = kT2MmaWarp + 1;         // warps 12-15: lane quarters 0-3
constexpr int kT2Threads = (kT2EpiWarp0 + 4) * 32;
constexpr int kT2Stages = 4;
constexpr int kT2Pad = 193;                // floats per node and dimension in the tap tables (odd)
constexpr int kT2Zero = 64;                // table index of tap 0 (p0 - o0 >= -63)
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
  uint32_t rec_off;   // kTcRing record slots
  uint32_t tab_off;   // 2 x table buffer
  uint32_t tab_bytes; // w0 [16][kT2Pad], w1 [16][kT2Pad] floats, then samples [16] float2, offsets [16] int2
  uint32_t bar_off;   // full[4], empty[4], acc_full[2], acc_empty[2], tab_full[2], tab_empty[2];
                      // tensor-memory base, abort flag
  uint32_t stg_off;   // [128][kT2StgStride] accumulator rows staged for the reductions
  uint32_t total;
};

__host__ __device__ constexpr T2Layout t2_layout() {
  T2Layout L{};
  L.b_off = 0;
  L.rec_off = kT2Stages * 2u * kT2BBytes;
  L.tab_off = L.rec_off + kTcRing * kT2SlotBytes;
  L.tab_bytes = 2u * kTcK * kT2Pad * 4u + kTcK * 8u + kTcK * 8u;
  L.bar_off = (L.tab_off + 2u * L.tab_bytes + 15u) & ~15u;
  L.stg_off = L.bar_off + 16u * 8u + 16u;
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
  uint64_t* tab_full = full + 12;                                   // [2] table buffer b written
  uint64_t* tab_empty = full + 14;                                  // [2] table buffer b read
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 128);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + L.bar_off + 132);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  // the tap tables are zero outside the taps, which the table warps rewrite per batch
  for (int i = tid; i < (int)(2u * L.tab_bytes / 4u); i += kT2Threads)
    reinterpret_cast<float*>(smem + L.tab_off)[i] = 0.f;
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) {
      tc::mbar_init(&full[i], kT2AWarps + kT2BWarps);  // one arrival per operand warp
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&acc_full[i], 1);
      tc::mbar_init(&acc_empty[i], 4);                 // one arrival per epilogue warp
      tc::mbar_init(&tab_full[i], 2);                  // one arrival per table warp
      tc::mbar_init(&tab_empty[i], kT2AWarps + kT2BWarps);
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

  auto tab_w = [&](uint32_t b, int dim) {
    return reinterpret_cast<float*>(smem + L.tab_off + b * L.tab_bytes) + dim * kTcK * kT2Pad;
  };
  auto tab_val = [&](uint32_t b) {
    return reinterpret_cast<float2*>(smem + L.tab_off + b * L.tab_bytes + 2u * kTcK * kT2Pad * 4u);
  };
  auto tab_off = [&](uint32_t b) {
    return reinterpret_cast<int2*>(smem + L.tab_off + b * L.tab_bytes + 2u * kTcK * kT2Pad * 4u + kTcK * 8u);
  };

  // Every role walks items c, c + G, ... (CTA c) in batches of kTcK nodes; batch gb
  // (counted across the CTA's items) uses operand stage gb % 4 in its cycle gb / 4, table
  // buffer gb & 1 and record slot gb % kTcRing; item k of the CTA accumulates into set k & 1.
  if (warp >= kT2TabWarp0 && warp < kT2MmaWarp) {
    // ======================= table warps =======================
    const int half = warp - kT2TabWarp0;
    const float* sfrac = reinterpret_cast<const float*>(bins.sfrac);
    const float2* fperm = reinterpret_cast<const float2*>(bins.fperm);
    const float norm = (float)geo.norm;
    const float bscale = norm * tc_scale_b(bins, norm);
    const float mf = (float)geo.m;
    const int j = lane & (kTcK - 1), dim = lane >> 4;
    const TapK kd = tap_k<WIN>(geo, dim);
    const float sc = dim == 0 ? kTcScaleA : 1.f;  // A = w0 2^10
    constexpr int kHalf = W / 2;
    // the records of one batch into ring slot `slot` (warp kT2TabWarp0 only)
    auto load = [&](const TcCursor& c, int slot) {
      unsigned char* sl = smem + L.rec_off + slot * kT2SlotBytes;
      const int base = c.item.y + c.b * kTcK, n = min(kTcK, c.item.z - base);
      if (lane < kTcK) {
        if (lane < n) {
          cp_async4(sl + kT2SlotOff + lane * 4, bins.soff + base + lane);
          cp_async8(sl + kT2SlotVal + lane * 8, fperm + base + lane);
        } else {
          reinterpret_cast<int*>(sl + kT2SlotOff)[lane] = -1;  // no node: zero taps, zero sample
          reinterpret_cast<float2*>(sl + kT2SlotVal)[lane] = make_float2(0.f, 0.f);
        }
      }
      if (lane < 2 * n) cp_async4(sl + kT2SlotFrac + lane * 4, sfrac + (int64_t)base * 2 + lane);
      else reinterpret_cast<float*>(sl + kT2SlotFrac)[lane] = 0.f;
    };
    TcCursor cc, lc;
    tc_cursor_init(cc, bins, num_items);
    lc = cc;
    if (half == 0) {
#pragma unroll
      for (int d = 0; d < kTcAhead; ++d) {
        if (lc.it < num_items) {
          load(lc, d);
          tc_cursor_step(lc, bins, num_items);
        }
        cp_async_commit();
      }
    }
    uint32_t gb = 0;
    for (; cc.it < num_items; tc_cursor_step(cc, bins, num_items), ++gb) {
      const uint32_t tb = gb & 1u;
      bool fail = false;
      if (half == 0) cp_async_wait_group<kTcAhead - 1>();  // the records of batch gb have landed
      // table buffer tb free once the operand warps have read batch gb - 2 from it
      if (gb >= 2 && lane == 0)
        fail = !tc::mbar_wait_bounded(&tab_empty[tb], ((gb - 2u) >> 1) & 1u, kTcPolls);
      if (tc::named_sync_or(3, 64, fail || *abort_flag != 0)) {  // records visible to both table warps
        healthy = false;
        break;
      }
      const unsigned char* sl = smem + L.rec_off + (gb % kTcRing) * kT2SlotBytes;
      const uint32_t off = reinterpret_cast<const uint32_t*>(sl + kT2SlotOff)[j];
      const bool node = off != 0xffffffffu;
      // taps of half `half` of the window: l = half kHalf .. (half + 1) kHalf - 1
      {
        const float fr = reinterpret_cast<const float*>(sl + kT2SlotFrac)[j * 2 + dim];
        float* const row = tab_w(tb, dim) + j * kT2Pad + kT2Zero;
#pragma unroll
        for (int i = 0; i < kHalf; ++i) {
          const int l = half * kHalf + i;
          row[l] = node ? tc_tap<WIN>(fr, mf, l, W, kd) * sc : 0.f;
        }
      }
      if (half == 0 && lane < kTcK) {
        const float2 v = reinterpret_cast<const float2*>(sl + kT2SlotVal)[j];
        tab_val(tb)[j] = make_float2(v.x * bscale, v.y * bscale);
        // window starts inside the tile by construction; clamped so that table reads
        // always stay inside the padded rows
        const int o0 = node ? min((int)(off & MASK), kT2Zero - 1) : 0;
        const int o1 = node ? min((int)((off >> SH) & MASK), kT2Zero - 1) : 0;
        tab_off(tb)[j] = make_int2(o0, o1);
      }
      // the next record load into the slot batch gb - 1 used (both table warps are past it)
      if (half == 0) {
        if (lc.it < num_items) {
          load(lc, (int)((gb + kTcAhead) % kTcRing));
          tc_cursor_step(lc, bins, num_items);
        }
        cp_async_commit();
      }
      tc::mbar_arrive_warp(&tab_full[tb]);
    }
    if (half == 0) cp_async_wait_group<0>();
    if (!healthy) *abort_flag = 1;
  } else if (warp < kT2AWarps + kT2BWarps) {
    // ======================= operand warps: A (0-3) and B (4-8) =======================
    const bool is_a = warp < kT2AWarps;
    const int p0 = 32 * warp + lane;                      // A: row (TMEM lane)
    const int bt = 32 * (warp - kT2AWarps) + lane;       // B: task
    const int p1 = bt >> 1, h = bt & 1;
    uint32_t gb = 0, st = 0, cyc = 0;
    TcCursor cc;
    tc_cursor_init(cc, bins, num_items);
    for (; cc.it < num_items; tc_cursor_step(cc, bins, num_items), ++gb) {
      const uint32_t tb = gb & 1u;
      bool ok = tc::mbar_wait_warp(&tab_full[tb], (gb >> 1) & 1u, kTcPolls);
      if (ok && cyc > 0) ok = tc::mbar_wait_warp(&empty[st], (cyc - 1u) & 1u, kTcPolls);
      if (!ok || *abort_flag != 0) {
        healthy = false;
        break;
      }
      const int2* offs = tab_off(tb);
      if (is_a) {
        tc::fence_after_sync();
        const float* w0 = tab_w(tb, 0) + kT2Zero + p0;
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float2 v =
              make_float2(w0[(2 * c) * kT2Pad - offs[2 * c].x], w0[(2 * c + 1) * kT2Pad - offs[2 * c + 1].x]);
          tc_split2_f16(v, hi[c], lo[c]);
        }
        const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + kT2ACol0 + st * 16u;
        tc::tmem_st8(ta, hi);
        tc::tmem_st8(ta + 8u, lo);
        tc::tmem_st_wait();
        tc::fence_before_sync();
      } else {
        const float* w1 = tab_w(tb, 1) + kT2Zero + p1;
        const float2* val = tab_val(tb);
        float re[8], im[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int jj = 8 * h + u;
          const float w = w1[jj * kT2Pad - offs[jj].y];
          const float2 v = val[jj];
          re[u] = w * v.x;
          im[u] = w * v.y;
        }
        uint4 rh, rl, ih, il;
        tc_split8_f16(re, rh, rl);
        tc_split8_f16(im, ih, il);
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
      tc::mbar_arrive_warp(&tab_empty[tb]);
      if (++st == kT2Stages) {
        st = 0;
        ++cyc;
      }
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
          healthy = tc::mbar_wait_bounded(&full[st], cyc & 1u, kTcPolls);
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
  } else {
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
