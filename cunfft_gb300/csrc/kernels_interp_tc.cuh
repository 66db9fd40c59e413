// kernels_interp_tc.cuh -- 3D FP32 interpolation on the tensor cores (tcgen05, 3xTF32).
//
// Same work items, tiles and weights as k_interp (kernels_grid.cuh).  For a tile
// with padded extents E0 x E1 x E2 and a batch of up to 128 of its nodes,
//     f_j = norm sum_{p0, p1} w0_j[p0 - o0_j] w1_j[p1 - o1_j] H[j, (p0, p1)],
//     H[j, (p0, p1, re|im)] = sum_{p2} w2_j[p2 - o2_j] G[(p0, p1), p2] (re|im)
// and H is the product D = A B^T of
//     A[j, p2]              = w2_j[p2 - o2_j]                  (128 nodes x 32 columns)
//     B[(p0, p1, re|im), p2] = Re|Im G[p0, p1, p2]             (the tile, K = p2)
// computed in chunks of kItCh planes so that a chunk's 2 E1 kItCh columns fit one
// MMA (N <= 256) and two chunks fit tensor memory.  D lives in tensor memory with
// node j in lane j, so the thread that owns node j finishes the w0 (x) w1 sum over
// its window from its own lane, chunk by chunk, in registers.
//
// Warp roles: 8 builder warps load the tile chunk by chunk from the grid (L2 / HBM),
// split it into TF32 hi + lo parts and store it in K-major core-matrix layout
// (double-buffered); one MMA warp issues hi*hi + hi*lo + lo*hi per k-step of 8
// columns into one of two tensor-memory buffers; 4 node warps (lane quarters) build
// A from their nodes' taps and reduce D.  Hand-offs are mbarriers; every wait is
// bounded and a wait that gives up sets the plan's device status flag.
#pragma once

#include "kernels_grid.cuh"
#include "tc_sm100.cuh"

namespace cg {

constexpr int kItMaxT0 = 16;       // outer tile extent limit (E0 <= 31 planes)
constexpr int kItK = 32;           // K: innermost tile columns p2 (E2 <= 31), padded
constexpr int kItNodes = 128;      // nodes per batch (MMA M)
constexpr int kItBuilders = 8;     // warps loading tile chunks
constexpr int kItMmaWarp = kItBuilders;
constexpr int kItNodeWarp0 = kItBuilders + 1;  // 4 node warps: lane quarter = warp % 4
constexpr int kItThreads = (kItBuilders + 1 + 4) * 32;
constexpr uint32_t kItLBO = 128;               // core matrices along K
constexpr uint32_t kItSBOA = 1024;             // A: 8-row groups (32 K values = 8 core matrices)
constexpr uint32_t kItSBOB = 1040;             // B: 8-row groups, shifted 16 bytes: conflict-free stores
constexpr uint32_t kItPolls = 1u << 20;        // mbarrier polls (<= 1 us each) before giving up

__host__ __device__ constexpr int it_e1(int W) { return fixed_t_mid(3, W) + W - 1; }
__host__ __device__ constexpr int it_ch(int W) { return 256 / (2 * it_e1(W)); }               // planes per chunk
__host__ __device__ constexpr int it_ncol(int W) { return it_ch(W) * 2 * it_e1(W); }          // used D columns
__host__ __device__ constexpr int it_n(int W) { return (it_ncol(W) + 15) / 16 * 16; }          // MMA N
__host__ __device__ constexpr int it_pairs_pad(int W) { return (it_ch(W) * it_e1(W) + 7) / 8 * 8; }

__host__ __device__ constexpr bool interp_tc_ok(int d, int W, int T0, int64_t n2) {
  return d == 3 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kItMaxT0 && n2 >= 4 && n2 % 4 == 0;
}

// Shared-memory layout (byte offsets; host and device agree).
struct ItLayout {
  uint32_t a_bytes;    // one A part: 16 row groups
  uint32_t b_bytes;    // one B part: N / 8 row groups
  uint32_t a_off;      // 2 buffers x (A hi, A lo)
  uint32_t b_off;      // 2 buffers x (B hi, B lo)
  uint32_t bar_off;    // afull[2], bfull[2], bempty[2], tfull[2], tempty[2]; tensor-memory base
  uint32_t total;
};

__host__ __device__ inline ItLayout it_layout(int W) {
  ItLayout L{};
  L.a_bytes = 16u * kItSBOA;
  L.b_bytes = (uint32_t)(it_n(W) / 8) * kItSBOB;
  L.a_off = 0;
  L.b_off = 4u * L.a_bytes;
  L.bar_off = (L.b_off + 4u * L.b_bytes + 15u) & ~15u;
  L.total = L.bar_off + 96u;
  return L;
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
__global__ void __launch_bounds__(kItThreads, 1) k_interp_tc(const float2* __restrict__ g, float2* __restrict__ f,
                                                             Geom geo, Tiling tl, Bins bins) {
  constexpr int E1 = it_e1(W), CH = it_ch(W), NCOL = it_ncol(W), N = it_n(W);
  constexpr int E0MAX = kItMaxT0 + W - 1;
  constexpr int MAXCH = (E0MAX + CH - 1) / CH;
  constexpr int PPAD = it_pairs_pad(W);
  constexpr int BIT = (PPAD + kItBuilders * 8 - 1) / (kItBuilders * 8);  // pair blocks per builder warp
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  static_assert(NCOL <= 256 && N <= 256 && 2 * N <= 512, "two chunk accumulators must fit tensor memory");
  static_assert(fixed_t_last(3, W) + W - 1 <= kItK, "innermost padded extent must fit K");
  extern __shared__ __align__(16) unsigned char smem[];
  const ItLayout L = it_layout(W);
  uint64_t* afull = reinterpret_cast<uint64_t*>(smem + L.bar_off);  // [2] A of the batch built
  uint64_t* bfull = afull + 2;                                       // [2] tile chunk built
  uint64_t* bempty = afull + 4;                                      // [2] MMAs of the chunk complete
  uint64_t* tfull = afull + 6;                                       // [2] accumulator complete
  uint64_t* tempty = afull + 8;                                      // [2] accumulator read out
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 80);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int E0 = tl.E[0];
  const int nch = (E0 + CH - 1) / CH;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&afull[i], 4);             // one arrival per node warp
      tc::mbar_init(&bfull[i], kItBuilders);   // one arrival per builder warp
      tc::mbar_init(&bempty[i], 1);
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], 4);            // one arrival per node warp
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
  // sequence) uses tile buffer and accumulator gc & 1 in their cycle gc >> 1.
  if (warp < kItBuilders) {
    // ======================= builder warps: tile chunks =======================
    const int pl8 = lane & 7, qq = lane >> 3;
    const int64_t n0 = geo.n[0], n1 = geo.n[1], n2 = geo.n[2];
    uint32_t gc = 0;
    for (int it = blockIdx.x; it < num_items; it += G) {
      const int4 item = bins.items[it];
      const TileOrigin o = decode_tile<3>(geo, tl, item.x);
      const float2* gi = g + o.inst * geo.ntot;
      const int nbatch = (item.z - item.y + kItNodes - 1) / kItNodes;
      for (int bt = 0; bt < nbatch; ++bt) {
        for (int c = 0; c < nch; ++c, ++gc) {
          const uint32_t buf = gc & 1u;
          if (gc >= 2) healthy &= tc::mbar_wait_warp(&bempty[buf], ((gc >> 1) - 1u) & 1u, kItPolls);
          unsigned char* bh = smem + L.b_off + buf * 2u * L.b_bytes;
          unsigned char* bl = bh + L.b_bytes;
          const int ps = c * CH, np = min(CH, E0 - ps);
          // item (pair, quad): pair = (plane, row) of the chunk, quad = 4 consecutive p2;
          // all of this thread's loads go out before the first conversion
          float4 v[BIT][2][2];
#pragma unroll
          for (int i = 0; i < BIT; ++i) {
            const int pair = warp * 8 + i * kItBuilders * 8 + pl8;
            const int pl = pair / E1, p1 = pair - pl * E1;
            const bool on = pl < np;
            int64_t rowg = 0;
            if (on) rowg = (wrap_up(o.a[0] + ps + pl, n0) * n1 + wrap_up(o.a[1] + p1, n1)) * n2;
#pragma unroll
            for (int qh = 0; qh < 2; ++qh) {
              const int qd = qh * 4 + qq;  // p2 = 4 qd .. 4 qd + 3 (never straddles the wrap: n2 % 4 == 0)
              v[i][qh][0] = v[i][qh][1] = make_float4(0.f, 0.f, 0.f, 0.f);
              if (on) {
                const float4* src = reinterpret_cast<const float4*>(gi + rowg + wrap_up(o.a[2] + 4 * qd, n2));
                v[i][qh][0] = src[0];
                v[i][qh][1] = src[1];
              }
            }
          }
#pragma unroll
          for (int i = 0; i < BIT; ++i) {
            const int pair = warp * 8 + i * kItBuilders * 8 + pl8;
            if (pair < PPAD) {
#pragma unroll
              for (int qh = 0; qh < 2; ++qh) {
                const int qd = qh * 4 + qq;
                const float4 v0 = v[i][qh][0], v1 = v[i][qh][1];
                const float4 re = make_float4(v0.x, v0.z, v1.x, v1.z), im = make_float4(v0.y, v0.w, v1.y, v1.w);
                float4 h, l;
                const int nr = 2 * pair;
                const uint32_t ore = (uint32_t)(nr >> 3) * kItSBOB + (uint32_t)qd * kItLBO + (uint32_t)(nr & 7) * 16u;
                const uint32_t oim = ore + 16u;  // row 2 pair + 1: same group (nr even)
                tc_split4(re, h, l);
                *reinterpret_cast<float4*>(bh + ore) = h;
                *reinterpret_cast<float4*>(bl + ore) = l;
                tc_split4(im, h, l);
                *reinterpret_cast<float4*>(bh + oim) = h;
                *reinterpret_cast<float4*>(bl + oim) = l;
              }
            }
          }
          tc::fence_proxy_async_smem();
          tc::mbar_arrive_warp(&bfull[buf]);
        }
      }
    }
  } else if (warp == kItMmaWarp) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sa = tc::smem_u32(smem + L.a_off), sb = tc::smem_u32(smem + L.b_off);
      const uint64_t d_abuf = (uint64_t)((2u * L.a_bytes) >> 4);  // A buffer 1 = buffer 0 + d_abuf
      const uint64_t d_ah = tc::smem_desc(sa, kItLBO, kItSBOA);
      const uint64_t d_al = tc::smem_desc(sa + L.a_bytes, kItLBO, kItSBOA);
      const uint64_t d_bh = tc::smem_desc(sb, kItLBO, kItSBOB);
      const uint64_t d_bl = tc::smem_desc(sb + L.b_bytes, kItLBO, kItSBOB);
      const uint64_t d_buf = (uint64_t)((2u * L.b_bytes) >> 4);  // buffer 1 = buffer 0 + d_buf
      const uint32_t idesc = tc::idesc_tf32(128, N);
      uint32_t gc = 0, gbt = 0;
      for (int it = blockIdx.x; it < num_items; it += G) {
        const int4 item = bins.items[it];
        const int nbatch = (item.z - item.y + kItNodes - 1) / kItNodes;
        for (int bt = 0; bt < nbatch; ++bt, ++gbt) {
          const uint32_t ab = gbt & 1u;
          healthy &= tc::mbar_wait_bounded(&afull[ab], (gbt >> 1) & 1u, kItPolls);
          const uint64_t ao = ab ? d_abuf : 0ull;
          for (int c = 0; c < nch; ++c, ++gc) {
            const uint32_t buf = gc & 1u;
            healthy &= tc::mbar_wait_bounded(&bfull[buf], (gc >> 1) & 1u, kItPolls);
            if (gc >= 2) healthy &= tc::mbar_wait_bounded(&tempty[buf], ((gc >> 1) - 1u) & 1u, kItPolls);
            tc::fence_after_sync();
            const uint32_t d = tmem + buf * 256u;
            const uint64_t bo = buf ? d_buf : 0ull;
#pragma unroll
            for (int ks = 0; ks < kItK / 8; ++ks) {
              const uint64_t ko = (uint64_t)((ks * 2 * kItLBO) >> 4);
              tc::mma_tf32(d, d_ah + ao + ko, d_bh + bo + ko, idesc, ks > 0 ? 1u : 0u);
              tc::mma_tf32(d, d_ah + ao + ko, d_bl + bo + ko, idesc, 1u);
              tc::mma_tf32(d, d_al + ao + ko, d_bh + bo + ko, idesc, 1u);
            }
            tc::mma_commit(&bempty[buf]);
            tc::mma_commit(&tfull[buf]);
          }
        }
      }
      // the last chunk commits are waited by the node warps; the last bempty arrivals by nobody
      if (gc >= 1) healthy &= tc::mbar_wait_bounded(&bempty[(gc - 1) & 1u], ((gc - 1) >> 1) & 1u, kItPolls);
      if (gc >= 2) healthy &= tc::mbar_wait_bounded(&bempty[(gc - 2) & 1u], ((gc - 2) >> 1) & 1u, kItPolls);
    }
    __syncwarp();
  } else {
    // ======================= node warps: A, then the w0 (x) w1 reduction =======================
    // Records are loaded two batches ahead; A of batch gbt + 1 is built at the start
    // of batch gbt (its buffer's previous batch, gbt - 1, is complete: this thread
    // waited for all of its accumulators), so the MMAs never wait for A.
    const int q = warp & 3;             // tensor-memory lane quarter
    const int slot = 32 * q + lane;     // node slot in the batch = TMEM lane = A row
    const float norm = (float)geo.norm;
    const float mf = (float)geo.m;
    const TapK k0 = tap_k<WIN>(geo, 0), k1 = tap_k<WIN>(geo, 1), k2 = tap_k<WIN>(geo, 2);
    auto build_a = [&](const ItRec& r, uint32_t ab) {
      unsigned char* ah = smem + L.a_off + ab * 2u * L.a_bytes;
      unsigned char* al = ah + L.a_bytes;
      const int o2 = (int)(r.off >> (2 * SH));
#pragma unroll
      for (int k4 = 0; k4 < kItK / 4; ++k4) {
        float4 v;
        v.x = tc_tap<WIN>(r.fr2, mf, 4 * k4 + 0 - o2, W, k2);
        v.y = tc_tap<WIN>(r.fr2, mf, 4 * k4 + 1 - o2, W, k2);
        v.z = tc_tap<WIN>(r.fr2, mf, 4 * k4 + 2 - o2, W, k2);
        v.w = tc_tap<WIN>(r.fr2, mf, 4 * k4 + 3 - o2, W, k2);
        float4 h, l;
        tc_split4(v, h, l);
        const uint32_t oa = (uint32_t)(slot >> 3) * kItSBOA + (uint32_t)k4 * kItLBO + (uint32_t)(slot & 7) * 16u;
        *reinterpret_cast<float4*>(ah + oa) = h;
        *reinterpret_cast<float4*>(al + oa) = l;
      }
      tc::fence_proxy_async_smem();
      tc::mbar_arrive_warp(&afull[ab]);
    };
    ItCursor c0, c1, c2;  // batches gbt, gbt + 1, gbt + 2
    it_cursor_init(c0, bins, num_items);
    c1 = c0;
    it_cursor_step(c1, bins, num_items);
    c2 = c1;
    it_cursor_step(c2, bins, num_items);
    ItRec rc = it_load_rec(c0, num_items, slot, bins), rn = it_load_rec(c1, num_items, slot, bins);
    if (c0.it < num_items) build_a(rc, 0u);
    uint32_t gc = 0, gbt = 0;
    for (; c0.it < num_items; ++gbt) {
      if (c1.it < num_items) build_a(rn, (gbt + 1u) & 1u);
      const ItRec rnn = it_load_rec(c2, num_items, slot, bins);
      const int o0 = (int)(rc.off & MASK), o1 = (int)((rc.off >> SH) & MASK);
      // expanded w0 (planes) and w1 (rows) of this node
      float w0x[E0MAX], w1x[E1];
#pragma unroll
      for (int p = 0; p < E0MAX; ++p) w0x[p] = tc_tap<WIN>(rc.fr0, mf, p - o0, W, k0);
#pragma unroll
      for (int p = 0; p < E1; ++p) w1x[p] = tc_tap<WIN>(rc.fr1, mf, p - o1, W, k1);
      float accx = 0.f, accy = 0.f;
#pragma unroll
      for (int c = 0; c < MAXCH; ++c) {
        if (c < nch) {
          const uint32_t buf = gc & 1u;
          healthy &= tc::mbar_wait_warp(&tfull[buf], (gc >> 1) & 1u, kItPolls);
          tc::fence_after_sync();
          const uint32_t t0 = tmem + ((uint32_t)(32 * q) << 16) + buf * 256u;
#pragma unroll
          for (int gi = 0; gi < N / 16; ++gi) {
            float v[16];
            tc::tmem_ld16(t0 + (uint32_t)(gi * 16), v);
            tc::tmem_ld_wait();
#pragma unroll
            for (int u = 0; u < 16; u += 2) {
              const int col = gi * 16 + u;  // (re, im) of (plane pl, row p1)
              if (col < NCOL) {
                const int pl = col / (2 * E1), p1 = (col % (2 * E1)) / 2;
                if (c * CH + pl < E0MAX) {
                  const float w = w0x[c * CH + pl] * w1x[p1];
                  accx = fmaf(w, v[u], accx);
                  accy = fmaf(w, v[u + 1], accy);
                }
              }
            }
          }
          tc::fence_before_sync();
          tc::mbar_arrive_warp(&tempty[buf]);
          ++gc;
        }
      }
      if (rc.idx >= 0) f[rc.idx] = make_float2(accx * norm, accy * norm);
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
