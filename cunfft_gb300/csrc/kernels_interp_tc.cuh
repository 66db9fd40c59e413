// kernels_interp_tc.cuh -- 3D FP32 interpolation on the tensor cores (tcgen05, 3xTF32),
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
// The grid is first split (k_split_pad) into TF32 hi + lo parts of its real and
// imaginary parts, each a float array over the periodically padded index range
// [0, n_t + W - 1) per dimension.  Every tile's padded box then lies inside those
// arrays (no wrap), and one thread loads each chunk with four TMA boxes (hi re, hi im,
// lo re, lo im; 32 floats x E1 rows x CH planes) straight into the 128-byte swizzled
// K-major layout the MMAs read.  Warp roles: warp 0 lane 0 issues the TMA loads
// (four chunk stages), warp 1 lane 0 the MMAs hi*hi + hi*lo + lo*hi per k-step of 8
// columns, warps 2-5 (lane quarters) build A from their nodes' taps and reduce D.
// Hand-offs are mbarriers (the chunk stages' with TMA transaction counts); every wait
// is bounded and a wait that gives up sets the plan's device status flag.
#pragma once

#include <cuda.h>

#include "kernels_grid.cuh"
#include "tc_sm100.cuh"

namespace cg {

constexpr int kItMaxT0 = 16;       // outer tile extent limit (E0 <= 31 planes)
constexpr int kItK = 32;           // K: innermost tile columns p2 (E2 <= 31), padded; one 128-byte row
constexpr int kItNodes = 128;      // nodes per batch (MMA M)
constexpr int kItTmaWarp = 0;
constexpr int kItMmaWarp = 1;
constexpr int kItNodeWarp0 = 2;    // 4 node warps: lane quarter = warp % 4
constexpr int kItThreads = 6 * 32;
constexpr uint32_t kItLBO = 128;               // A: core matrices along K
constexpr uint32_t kItSBOA = 1024;             // A: 8-row groups (32 K values = 8 core matrices)
constexpr int kItHalf = 64;                    // B rows per part: real parts 0..63, imaginary 64..127
constexpr int kItN = 2 * kItHalf;              // MMA N
constexpr int kItStages = 4;                   // chunk stages = tensor-memory accumulators (kItN columns each)
constexpr uint32_t kItPart = kItHalf * 128;    // one B part (hi re, hi im, lo re, lo im): 64 rows x 128 bytes
constexpr uint32_t kItStage = 4 * kItPart;     // one chunk stage: B hi = parts 0-1, B lo = parts 2-3
constexpr uint32_t kItPolls = 1u << 20;        // mbarrier polls (<= 1 us each) before giving up

__host__ __device__ constexpr int it_e1(int W) { return fixed_t_mid(3, W) + W - 1; }
__host__ __device__ constexpr int it_ch(int W) { return kItHalf / it_e1(W); }                 // planes per chunk
__host__ __device__ constexpr int it_pairs(int W) { return it_ch(W) * it_e1(W); }            // (plane, row) pairs <= 64

__host__ __device__ constexpr bool interp_tc_ok(int d, int W, int T0, int64_t n2) {
  return d == 3 && W >= 4 && W <= 16 && T0 >= 1 && T0 <= kItMaxT0 && n2 >= 4 && n2 % 4 == 0;
}

// Shared-memory layout (byte offsets from a 1024-byte aligned base; host and device agree).
struct ItLayout {
  uint32_t b_off;      // kItStages chunk stages of kItStage
  uint32_t a_off;      // 2 buffers x (A hi, A lo), 16 KB each
  uint32_t bar_off;    // afull[2], bfull[4], bempty[4], tfull[4], tempty[4]; tensor-memory base
  uint32_t total;      // bytes past the aligned base
  uint32_t dyn;        // dynamic shared memory to request (alignment slack included)
};

__host__ __device__ constexpr ItLayout it_layout() {
  return ItLayout{0u, kItStages * kItStage, kItStages * kItStage + 4u * 16384u,
                  kItStages * kItStage + 4u * 16384u + 160u, kItStages * kItStage + 4u * 16384u + 160u + 1024u};
}

// Padded split planes of the grid: float [batch][4][P0][P1][P2s], component 0 hi re,
// 1 hi im, 2 lo re, 3 lo im; P_t = n_t + W - 1 holds grid index i mod n_t, P2s = P2
// rounded up to a multiple of 4 (16-byte rows).
struct ItSplit {
  int64_t P0, P1, P2, P2s;
};
__host__ __device__ inline ItSplit it_split_dims(const Geom& g) {
  ItSplit s;
  s.P0 = g.n[0] + g.W - 1;
  s.P1 = g.n[1] + g.W - 1;
  s.P2 = g.n[2] + g.W - 1;
  s.P2s = (s.P2 + 3) / 4 * 4;
  return s;
}

// One thread per 4 consecutive p2 of one padded row: the quad never straddles the grid's
// wrap (n2 % 4 == 0), reads two float4 of complex data and writes one float4 to each of
// the four components.
__global__ void k_split_pad(const float2* __restrict__ g, float* __restrict__ out, Geom geo, ItSplit sd) {
  const int64_t q4 = sd.P2s / 4, row_q = sd.P1 * q4, per = sd.P0 * row_q, total = per * geo.batch;
  const int64_t comp = sd.P0 * sd.P1 * sd.P2s;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t inst = e / per, r = e - inst * per;
    const int64_t i0 = r / row_q, r2 = r - i0 * row_q;
    const int64_t i1 = r2 / q4, i2 = (r2 - i1 * q4) * 4;
    const float2* src = g + inst * geo.ntot +
                        (wrap_up(i0, geo.n[0]) * geo.n[1] + wrap_up(i1, geo.n[1])) * geo.n[2] + wrap_up(i2, geo.n[2]);
    const float4 a = reinterpret_cast<const float4*>(src)[0], b = reinterpret_cast<const float4*>(src)[1];
    float4 h, l;
    float* o = out + inst * 4 * comp + (i0 * sd.P1 + i1) * sd.P2s + i2;
    tc_split4(make_float4(a.x, a.z, b.x, b.z), h, l);
    *reinterpret_cast<float4*>(o) = h;
    *reinterpret_cast<float4*>(o + 2 * comp) = l;
    tc_split4(make_float4(a.y, a.w, b.y, b.w), h, l);
    *reinterpret_cast<float4*>(o + comp) = h;
    *reinterpret_cast<float4*>(o + 3 * comp) = l;
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
                                                             float2* __restrict__ f, Geom geo, Tiling tl, Bins bins) {
  constexpr int E1 = it_e1(W), CH = it_ch(W), NP = it_pairs(W);
  constexpr int E0MAX = kItMaxT0 + W - 1;
  constexpr int MAXCH = (E0MAX + CH - 1) / CH;
  constexpr int GI = (NP + 15) / 16;  // 16-pair groups of the tensor-memory read-out
  constexpr int SH = off_bits(3);
  constexpr uint32_t MASK = (1u << SH) - 1u;
  constexpr uint32_t kBoxBytes = (uint32_t)(kItK * 4 * E1 * CH);
  static_assert(NP <= kItHalf && NP > 0, "a chunk's (plane, row) pairs must fit one B part");
  static_assert(kItStages * kItN <= 512, "the accumulators must fit tensor memory");
  static_assert(fixed_t_last(3, W) + W - 1 <= kItK, "innermost padded extent must fit K");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const ItLayout L = it_layout();
  uint64_t* afull = reinterpret_cast<uint64_t*>(smem + L.bar_off);  // [2] A of the batch built
  uint64_t* bfull = afull + 2;                                       // [4] tile chunk landed (TMA)
  uint64_t* bempty = afull + 6;                                      // [4] MMAs of the chunk complete
  uint64_t* tfull = afull + 10;                                      // [4] accumulator complete
  uint64_t* tempty = afull + 14;                                     // [4] accumulator read out
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 144);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int E0 = tl.E[0];
  const int nch = (E0 + CH - 1) / CH;
  const int num_items = *bins.num_items;
  const int G = (int)gridDim.x;

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) tc::mbar_init(&afull[i], 4);  // one arrival per node warp
    for (int i = 0; i < kItStages; ++i) {
      tc::mbar_init(&bfull[i], 1);    // the TMA thread's arrival (+ the boxes' bytes)
      tc::mbar_init(&bempty[i], 1);
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], 4);   // one arrival per node warp
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
  // sequence) uses chunk stage and accumulator gc & 3 in their cycle gc >> 2.
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
            const uint32_t buf = gc & 3u;
            if (gc >= 4) healthy &= tc::mbar_wait_bounded(&bempty[buf], ((gc >> 2) - 1u) & 1u, kItPolls);
            unsigned char* st = smem + L.b_off + buf * kItStage;
            tc::mbar_arrive_expect_tx(&bfull[buf], 4u * kBoxBytes);
            // x = o.a[2] is a multiple of the innermost tile extent (>= 4 floats: 16 bytes)
            for (int comp = 0; comp < 4; ++comp)
              tc::tma_load_5d(st + comp * kItPart, &tmap, (int)o.a[2], (int)o.a[1], (int)o.a[0] + c * CH, comp,
                              (int)o.inst, &bfull[buf]);
          }
        }
      }
      // the boxes of the last chunks have landed before this CTA can exit
      for (uint32_t k = 1; k <= (uint32_t)kItStages && k <= gc; ++k)
        healthy &= tc::mbar_wait_bounded(&bfull[(gc - k) & 3u], ((gc - k) >> 2) & 1u, kItPolls);
    }
    __syncwarp();
  } else if (warp == kItMmaWarp) {
    // ======================= MMA issuer: lane 0 =======================
    if (lane == 0) {
      const uint32_t sa = tc::smem_u32(smem + L.a_off), sb = tc::smem_u32(smem + L.b_off);
      const uint64_t d_abuf = (uint64_t)(32768u >> 4);  // A buffer 1 = buffer 0 + d_abuf
      const uint64_t d_ah = tc::smem_desc(sa, kItLBO, kItSBOA);
      const uint64_t d_al = tc::smem_desc(sa + 16384u, kItLBO, kItSBOA);
      const uint64_t d_bh = tc::smem_desc_sw128(sb);
      const uint64_t d_bl = tc::smem_desc_sw128(sb + 2u * kItPart);
      const uint64_t d_buf = (uint64_t)(kItStage >> 4);  // stage k = stage 0 + k d_buf
      const uint32_t idesc = tc::idesc_tf32(128, kItN);
      uint32_t gc = 0, gbt = 0;
      for (int it = blockIdx.x; it < num_items; it += G) {
        const int4 item = bins.items[it];
        const int nbatch = (item.z - item.y + kItNodes - 1) / kItNodes;
        for (int bt = 0; bt < nbatch; ++bt, ++gbt) {
          const uint32_t ab = gbt & 1u;
          healthy &= tc::mbar_wait_bounded(&afull[ab], (gbt >> 1) & 1u, kItPolls);
          const uint64_t ao = ab ? d_abuf : 0ull;
          for (int c = 0; c < nch; ++c, ++gc) {
            const uint32_t buf = gc & 3u;
            healthy &= tc::mbar_wait_bounded(&bfull[buf], (gc >> 2) & 1u, kItPolls);
            if (gc >= 4) healthy &= tc::mbar_wait_bounded(&tempty[buf], ((gc >> 2) - 1u) & 1u, kItPolls);
            tc::fence_after_sync();
            const uint32_t d = tmem + buf * (uint32_t)kItN;
            const uint64_t bo = (uint64_t)buf * d_buf;
#pragma unroll
            for (int ks = 0; ks < kItK / 8; ++ks) {
              const uint64_t ka = (uint64_t)((ks * 2 * kItLBO) >> 4);  // A: two core matrices per k-step
              const uint64_t kb = (uint64_t)((ks * 32) >> 4);          // B: 32 bytes into the swizzled row
              tc::mma_tf32(d, d_ah + ao + ka, d_bh + bo + kb, idesc, ks > 0 ? 1u : 0u);
              tc::mma_tf32(d, d_ah + ao + ka, d_bl + bo + kb, idesc, 1u);
              tc::mma_tf32(d, d_al + ao + ka, d_bh + bo + kb, idesc, 1u);
            }
            tc::mma_commit(&bempty[buf]);
            tc::mma_commit(&tfull[buf]);
          }
        }
      }
      // the last chunk commits are waited by the node warps; the last bempty arrivals here
      for (uint32_t k = 1; k <= (uint32_t)kItStages && k <= gc; ++k)
        healthy &= tc::mbar_wait_bounded(&bempty[(gc - k) & 3u], ((gc - k) >> 2) & 1u, kItPolls);
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
      unsigned char* ah = smem + L.a_off + ab * 32768u;
      unsigned char* al = ah + 16384u;
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
          const uint32_t buf = gc & 3u;
          healthy &= tc::mbar_wait_warp(&tfull[buf], (gc >> 2) & 1u, kItPolls);
          tc::fence_after_sync();
          const uint32_t t0 = tmem + ((uint32_t)(32 * q) << 16) + buf * (uint32_t)kItN;
#pragma unroll
          for (int gi = 0; gi < GI; ++gi) {
            float vr[16], vi[16];
            tc::tmem_ld16(t0 + (uint32_t)(gi * 16), vr);         // real parts of pairs 16 gi ..
            tc::tmem_ld16(t0 + (uint32_t)kItHalf + (uint32_t)(gi * 16), vi);  // imaginary parts
            tc::tmem_ld_wait();
#pragma unroll
            for (int u = 0; u < 16; ++u) {
              const int pr = gi * 16 + u;  // (plane pl, row p1) of the chunk
              if (pr < NP) {
                const int pl = pr / E1, p1 = pr - (pr / E1) * E1;
                if (c * CH + pl < E0MAX) {
                  const float w = w0x[c * CH + pl] * w1x[p1];
                  accx = fmaf(w, vr[u], accx);
                  accy = fmaf(w, vi[u], accy);
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
