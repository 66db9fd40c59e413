// kernels_bin.cu -- node binning: FP64 node-to-grid reduction and counting sort by tile.
//
// For every node and dimension t the window start is the reference's rule
// (src/cunfft_kernel.cu:175-182)
//     u_t = llrint(n_t x_t) - signbit(x_t) - m,    c_t = n_t x_t - u_t,
// and the 2m+2 taps of the node cover grid indices (u_t + l) mod n_t.  The node is
// filed under the tile that holds its wrapped window start s_t = u_t mod n_t; the
// tile-local start o_t = s_t mod T_t and the fraction c_t - m (exact in FP64, then
// rounded to the plan's real type) are what the gridding kernels need.
#include "bin_coord.h"
#include "runtime.h"

namespace cg {

// log2 n_t for power-of-two sizes, else -1: those dimensions reduce x by integer
// arithmetic on its bits (bin_coord.h), the others in FP64
struct BinLog2 {
  int k[kMaxDim];
};

// bits per dimension of the packed tile-local window start (30 / d)
__host__ __device__ inline int off_bits_host(int d) { return d == 1 ? 30 : (d == 2 ? 15 : 10); }

__device__ __forceinline__ int find_instance(const int32_t* __restrict__ inst_off, int batch, int64_t j) {
  int lo = 0, hi = batch;  // inst_off[lo] <= j < inst_off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (inst_off[mid] <= j) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void reduce_coord(double x, int64_t n, int m, int64_t& u, double& c) {
  double nx = __dmul_rn(x, (double)n);
  u = (int64_t)__double2ll_rn(nx) - (signbit(x) ? 1 : 0) - (int64_t)m;
  c = __dsub_rn(nx, (double)u);
}

__global__ void k_bin_count(const double* __restrict__ x, int64_t M, Geom geo, Tiling tl, BinLog2 lg,
                            const int32_t* __restrict__ inst_off, int32_t* __restrict__ count,
                            int2* __restrict__ tile_rank) {
  const int d = geo.d;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
    int inst = geo.batch > 1 ? find_instance(inst_off, geo.batch, j) : 0;
    int64_t tile = 0;
    int sub = 0;  // sub-bin of the window start inside the tile (Tiling::sub_on)
    for (int t = 0; t < d; ++t) {
      const double xt = x[j * d + t];
      int64_t u;
      CoordPow2 cp;
      if (lg.k[t] >= 0 && coord_pow2(xt, lg.k[t], geo.m, cp)) {
        u = cp.u;
      } else {
        double c;
        reduce_coord(xt, geo.n[t], geo.m, u, c);
      }
      int64_t s = wrap_n(u, geo.n[t]);
      tile = tile * tl.nb[t] + (s >> (__ffs(tl.T[t]) - 1));  // T_t is a power of two
      if (tl.sub_on && t < 2) {
        const int o = (int)(s & (tl.T[t] - 1));
        sub = t == 0 ? (o >> tl.ssh[0]) * tl.snb1 : sub + (o >> tl.ssh[1]);
      }
    }
    tile += (int64_t)inst * tl.tiles_per_inst;
    if (tl.sub_on) tile = tile * tl.ns + sub;  // the counting sort's key
    // one atomic per tile and warp: the lanes that share a tile (clustered nodes fill a
    // few tiles) take consecutive ranks from their leader's single add
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, (unsigned long long)tile);
    const int leader = __ffs(peers) - 1, lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader) base = atomicAdd(&count[tile], __popc(peers));
    base = __shfl_sync(act, base, leader);
    const int rank = base + __popc(peers & ((1u << lane) - 1u));
    tile_rank[j] = make_int2((int)tile, rank);
  }
}

// FP32 fractions on power-of-two sizes come from the integer form: the exact c - m
// rounded once to FP32 (the FP64 form rounds c to FP64 first; the two differ by at most
// one FP32 ulp plus 2^-49).  FP64 fractions always take the FP64 form.
// With sub-bins the key is tile * ns + sub-bin (ns a power of two): the node's place is its
// tile's first place, then the tile's sub-bins before its own, then its rank.
template <typename T>
__global__ void k_bin_scatter(const double* __restrict__ x, int64_t M, Geom geo, Tiling tl, BinLog2 lg,
                              const int2* __restrict__ tile_rank, const int32_t* __restrict__ tile_off,
                              const int32_t* __restrict__ sub_pre, int32_t* __restrict__ sidx,
                              int32_t* __restrict__ soff, T* __restrict__ sfrac) {
  const int d = geo.d;
  const int nsh = __ffs(tl.ns) - 1;  // ns = 2^nsh
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
    int2 tr = tile_rank[j];
    int64_t pos = tl.sub_on ? (int64_t)tile_off[tr.x >> nsh] + sub_pre[tr.x] + tr.y : (int64_t)tile_off[tr.x] + tr.y;
    uint32_t packed = 0;
    for (int t = 0; t < d; ++t) {
      const double xt = x[j * d + t];
      int64_t u;
      T frac;
      CoordPow2 cp;
      if (sizeof(T) == 4 && lg.k[t] >= 0 && coord_pow2(xt, lg.k[t], geo.m, cp)) {
        u = cp.u;
        frac = (T)coord_pow2_frac(cp);
      } else {
        double c;
        reduce_coord(xt, geo.n[t], geo.m, u, c);
        frac = (T)(c - (double)geo.m);
      }
      int64_t s = wrap_n(u, geo.n[t]);
      uint32_t o = (uint32_t)(s & (tl.T[t] - 1));  // T_t is a power of two
      packed |= o << (off_bits_host(d) * t);
      sfrac[pos * d + t] = frac;
    }
    sidx[pos] = (int32_t)j;
    soff[pos] = (int32_t)packed;
  }
}

// Single-CTA exclusive scan of the per-tile counts and of the per-tile work-item
// counts ceil(count / chunk), in rounds of kScanRound tiles: warp w takes the 256
// tiles w * 256 .. w * 256 + 255 of the round, lane l the tiles l, l + 32, ... of them,
// so every load and store of a warp is one contiguous 128-byte line.  A warp scans its
// tiles in eight steps of 32 (warp shuffles, carrying the step totals), the 32 warp
// totals are scanned in shared memory, and the round's total carries into the next.
constexpr int kScanRound = 1024 * 8;

__device__ __forceinline__ void warp_incl_scan2(int32_t& a, int32_t& b) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t x = __shfl_up_sync(0xffffffffu, a, o), y = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o) {
      a += x;
      b += y;
    }
  }
}

// Positions and item counts fit 32 bits: the sorted arrays are int32-indexed.
__global__ void __launch_bounds__(1024) k_scan_tiles(const int32_t* __restrict__ count, int64_t ntiles, int chunk,
                                                     int32_t* __restrict__ tile_off, int32_t* __restrict__ item_off,
                                                     int32_t* __restrict__ num_items) {
  __shared__ int32_t wc[32], wi[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int per = kScanRound / (int)blockDim.x;  // tiles per lane and round (8 at 1024 threads)
  const int csh = (chunk & (chunk - 1)) == 0 ? __ffs(chunk) - 1 : -1;  // chunk = 2^csh
  int32_t run_c = 0, run_i = 0;  // totals of the rounds before (the same in every thread)
  for (int64_t r0 = 0; r0 < ntiles; r0 += kScanRound) {
    const int64_t wb = r0 + (int64_t)warp * 32 * per;
    int32_t ec[8], ei[8], cc = 0, ci = 0;  // exclusive prefixes within the warp's tiles
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int64_t e = wb + 32 * k + lane;
      const int32_t v = (k < per && e < ntiles) ? count[e] : 0;
      const int32_t w = csh >= 0 ? (v + chunk - 1) >> csh : (v + chunk - 1) / chunk;
      int32_t a = v, b = w;
      warp_incl_scan2(a, b);
      ec[k] = cc + a - v;
      ei[k] = ci + b - w;
      cc += __shfl_sync(0xffffffffu, a, 31);
      ci += __shfl_sync(0xffffffffu, b, 31);
    }
    if (lane == 0) {
      wc[warp] = cc;
      wi[warp] = ci;
    }
    __syncthreads();
    if (warp == 0) {
      int32_t a = lane < nw ? wc[lane] : 0, b = lane < nw ? wi[lane] : 0;
      warp_incl_scan2(a, b);
      wc[lane] = a;
      wi[lane] = b;
    }
    __syncthreads();
    const int32_t bc = run_c + (warp > 0 ? wc[warp - 1] : 0), bi = run_i + (warp > 0 ? wi[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int64_t e = wb + 32 * k + lane;
      if (k < per && e < ntiles) {
        tile_off[e] = bc + ec[k];
        item_off[e] = bi + ei[k];
      }
    }
    run_c += wc[nw - 1];
    run_i += wi[nw - 1];
    __syncthreads();  // wc / wi are rewritten by the next round
  }
  if (tid == 0) {
    tile_off[ntiles] = run_c;
    item_off[ntiles] = run_i;
    *num_items = run_i;
  }
}

// Per tile from its sub-bin counts (the tile's ns consecutive keys): the tile's node
// count, each sub-bin's place inside the tile, and the tile's interpolation items of at
// most kSubItem nodes of one sub-bin (with sub_items).
__global__ void k_tile_subs(const int32_t* __restrict__ scount, int64_t ntiles, int ns, int sub_items,
                            int32_t* __restrict__ count, int32_t* __restrict__ sub_pre, int32_t* __restrict__ icount) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = 0, ic = 0;
    for (int s = 0; s < ns; ++s) {
      const int32_t v = scount[t * ns + s];
      sub_pre[t * ns + s] = c;
      c += v;
      ic += (v + kSubItem - 1) / kSubItem;
    }
    count[t] = c;
    if (sub_items) icount[t] = ic;
  }
}

// The interpolation items of each sub-bin, kSubItem nodes at a time (thread per sub-bin:
// its first item follows the items of its tile's sub-bins before it).
__global__ void k_make_sub_items(const int32_t* __restrict__ scount, const int32_t* __restrict__ sub_pre,
                                 const int32_t* __restrict__ tile_off, const int32_t* __restrict__ iitem_off,
                                 int64_t nkeys, int ns, int4* __restrict__ iitems) {
  for (int64_t key = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; key < nkeys;
       key += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = key / ns, k0 = t * ns;
    int32_t io = iitem_off[t];
    for (int64_t q = k0; q < key; ++q) io += (scount[q] + kSubItem - 1) / kSubItem;
    const int32_t c = scount[key], a0 = tile_off[t] + sub_pre[key];
    for (int32_t k = 0; k * kSubItem < c; ++k, ++io)
      iitems[io] = make_int4((int)key, a0 + k * kSubItem, min(a0 + c, a0 + (k + 1) * kSubItem), 0);
  }
}

__global__ void k_make_items(const int32_t* __restrict__ count, const int32_t* __restrict__ tile_off,
                             const int32_t* __restrict__ item_off, int64_t ntiles, int chunk,
                             int4* __restrict__ items) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = count[t], s = tile_off[t], io = item_off[t];
    for (int32_t k = 0; k * chunk < c; ++k) {
      int32_t a = s + k * chunk;
      items[io + k] = make_int4((int)t, a, min(s + c, a + chunk), 0);
    }
  }
}

static inline int grid_for(int64_t work, int threads, int sms) {
  int64_t b = (work + threads - 1) / threads;
  int64_t cap = (int64_t)sms * 32;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_binning(const Plan& p, const double* x, cudaStream_t st) {
  const Bins& B = p.bins;
  const Tiling& tl = p.tl;
  BinLog2 lg;
  for (int t = 0; t < kMaxDim; ++t) {
    const int64_t n = t < p.geo.d ? p.geo.n[t] : 0;
    int k = -1;
    if (n > 0 && (n & (n - 1)) == 0)
      for (k = 0; (int64_t(1) << k) < n; ++k) {
      }
    lg.k[t] = k;
  }
  // counting sort over keys: tiles, or tile * ns + sub-bin with sub-bins; the tile counts
  // then come from the sub-bin counts, and only the tiles are scanned
  const bool sub = tl.sub_on != 0;
  const int64_t nkeys = tl.tiles_total * (sub ? tl.ns : 1);
  int32_t* kcount = sub ? B.scount : B.count;
  cudaError_t e = cudaMemsetAsync(kcount, 0, sizeof(int32_t) * (nkeys + 1), st);
  if (e != cudaSuccess) return e;
  if (B.M > 0) {
    k_bin_count<<<grid_for(B.M, 256, p.num_sms), 256, 0, st>>>(x, B.M, p.geo, tl, lg, B.inst_off, kcount,
                                                                 B.tile_rank);
  }
  if (sub)
    k_tile_subs<<<grid_for(tl.tiles_total, 256, p.num_sms), 256, 0, st>>>(B.scount, tl.tiles_total, tl.ns,
                                                                           tl.sub_items, B.count, B.sub_pre,
                                                                           B.icount);
  k_scan_tiles<<<1, 1024, 0, st>>>(B.count, tl.tiles_total, tl.chunk, B.tile_off, B.item_off, B.num_items);
  if (sub && tl.sub_items)  // chunk 1: the scan of the item counts themselves
    k_scan_tiles<<<1, 1024, 0, st>>>(B.icount, tl.tiles_total, 1, B.iitem_off, B.iscratch, B.num_iitems);
  if (B.M > 0) {
    if (p.prec == kF64)
      k_bin_scatter<double><<<grid_for(B.M, 256, p.num_sms), 256, 0, st>>>(
          x, B.M, p.geo, tl, lg, B.tile_rank, B.tile_off, B.sub_pre, B.sidx, B.soff, (double*)B.sfrac);
    else
      k_bin_scatter<float><<<grid_for(B.M, 256, p.num_sms), 256, 0, st>>>(
          x, B.M, p.geo, tl, lg, B.tile_rank, B.tile_off, B.sub_pre, B.sidx, B.soff, (float*)B.sfrac);
    k_make_items<<<grid_for(tl.tiles_total, 256, p.num_sms), 256, 0, st>>>(B.count, B.tile_off, B.item_off,
                                                                            tl.tiles_total, tl.chunk, B.items);
    if (sub && tl.sub_items)
      k_make_sub_items<<<grid_for(nkeys, 256, p.num_sms), 256, 0, st>>>(B.scount, B.sub_pre, B.tile_off,
                                                                          B.iitem_off, nkeys, tl.ns, B.iitems);
  }
  return cudaGetLastError();
}

}  // namespace cg
