// kernels_grid_global.cu -- gridding without a shared-memory tile.
//
// Used when the padded tile of even a single grid cell does not fit in the 227 KB
// of shared memory a CTA may use: wide windows in 3D, e.g. m >= 11 in the FP64
// form ((2m+2)^3 * 16 bytes > 227 KB).  Same work items as the tiled kernels;
// one thread per node, taps read from (interpolation) or atomically added to
// (spreading) the oversampled grid in global memory, weights in the plan's real
// type from the binned fractions.  Results agree with the tiled kernels.
#include "kernels_grid.cuh"

namespace cg {

template <int D, typename T, bool SPREAD>
__global__ void __launch_bounds__(128) k_grid_global(const typename Cx<T>::t* __restrict__ in,
                                                     typename Cx<T>::t* __restrict__ out, Geom geo, Tiling tl,
                                                     Bins bins) {
  using C = typename Cx<T>::t;
  __shared__ int4 cur;
  const int W = geo.W;
  const T* sfrac = reinterpret_cast<const T*>(bins.sfrac);
  const T norm = (T)geo.norm;
  while (next_item(bins, SPREAD ? 1 : 0, &cur)) {
    const int4 item = cur;
    const TileOrigin o = decode_tile<D>(geo, tl, item.x);
    for (int64_t k = item.y + threadIdx.x; k < item.z; k += blockDim.x) {
      const int idx = bins.sidx[k];
      const uint32_t off = (uint32_t)bins.soff[k];
      int64_t s[kMaxDim];
      T w[kMaxDim][kMaxTaps];
      for (int t = 0; t < D; ++t) {
        s[t] = o.a[t] + ((off >> (off_bits(D) * t)) & ((1u << off_bits(D)) - 1u));
        WeightMath<T>::taps(sfrac[k * D + t], geo.m, geo, t, W, w[t]);
      }
      const int64_t inst_base = o.inst * geo.ntot;
      if (!SPREAD) {
        C acc;
        acc.x = (T)0;
        acc.y = (T)0;
        for (int l0 = 0; l0 < W; ++l0) {
          const int64_t i0 = wrap_up(s[0] + l0, geo.n[0]);
          if (D == 1) {
            acc = cmul_add(acc, w[0][l0], in[inst_base + i0]);
            continue;
          }
          C a1;
          a1.x = (T)0;
          a1.y = (T)0;
          for (int l1 = 0; l1 < W; ++l1) {
            const int64_t i1 = wrap_up(s[1] + l1, geo.n[1]);
            if (D == 2) {
              a1 = cmul_add(a1, w[1][l1], in[inst_base + i0 * geo.n[1] + i1]);
              continue;
            }
            C a2;
            a2.x = (T)0;
            a2.y = (T)0;
            const int64_t rowb = inst_base + (i0 * geo.n[1] + i1) * geo.n[D - 1];
            for (int l2 = 0; l2 < W; ++l2)
              a2 = cmul_add(a2, w[D - 1][l2], in[rowb + wrap_up(s[D - 1] + l2, geo.n[D - 1])]);
            a1 = cmul_add(a1, w[1][l1], a2);
          }
          acc = cmul_add(acc, w[0][l0], a1);
        }
        out[idx] = cscale(acc, norm);
      } else {
        const C v = cscale(in[idx], norm);
        for (int l0 = 0; l0 < W; ++l0) {
          const int64_t i0 = wrap_up(s[0] + l0, geo.n[0]);
          const C v0 = cscale(v, w[0][l0]);
          if (D == 1) {
            global_add(&out[inst_base + i0], v0);
            continue;
          }
          for (int l1 = 0; l1 < W; ++l1) {
            const int64_t i1 = wrap_up(s[1] + l1, geo.n[1]);
            const C v1 = cscale(v0, w[1][l1]);
            if (D == 2) {
              global_add(&out[inst_base + i0 * geo.n[1] + i1], v1);
              continue;
            }
            const int64_t rowb = inst_base + (i0 * geo.n[1] + i1) * geo.n[D - 1];
            for (int l2 = 0; l2 < W; ++l2)
              global_add(&out[rowb + wrap_up(s[D - 1] + l2, geo.n[D - 1])], cscale(v1, w[D - 1][l2]));
          }
        }
      }
    }
    __syncthreads();
  }
}

template <int D, typename T, bool SPREAD>
static cudaError_t launch_global(const Plan& p, const void* in, void* out, cudaStream_t st) {
  using C = typename Cx<T>::t;
  auto kern = k_grid_global<D, T, SPREAD>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
  if (e != cudaSuccess) return e;
  kern<<<p.num_sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>((const C*)in, (C*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_global(const Plan& p, bool spread, const void* in, void* out, cudaStream_t st) {
  const int d = p.geo.d;
  if (p.prec == kF64) {
    if (d == 1) return spread ? launch_global<1, double, true>(p, in, out, st) : launch_global<1, double, false>(p, in, out, st);
    if (d == 2) return spread ? launch_global<2, double, true>(p, in, out, st) : launch_global<2, double, false>(p, in, out, st);
    return spread ? launch_global<3, double, true>(p, in, out, st) : launch_global<3, double, false>(p, in, out, st);
  }
  if (d == 1) return spread ? launch_global<1, float, true>(p, in, out, st) : launch_global<1, float, false>(p, in, out, st);
  if (d == 2) return spread ? launch_global<2, float, true>(p, in, out, st) : launch_global<2, float, false>(p, in, out, st);
  return spread ? launch_global<3, float, true>(p, in, out, st) : launch_global<3, float, false>(p, in, out, st);
}

}  // namespace cg
