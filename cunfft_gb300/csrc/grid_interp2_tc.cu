// grid_interp2_tc.cu -- the 2D tensor-core FP32 interpolation: the sub-bins of the tilings
// it covers, the grid's padded FP16 hi/lo rows and their TMA map, and the launches.
#include <cudaTypedefs.h>

#include <algorithm>

#include "kernels_interp2_tc.cuh"

namespace cg {

static int log2_of(int v) {
  int k = 0;
  while ((1 << k) < v) ++k;
  return k;
}

// 16 x 16 sub-tiles of window starts (fewer rows when the tile has fewer): the sub-bins
// the binning sorts every tile's nodes by, for a 2D FP32 tiling this kernel covers.
void interp2_tc_subbins(const Plan& p, Tiling& tl) {
  tl.sub_on = 0;
  tl.sub_items = 0;
  tl.ns = 1;
  tl.ssh[0] = tl.ssh[1] = 0;
  tl.snb1 = 1;
  if (p.prec != kF32 || tl.use_global || !interp2_tc_ok(p.geo.d, p.geo.W, tl.T[1], p.geo.n[1])) return;
  const int s0 = std::min(tl.T[0], kI2Sub);
  const int ns = (tl.T[0] / s0) * (tl.T[1] / kI2Sub);
  if (tl.tiles_total * ns >= ((int64_t)1 << 31)) return;  // sort keys are 32-bit
  tl.ssh[0] = log2_of(s0);
  tl.ssh[1] = log2_of(kI2Sub);
  tl.snb1 = tl.T[1] / kI2Sub;
  tl.ns = ns;
  tl.sub_on = 1;
  tl.sub_items = 1;
}

bool interp2_tc_supported(const Plan& p) {
  return p.geo.d == 2 && p.prec == kF32 && !p.tl.use_global && p.tl.sub_on && p.tl.sub_items;
}

// Split rows half [batch][4][P0][P2s], row scales float [batch][P0], and the 5-D map over
// the rows (dims P2s, P0, 1, component, instance; box 32 halves x (16 + W - 1) rows,
// 64-byte swizzle, zero fill outside).  Box rows are 64 bytes (32 halves); rows of the
// arrays are multiples of 16 bytes (P2s % 8 == 0).
cudaError_t interp2_tc_prepare(Plan& p, PFN_cuTensorMapEncodeTiled_v12000 enc) {
  if (p.it_ready) return cudaSuccess;
  const ItSplit sd = i2_split_dims(p.geo);
  const size_t comp = (size_t)(sd.P0 * sd.P2s);
  const size_t bytes = sizeof(__half) * 4 * comp * (size_t)p.geo.batch;
  if (!enc) return cudaErrorNotSupported;
  if (!p.it_split) {
    cudaError_t e = plan_malloc(&p.it_split, bytes);
    if (e == cudaSuccess) e = plan_malloc(&p.it_pinv, sizeof(float) * (size_t)(sd.P0 * p.geo.batch));
    if (e != cudaSuccess) {
      interp_tc_release(p);
      return e;
    }
  }
  const int E0S = kI2Sub + p.geo.W - 1;  // rows of a 16-row sub-tile's windows (the kernel's B rows)
  const cuuint64_t dims[5] = {(cuuint64_t)sd.P2s, (cuuint64_t)sd.P0, 1u, 4u, (cuuint64_t)p.geo.batch};
  const cuuint64_t strides[4] = {(cuuint64_t)(sd.P2s * 2), (cuuint64_t)(comp * 2), (cuuint64_t)(comp * 2),
                                 (cuuint64_t)(4 * comp * 2)};
  const cuuint32_t box[5] = {(cuuint32_t)kI2K, (cuuint32_t)E0S, 1u, 1u, 1u};
  const cuuint32_t estr[5] = {1u, 1u, 1u, 1u, 1u};
  const CUresult r = enc(&p.it_tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, p.it_split, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  p.it_ready = true;
  return cudaSuccess;
}

template <int W>
static cudaError_t launch_i2(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (!interp2_tc_supported(p) || !p.it_ready) return cudaErrorInvalidConfiguration;
  const ItSplit sd = i2_split_dims(p.geo);
  const int64_t rows = sd.P0 * p.geo.batch;
  const int sblocks = (int)std::min<int64_t>((rows + kI2SplitThreads / 32 - 1) / (kI2SplitThreads / 32),
                                             (int64_t)p.num_sms * 8);
  k_split_rows<<<sblocks, kI2SplitThreads, 0, st>>>((const float2*)in, (__half*)p.it_split, p.it_pinv, p.geo, sd);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // 512 tensor-memory columns per CTA: at most one CTA per SM (more than half the SM's
  // 228 KB of shared memory), so tcgen05.alloc never waits
  const size_t smem = std::max<size_t>(i2_layout().dyn, 228u * 1024u / 2u + 1024u);
  auto kern = p.geo.window == kWinES ? k_interp2_tc<W, kWinES> : k_interp2_tc<W, kWinGauss>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kI2Threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm != 1) return cudaErrorInvalidConfiguration;
  kern<<<p.num_sms, kI2Threads, smem, st>>>(p.it_tmap, p.it_pinv, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_interp2_tc(const Plan& p, const void* in, void* out, cudaStream_t st) {
  switch (p.geo.W) {
    case 4: return launch_i2<4>(p, in, out, st);
    case 6: return launch_i2<6>(p, in, out, st);
    case 8: return launch_i2<8>(p, in, out, st);
    case 10: return launch_i2<10>(p, in, out, st);
    case 12: return launch_i2<12>(p, in, out, st);
    case 14: return launch_i2<14>(p, in, out, st);
    case 16: return launch_i2<16>(p, in, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cg
