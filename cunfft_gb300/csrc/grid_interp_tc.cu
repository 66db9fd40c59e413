// grid_interp_tc.cu -- launcher of the tensor-core FP32 interpolation: the split of the
// grid into padded, per-plane scaled FP16 hi/lo planes (one kernel, one pass), then the
// TMA-fed kernel; the 2D form's rows and kernel are in grid_interp2_tc.cu.
#include <cudaTypedefs.h>

#include <algorithm>

#include "kernels_interp_tc.cuh"

namespace cg {

// the 2D form (grid_interp2_tc.cu)
bool interp2_tc_supported(const Plan& p);
cudaError_t interp2_tc_prepare(Plan& p, PFN_cuTensorMapEncodeTiled_v12000 enc);
cudaError_t grid_launch_interp2_tc(const Plan& p, const void* in, void* out, cudaStream_t st);

bool interp_tc_supported(const Plan& p) {
  if (p.geo.d == 2) return interp2_tc_supported(p);
  return p.prec == kF32 && !p.tl.use_global && interp_tc_ok(p.geo.d, p.geo.W, p.tl.T[0], p.geo.n[2]);
}

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point query
// (no link-time dependency on the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

void interp_tc_release(Plan& p) {
  cudaFree(p.it_split);
  cudaFree(p.it_pinv);
  p.it_split = nullptr;
  p.it_pinv = nullptr;
  p.it_ready = false;
}

// Split planes half [batch][4][P0][P1][P2s], plane scales float [batch][P0], and the
// 5-D map over the planes (dims P2s, P1, P0, component, instance; box 32 halves x E1
// rows x CH planes, 64-byte swizzle, zero fill outside).  Box rows are 64 bytes (32
// halves), the innermost box extent the swizzle allows; rows are multiples of 16
// bytes (P2s % 8 == 0).
cudaError_t interp_tc_prepare(Plan& p) {
  if (p.it_ready) return cudaSuccess;
  if (p.geo.d == 2) return interp2_tc_prepare(p, encode_tiled());
  const ItSplit sd = it_split_dims(p.geo);
  const size_t comp = (size_t)(sd.P0 * sd.P1 * sd.P2s);
  const size_t bytes = sizeof(__half) * 4 * comp * (size_t)p.geo.batch;
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_tiled();
  if (!enc) return cudaErrorNotSupported;
  if (!p.it_split) {
    cudaError_t e = plan_malloc(&p.it_split, bytes);
    if (e == cudaSuccess) e = plan_malloc(&p.it_pinv, sizeof(float) * (size_t)(sd.P0 * p.geo.batch));
    if (e != cudaSuccess) {
      interp_tc_release(p);
      return e;
    }
  }
  const int E1 = it_e1(p.geo.W), CH = it_ch(p.geo.W);
  const cuuint64_t dims[5] = {(cuuint64_t)sd.P2s, (cuuint64_t)sd.P1, (cuuint64_t)sd.P0, 4u, (cuuint64_t)p.geo.batch};
  const cuuint64_t strides[4] = {(cuuint64_t)(sd.P2s * 2), (cuuint64_t)(sd.P2s * sd.P1 * 2),
                                 (cuuint64_t)(comp * 2), (cuuint64_t)(4 * comp * 2)};
  const cuuint32_t box[5] = {(cuuint32_t)kItK, (cuuint32_t)E1, (cuuint32_t)CH, 1u, 1u};
  const cuuint32_t estr[5] = {1u, 1u, 1u, 1u, 1u};
  const CUresult r = enc(&p.it_tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, p.it_split, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  p.it_ready = true;
  return cudaSuccess;
}


template <int W>
static cudaError_t launch_it(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (!interp_tc_supported(p) || !p.it_ready) return cudaErrorInvalidConfiguration;
  const ItSplit sd = it_split_dims(p.geo);
  // one CTA per SM at a time over the padded planes: the planes being split stay in L2
  // between their two reads
  const int sblocks = (int)std::min<int64_t>(sd.P0 * p.geo.batch, (int64_t)p.num_sms);
  k_split_planes<<<sblocks, kItSplitThreads, 0, st>>>((const float2*)in, (__half*)p.it_split, p.it_pinv, p.geo, sd);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // 512 tensor-memory columns per CTA: at most one CTA per SM (more than half the
  // SM's 228 KB of shared memory), so tcgen05.alloc never waits
  const ItLayout L = it_layout();
  const size_t smem = L.dyn;
  static_assert(it_layout().dyn > 116u * 1024u, "one CTA per SM");
  auto kern = p.geo.window == kWinES ? k_interp_tc<W, kWinES> : k_interp_tc<W, kWinGauss>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kItThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm != 1) return cudaErrorInvalidConfiguration;
  kern<<<p.num_sms, kItThreads, smem, st>>>(p.it_tmap, p.it_pinv, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_interp_tc(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (p.geo.d == 2) return grid_launch_interp2_tc(p, in, out, st);
  switch (p.geo.W) {
    case 4: return launch_it<4>(p, in, out, st);
    case 6: return launch_it<6>(p, in, out, st);
    case 8: return launch_it<8>(p, in, out, st);
    case 10: return launch_it<10>(p, in, out, st);
    case 12: return launch_it<12>(p, in, out, st);
    case 14: return launch_it<14>(p, in, out, st);
    case 16: return launch_it<16>(p, in, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cg
