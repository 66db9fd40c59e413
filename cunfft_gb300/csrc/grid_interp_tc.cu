// grid_interp_tc.cu -- launcher of the tensor-core 3D FP32 interpolation kernel.
#include "kernels_interp_tc.cuh"

namespace cg {

bool interp_tc_supported(const Plan& p) {
  return p.prec == kF32 && !p.tl.use_global && interp_tc_ok(p.geo.d, p.geo.W, p.tl.T[0], p.geo.n[2]);
}

template <int W>
static cudaError_t launch_it(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (!interp_tc_supported(p)) return cudaErrorInvalidConfiguration;
  // 512 tensor-memory columns per CTA: at most one CTA per SM (more than half the
  // SM's 228 KB of shared memory), so tcgen05.alloc never waits
  const ItLayout L = it_layout(W);
  const size_t smem = L.total > 116u * 1024u + 1u ? L.total : 116u * 1024u + 1u;
  auto kern = p.geo.window == kWinES ? k_interp_tc<W, kWinES> : k_interp_tc<W, kWinGauss>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kItThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm != 1) return cudaErrorInvalidConfiguration;
  kern<<<p.num_sms, kItThreads, smem, st>>>((const float2*)in, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_interp_tc(const Plan& p, const void* in, void* out, cudaStream_t st) {
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
