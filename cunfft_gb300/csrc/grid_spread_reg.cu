// grid_spread_reg.cu -- launcher of the register-tile 3D FP32 spreading kernel.
#include "kernels_spread_reg.cuh"

namespace cg {

template <int W>
static cudaError_t launch_reg(const Plan& p, const void* in, void* out, cudaStream_t st) {
  const int threads = 32 * p.tl.E[0];
  if (!spread_reg_ok(p.geo.d, W, p.tl.T[0]) || threads > spread_reg_threads_max<W>()) return cudaErrorInvalidConfiguration;
  const size_t smem = spread_reg_smem<W>(p.tl.smem_tile);
  auto kern = k_spread_reg<W>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kern<<<p.num_sms * per_sm, threads, smem, st>>>((const float2*)in, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

size_t spread_reg_smem_bytes(const Plan& p) {
  switch (p.geo.W) {
    case 4: return spread_reg_smem<4>(p.tl.smem_tile);
    case 6: return spread_reg_smem<6>(p.tl.smem_tile);
    case 8: return spread_reg_smem<8>(p.tl.smem_tile);
    case 10: return spread_reg_smem<10>(p.tl.smem_tile);
    case 12: return spread_reg_smem<12>(p.tl.smem_tile);
    case 14: return spread_reg_smem<14>(p.tl.smem_tile);
    case 16: return spread_reg_smem<16>(p.tl.smem_tile);
    default: return 0;
  }
}

bool spread_reg_supported(const Plan& p) {
  return p.prec == kF32 && !p.tl.use_global && spread_reg_ok(p.geo.d, p.geo.W, p.tl.T[0]);
}

cudaError_t grid_launch_spread_reg(const Plan& p, const void* in, void* out, cudaStream_t st) {
  switch (p.geo.W) {
    case 4: return launch_reg<4>(p, in, out, st);
    case 6: return launch_reg<6>(p, in, out, st);
    case 8: return launch_reg<8>(p, in, out, st);
    case 10: return launch_reg<10>(p, in, out, st);
    case 12: return launch_reg<12>(p, in, out, st);
    case 14: return launch_reg<14>(p, in, out, st);
    case 16: return launch_reg<16>(p, in, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cg
