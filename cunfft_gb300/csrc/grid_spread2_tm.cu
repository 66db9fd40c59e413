// grid_spread2_tm.cu -- launcher of the 2D FP32 tensor-core spreading kernel
// (kernels_spread2_tm.cuh).
#include <algorithm>

#include "kernels_spread2_tm.cuh"

namespace cg {

bool spread2_tm_supported(const Plan& p) {
  return p.prec == kF32 && !p.tl.use_global && spread2_tm_ok(p.geo.d, p.geo.W, p.tl.T[0], p.tl.T[1]);
}

// The kernel allocates all 512 tensor-memory columns; its dynamic shared memory is at
// least half of the SM's 228 KB, so that two CTAs never share an SM and tcgen05.alloc
// never waits.
static constexpr size_t kT2SmemFloor = 228u * 1024u / 2u + 1u;

template <int W>
static cudaError_t launch_t2(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (!spread2_tm_supported(p)) return cudaErrorInvalidConfiguration;
  const size_t smem = std::max<size_t>(t2_layout().total, kT2SmemFloor);
  auto kern = p.geo.window == kWinES ? k_spread2_tm<W, kWinES> : k_spread2_tm<W, kWinGauss>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kT2Threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm != 1) return cudaErrorInvalidConfiguration;
  e = spread_tc_permute(p, in, st);
  if (e != cudaSuccess) return e;
  kern<<<p.num_sms, kT2Threads, smem, st>>>((const float2*)in, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_spread2_tm(const Plan& p, const void* in, void* out, cudaStream_t st) {
  switch (p.geo.W) {
    case 4: return launch_t2<4>(p, in, out, st);
    case 6: return launch_t2<6>(p, in, out, st);
    case 8: return launch_t2<8>(p, in, out, st);
    case 10: return launch_t2<10>(p, in, out, st);
    case 12: return launch_t2<12>(p, in, out, st);
    case 14: return launch_t2<14>(p, in, out, st);
    case 16: return launch_t2<16>(p, in, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cg
