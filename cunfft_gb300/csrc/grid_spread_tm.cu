// grid_spread_tm.cu -- launcher of the 3D FP32 spreading kernel with the A operand in
// tensor memory (kernels_spread_tm.cuh).
#include <algorithm>

#include "kernels_spread_tm.cuh"

namespace cg {

bool spread_tm_supported(const Plan& p) {
  return p.prec == kF32 && !p.tl.use_global && spread_tm_ok(p.geo.d, p.geo.W, p.tl.T[0], p.tl.E[0]);
}

// The kernel allocates all 512 tensor-memory columns; its dynamic shared memory is at
// least half of the SM's 228 KB, so that two CTAs never share an SM and tcgen05.alloc
// never waits.
static constexpr size_t kTmSmemFloor = 228u * 1024u / 2u + 1u;

template <int W>
static cudaError_t launch_tm(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (!spread_tm_supported(p)) return cudaErrorInvalidConfiguration;
  const size_t smem = std::max<size_t>(tm_layout(W, p.tl.E[0]).total, kTmSmemFloor);
  auto kern = p.geo.window == kWinES ? k_spread_tm<W, kWinES> : k_spread_tm<W, kWinGauss>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTmThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm != 1) return cudaErrorInvalidConfiguration;
  e = spread_tc_permute(p, in, st);
  if (e != cudaSuccess) return e;
  kern<<<p.num_sms, kTmThreads, smem, st>>>((const float2*)in, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_spread_tm(const Plan& p, const void* in, void* out, cudaStream_t st) {
  switch (p.geo.W) {
    case 4: return launch_tm<4>(p, in, out, st);
    case 6: return launch_tm<6>(p, in, out, st);
    case 8: return launch_tm<8>(p, in, out, st);
    case 10: return launch_tm<10>(p, in, out, st);
    case 12: return launch_tm<12>(p, in, out, st);
    case 14: return launch_tm<14>(p, in, out, st);
    case 16: return launch_tm<16>(p, in, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cg
