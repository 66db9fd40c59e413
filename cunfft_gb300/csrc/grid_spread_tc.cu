// grid_spread_tc.cu -- launcher of the tensor-core 3D FP32 spreading kernel.
#include <algorithm>

#include "kernels_spread_tc.cuh"

namespace cg {

bool spread_tc_supported(const Plan& p) {
  return (p.prec == kF32 && !p.tl.use_global && spread_tc_ok(p.geo.d, p.geo.W, p.tl.T[0])) ||
         spread2_tm_supported(p);
}

// Dynamic shared memory of one CTA.  Besides the kernel's own needs it is large
// enough that at most k = 512 / tmem_cols CTAs fit on one SM (228 KB of shared
// memory, 1 KB reserved per CTA), so the resident CTAs never ask for more than
// the SM's 512 tensor-memory columns and tcgen05.alloc never waits.
static constexpr size_t kSmemPerSm = 228u * 1024u;  // per SM; each resident CTA also reserves 1 KB
size_t spread_tc_smem_bytes(const Plan& p) {
  const TcLayout L = tc_layout(p.geo.W, p.tl.E[0]);
  const size_t k = 512u / L.tmem_cols;
  const size_t floor_bytes = kSmemPerSm / (k + 1) + 1;  // k + 1 CTAs of this size exceed the SM
  return L.total > floor_bytes ? L.total : floor_bytes;
}

// Samples in sorted order (fp[k] = f[sidx[k]]), so that the spreading kernel's
// per-batch record loads are contiguous, and their largest |Re|, |Im| into *fmax
// (float bits: the unsigned order of non-negative floats; zeroed before the launch).
__global__ void k_permute_samples(const float2* __restrict__ f, const int32_t* __restrict__ sidx, int64_t M,
                                  float2* __restrict__ fp, uint32_t* __restrict__ fmax) {
  float mx = 0.f;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < M; k += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = f[sidx[k]];
    fp[k] = v;
    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  const uint32_t m = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
  if ((threadIdx.x & 31) == 0 && m != 0u) atomicMax(fmax, m);
}

// Samples in sorted order, read contiguously by the kernels' record loads, and their
// largest component (the B scale).
cudaError_t spread_tc_permute(const Plan& p, const void* in, cudaStream_t st) {
  const int64_t M = p.bins.M;
  const int pblocks = (int)std::min<int64_t>((M + 255) / 256, (int64_t)p.num_sms * 16);
  cudaError_t e = cudaMemsetAsync(p.bins.fmax, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_permute_samples<<<pblocks, 256, 0, st>>>((const float2*)in, p.bins.sidx, M, (float2*)p.bins.fperm, p.bins.fmax);
  return cudaGetLastError();
}

template <int W>
static cudaError_t launch_tc(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (!spread_tc_supported(p)) return cudaErrorInvalidConfiguration;
  const size_t smem = spread_tc_smem_bytes(p);
  auto kern = p.geo.window == kWinES ? k_spread_tc<W, kWinES> : k_spread_tc<W, kWinGauss>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTcThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if ((size_t)per_sm * tc_layout(W, p.tl.E[0]).tmem_cols > 512u) return cudaErrorInvalidConfiguration;
  e = spread_tc_permute(p, in, st);
  if (e != cudaSuccess) return e;
  kern<<<p.num_sms * per_sm, kTcThreads, smem, st>>>((const float2*)in, (float2*)out, p.geo, p.tl, p.bins);
  return cudaGetLastError();
}

cudaError_t grid_launch_spread_tc(const Plan& p, const void* in, void* out, cudaStream_t st) {
  if (p.geo.d == 2) return grid_launch_spread2_tm(p, in, out, st);
  if (spread_tm_supported(p)) return grid_launch_spread_tm(p, in, out, st);
  switch (p.geo.W) {
    case 4: return launch_tc<4>(p, in, out, st);
    case 6: return launch_tc<6>(p, in, out, st);
    case 8: return launch_tc<8>(p, in, out, st);
    case 10: return launch_tc<10>(p, in, out, st);
    case 12: return launch_tc<12>(p, in, out, st);
    case 14: return launch_tc<14>(p, in, out, st);
    case 16: return launch_tc<16>(p, in, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cg
