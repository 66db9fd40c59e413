// grid_dispatch.cu -- selects the gridding kernel instance for the plan's tap count.
#include "kernels_grid.cuh"

namespace cg {

#define CG_DECL(W) cudaError_t grid_launch_w##W(const Plan&, bool, const void*, void*, cudaStream_t);
CG_DECL(4) CG_DECL(6) CG_DECL(8) CG_DECL(10) CG_DECL(12) CG_DECL(14) CG_DECL(16) CG_DECL(18)
CG_DECL(20) CG_DECL(22) CG_DECL(24) CG_DECL(26) CG_DECL(28) CG_DECL(30) CG_DECL(32)
#undef CG_DECL

bool gridding_supported(int d, int W) { return d >= 1 && d <= 3 && W >= 4 && W <= 32 && (W % 2) == 0; }

// Larger of the interpolation and spreading kernels' shared-memory needs.
size_t gridding_smem_bytes(const Plan& p) {
  const int d = p.geo.d, W = p.geo.W;
  const size_t real = p.prec == kF64 ? 8 : 4;
  const int nwarps = p.tl.threads / 32;
  const size_t a = grid_extra_smem(d, W, real, nwarps, p.tl.smem_tile, false);
  const size_t b = grid_extra_smem(d, W, real, nwarps, p.tl.smem_tile, true);
  return p.tl.smem_tile + (a > b ? a : b);
}

cudaError_t grid_launch_global(const Plan&, bool, const void*, void*, cudaStream_t);

static cudaError_t dispatch(const Plan& p, bool spread, const void* in, void* out, cudaStream_t st) {
  if (p.tl.use_global) return grid_launch_global(p, spread, in, out, st);
  if (spread && p.tl.spread_kernel == CUNFFT_X_SPREAD_TENSOR) return grid_launch_spread_tc(p, in, out, st);
  if (!spread && p.tl.interp_kernel == CUNFFT_X_INTERP_TENSOR) return grid_launch_interp_tc(p, in, out, st);
  if (spread && p.tl.spread_kernel == CUNFFT_X_SPREAD_REGISTER) return grid_launch_spread_reg(p, in, out, st);
  switch (p.geo.W) {
#define CG_CASE(W) case W: return grid_launch_w##W(p, spread, in, out, st);
    CG_CASE(4) CG_CASE(6) CG_CASE(8) CG_CASE(10) CG_CASE(12) CG_CASE(14) CG_CASE(16) CG_CASE(18)
    CG_CASE(20) CG_CASE(22) CG_CASE(24) CG_CASE(26) CG_CASE(28) CG_CASE(30) CG_CASE(32)
#undef CG_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_interp(const Plan& p, const void* g, void* f, cudaStream_t st) {
  if (p.bins.M == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(p.bins.work, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  return dispatch(p, false, g, f, st);
}

cudaError_t launch_spread(const Plan& p, const void* f, void* g, cudaStream_t st) {
  if (p.bins.M == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(p.bins.work + 1, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  return dispatch(p, true, f, g, st);
}

}  // namespace cg
