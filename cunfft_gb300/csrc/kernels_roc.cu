// kernels_roc.cu -- roll-off correction (deconvolution) fused with zero-pad and crop.
//
// Forward  (src/cunfft_kernel.cu:240-412 + the cudaMemset of src/cunfft_wrapper.cu:34):
//   g[k mod n] = f_hat[k] * prod_t exp(fac_t k_t^2)  for k in I_N,  g = 0 elsewhere,
// written as one pass over the whole grid (no separate memset).
// Adjoint  (src/cunfft_kernel.cu:264-275, 318-343, 418-467):
//   f_hat[k] = g[k mod n] * prod_t exp(fac_t k_t^2).
// fac_t = pi^2 b_t / n_t^2 (src/cunfft.cu:87).  The factor tables are FP64 in both
// forms; the FP32 form multiplies the FP64 factor product, rounded once, into
// FP32 data.  Frequencies run over k_t in [-floor(N_t/2), N_t - floor(N_t/2)).
#include "runtime.h"

namespace cg {

template <typename T>
__global__ void k_roc_forward(const typename Cx<T>::t* __restrict__ fhat, typename Cx<T>::t* __restrict__ g,
                              Geom geo, const double* __restrict__ tab) {
  using C = typename Cx<T>::t;
  const int d = geo.d;
  const int64_t total = geo.ntot * geo.batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t inst = e / geo.ntot, gi = e - inst * geo.ntot;
    int64_t ci = 0;
    double fac = 1.0;
    bool inside = true;
    int64_t rem = gi, tab_base = 0;
    int64_t idx[kMaxDim];
    for (int t = d - 1; t >= 0; --t) {
      idx[t] = rem & (geo.n[t] - 1);
      rem >>= __ffsll(geo.n[t]) - 1;
    }
    for (int t = 0; t < d; ++t) {
      const int64_t Nt = geo.N[t], half = Nt / 2, i = idx[t];
      int64_t k;
      if (i < Nt - half) k = i;
      else if (i >= geo.n[t] - half) k = i - geo.n[t];
      else { inside = false; break; }
      const int64_t c = k + half;
      ci = ci * Nt + c;
      fac *= tab[tab_base + c];
      tab_base += Nt;
    }
    C out;
    if (inside) {
      C a = fhat[inst * geo.Ntot + ci];
      T s = (T)fac;
      out.x = a.x * s;
      out.y = a.y * s;
    } else {
      out.x = (T)0;
      out.y = (T)0;
    }
    g[e] = out;
  }
}

template <typename T>
__global__ void k_roc_adjoint(const typename Cx<T>::t* __restrict__ g, typename Cx<T>::t* __restrict__ fhat,
                              Geom geo, const double* __restrict__ tab) {
  using C = typename Cx<T>::t;
  const int d = geo.d;
  const int64_t total = geo.Ntot * geo.batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t inst = e / geo.Ntot, ci = e - inst * geo.Ntot;
    int64_t c[kMaxDim];
    int64_t rem = ci;
    for (int t = d - 1; t >= 0; --t) {
      c[t] = rem % geo.N[t];
      rem /= geo.N[t];
    }
    double fac = 1.0;
    int64_t gi = 0, tab_base = 0;
    for (int t = 0; t < d; ++t) {
      const int64_t k = c[t] - geo.N[t] / 2;
      gi = gi * geo.n[t] + (k & (geo.n[t] - 1));
      fac *= tab[tab_base + c[t]];
      tab_base += geo.N[t];
    }
    C a = g[inst * geo.ntot + gi];
    T s = (T)fac;
    C out;
    out.x = a.x * s;
    out.y = a.y * s;
    fhat[e] = out;
  }
}

static inline int roc_grid(const Plan& p, int64_t work) {
  int64_t b = (work + 255) / 256;
  int64_t cap = (int64_t)p.num_sms * 16;
  return (int)(b > cap ? cap : (b < 1 ? 1 : b));
}

cudaError_t launch_roc_forward(const Plan& p, const void* fhat, void* g, cudaStream_t st) {
  const int64_t work = p.geo.ntot * p.geo.batch;
  if (p.prec == kF64)
    k_roc_forward<double><<<roc_grid(p, work), 256, 0, st>>>((const double2*)fhat, (double2*)g, p.geo, p.roc_tab);
  else
    k_roc_forward<float><<<roc_grid(p, work), 256, 0, st>>>((const float2*)fhat, (float2*)g, p.geo, p.roc_tab);
  return cudaGetLastError();
}

cudaError_t launch_roc_adjoint(const Plan& p, const void* g, void* fhat, cudaStream_t st) {
  const int64_t work = p.geo.Ntot * p.geo.batch;
  if (p.prec == kF64)
    k_roc_adjoint<double><<<roc_grid(p, work), 256, 0, st>>>((const double2*)g, (double2*)fhat, p.geo, p.roc_tab);
  else
    k_roc_adjoint<float><<<roc_grid(p, work), 256, 0, st>>>((const float2*)g, (float2*)fhat, p.geo, p.roc_tab);
  return cudaGetLastError();
}

}  // namespace cg
