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

// log2 of the grid sizes when every one is a power of two, computed on the host
struct RocShifts {
  int lg_n[kMaxDim];
  int lg_ntot;
};

// Frequency slot c = k + floor(N/2) of grid index i along a dimension (k = i or i - n),
// or -1 when i lies in the zero padding.
__device__ __forceinline__ int64_t roc_slot(int64_t i, int64_t N, int64_t n) {
  const int64_t half = N / 2;
  if (i < N - half) return i + half;
  if (i >= n - half) return i - n + half;
  return -1;
}

// EPT consecutive grid points per thread (2 when the last grid size is even, so a
// pair never leaves its row; 1 otherwise); integer decoding by shifts and masks when
// every grid size is a power of two (P2), by division otherwise, and the FP64 factor
// product, in the order dimension 0, 1, ..., only for points inside I_N.
template <typename T, int EPT, bool P2>
__global__ void k_roc_forward(const typename Cx<T>::t* __restrict__ fhat, typename Cx<T>::t* __restrict__ g,
                              Geom geo, const double* __restrict__ tab, RocShifts sh) {
  using C = typename Cx<T>::t;
  const int d = geo.d;
  const int64_t total2 = geo.ntot * geo.batch / EPT;
  const int64_t n_last = geo.n[d - 1], N_last = geo.N[d - 1];
  for (int64_t e2 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e2 < total2;
       e2 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = EPT * e2;
    const int64_t inst = P2 ? e >> sh.lg_ntot : e / geo.ntot;
    const int64_t gi = P2 ? e & (geo.ntot - 1) : e - inst * geo.ntot;
    const int64_t i_last = P2 ? gi & (n_last - 1) : gi % n_last;
    int64_t rest = P2 ? gi >> sh.lg_n[d - 1] : gi / n_last;
    // leading dimensions 0 .. d-2
    int64_t lead_idx[kMaxDim];
    for (int t = d - 2; t >= 0; --t) {
      if (P2) {
        lead_idx[t] = rest & (geo.n[t] - 1);
        rest >>= sh.lg_n[t];
      } else {
        const int64_t q = rest / geo.n[t];
        lead_idx[t] = rest - q * geo.n[t];
        rest = q;
      }
    }
    bool lead_in = true;
    int64_t ci = 0, tab_base = 0;
    double fac = 1.0;
    for (int t = 0; t < d - 1 && lead_in; ++t) {
      const int64_t c = roc_slot(lead_idx[t], geo.N[t], geo.n[t]);
      if (c < 0) {
        lead_in = false;
      } else {
        ci = ci * geo.N[t] + c;
        fac *= tab[tab_base + c];
        tab_base += geo.N[t];
      }
    }
    C out[EPT];
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
      out[u].x = (T)0;
      out[u].y = (T)0;
      const int64_t c = lead_in ? roc_slot(i_last + u, N_last, n_last) : -1;
      if (c >= 0) {
        const C a = fhat[inst * geo.Ntot + ci * N_last + c];
        const T s = (T)(fac * tab[tab_base + c]);
        out[u].x = a.x * s;
        out[u].y = a.y * s;
      }
    }
#pragma unroll
    for (int u = 0; u < EPT; ++u) g[e + u] = out[u];
  }
}

// Coefficient crop; 32-bit index arithmetic when the coefficient count allows it.
template <typename T, typename I>
__global__ void k_roc_adjoint(const typename Cx<T>::t* __restrict__ g, typename Cx<T>::t* __restrict__ fhat,
                              Geom geo, const double* __restrict__ tab) {
  using C = typename Cx<T>::t;
  const int d = geo.d;
  const I Ntot = (I)geo.Ntot;
  const I total = Ntot * (I)geo.batch;
  for (I e = blockIdx.x * (I)blockDim.x + threadIdx.x; e < total; e += (I)gridDim.x * blockDim.x) {
    const I inst = geo.batch > 1 ? e / Ntot : (I)0, ci = e - inst * Ntot;
    I c[kMaxDim];
    I rem = ci;
    for (int t = d - 1; t >= 0; --t) {
      const I Nt = (I)geo.N[t];
      const I q = rem / Nt;
      c[t] = rem - q * Nt;
      rem = q;
    }
    double fac = 1.0;
    int64_t gidx = 0, tab_base = 0;
    for (int t = 0; t < d; ++t) {
      const int64_t k = (int64_t)c[t] - geo.N[t] / 2;
      gidx = gidx * geo.n[t] + (k < 0 ? k + geo.n[t] : k);  // |k| <= N_t / 2 <= n_t / 2
      fac *= tab[tab_base + c[t]];
      tab_base += geo.N[t];
    }
    const C a = g[(int64_t)inst * geo.ntot + gidx];
    const T s = (T)fac;
    C out;
    out.x = a.x * s;
    out.y = a.y * s;
    fhat[e] = out;
  }
}

static bool all_pow2(const Geom& geo) {
  for (int t = 0; t < kMaxDim; ++t)
    if ((geo.n[t] & (geo.n[t] - 1)) != 0) return false;
  return true;
}

static RocShifts roc_shifts(const Geom& geo) {
  RocShifts sh{};
  for (int t = 0; t < kMaxDim; ++t) {
    int l = 0;
    while (((int64_t)1 << l) < geo.n[t]) ++l;
    sh.lg_n[t] = l;
  }
  int l = 0;
  while (((int64_t)1 << l) < geo.ntot) ++l;
  sh.lg_ntot = l;
  return sh;
}

static inline int roc_grid(const Plan& p, int64_t work) {
  int64_t b = (work + 255) / 256;
  int64_t cap = (int64_t)p.num_sms * 16;
  return (int)(b > cap ? cap : (b < 1 ? 1 : b));
}

template <typename T>
static cudaError_t launch_roc_fwd_t(const Plan& p, bool pairs, bool p2, int blocks, const void* fhat, void* g,
                                   const RocShifts& sh, cudaStream_t st) {
  using C = typename Cx<T>::t;
  const C* in = (const C*)fhat;
  C* out = (C*)g;
  if (pairs && p2) k_roc_forward<T, 2, true><<<blocks, 256, 0, st>>>(in, out, p.geo, p.roc_tab, sh);
  else if (pairs) k_roc_forward<T, 2, false><<<blocks, 256, 0, st>>>(in, out, p.geo, p.roc_tab, sh);
  else if (p2) k_roc_forward<T, 1, true><<<blocks, 256, 0, st>>>(in, out, p.geo, p.roc_tab, sh);
  else k_roc_forward<T, 1, false><<<blocks, 256, 0, st>>>(in, out, p.geo, p.roc_tab, sh);
  return cudaGetLastError();
}

cudaError_t launch_roc_forward(const Plan& p, const void* fhat, void* g, cudaStream_t st) {
  const bool pairs = (p.geo.n[p.geo.d - 1] & 1) == 0;
  const int64_t work = p.geo.ntot * p.geo.batch / (pairs ? 2 : 1);
  const RocShifts sh = roc_shifts(p.geo);
  const int blocks = roc_grid(p, work);
  if (p.prec == kF64) return launch_roc_fwd_t<double>(p, pairs, all_pow2(p.geo), blocks, fhat, g, sh, st);
  return launch_roc_fwd_t<float>(p, pairs, all_pow2(p.geo), blocks, fhat, g, sh, st);
}

cudaError_t launch_roc_adjoint(const Plan& p, const void* g, void* fhat, cudaStream_t st) {
  const int64_t work = p.geo.Ntot * p.geo.batch;
  const bool small = work < ((int64_t)1 << 31);
  if (p.prec == kF64) {
    if (small)
      k_roc_adjoint<double, uint32_t><<<roc_grid(p, work), 256, 0, st>>>((const double2*)g, (double2*)fhat, p.geo, p.roc_tab);
    else
      k_roc_adjoint<double, int64_t><<<roc_grid(p, work), 256, 0, st>>>((const double2*)g, (double2*)fhat, p.geo, p.roc_tab);
  } else {
    if (small)
      k_roc_adjoint<float, uint32_t><<<roc_grid(p, work), 256, 0, st>>>((const float2*)g, (float2*)fhat, p.geo, p.roc_tab);
    else
      k_roc_adjoint<float, int64_t><<<roc_grid(p, work), 256, 0, st>>>((const float2*)g, (float2*)fhat, p.geo, p.roc_tab);
  }
  return cudaGetLastError();
}

}  // namespace cg
