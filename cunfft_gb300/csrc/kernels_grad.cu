// kernels_grad.cu -- node-position gradient of the forward NFFT (derivative-of-window gridding).
//
// f_j = sum_l g[u + l] prod_t psi_t(c_t - l_t),  c_t = n_t x_t - u_t, so
//   d f_j / d x_{j,t} = n_t sum_l g[u + l] psi_t'(c_t - l_t) prod_{s != t} psi_s(c_s - l_s),
//   Gaussian psi(y) = K exp(-y^2/b): psi'(y) = -(2 y / b) psi(y);
//   ES psi(y) = exp(beta (s - 1)), s = sqrt(1 - y^2/alpha^2): psi'(y) = -psi(y) beta y / (alpha^2 s).
// The kernel evaluates the d partial derivatives on the same roll-off-corrected,
// FFT'd grid g as the forward transform and contracts them with the incoming
// gradient: grad_x[j, t] = Re(conj(grad_f_j) * d f_j / d x_{j,t}).
// No reference counterpart (the reference has no differentiable transform).
// One thread per node, FP64 node reduction and weights, grid read through L1/L2;
// accumulation in the plan's real type.
#include "runtime.h"

namespace cg {

template <typename T>
__global__ void __launch_bounds__(128) k_interp_grad(const double* __restrict__ x,
                                                     const typename Cx<T>::t* __restrict__ g,
                                                     const typename Cx<T>::t* __restrict__ grad_f,
                                                     double* __restrict__ grad_x, Geom geo,
                                                     const int32_t* __restrict__ inst_off, int64_t M) {
  using C = typename Cx<T>::t;
  const int d = geo.d, W = geo.W;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
    int inst = 0;
    if (geo.batch > 1) {
      int lo = 0, hi = geo.batch;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (inst_off[mid] <= j) lo = mid; else hi = mid;
      }
      inst = lo;
    }
    const C* gi = g + (int64_t)inst * geo.ntot;
    T w[kMaxDim][kMaxTaps], dw[kMaxDim][kMaxTaps];
    int64_t u[kMaxDim] = {0, 0, 0};
    for (int t = 0; t < d; ++t) {
      const double xt = x[j * d + t];
      const double nx = __dmul_rn(xt, (double)geo.n[t]);
      u[t] = (int64_t)__double2ll_rn(nx) - (signbit(xt) ? 1 : 0) - geo.m;
      const double c = __dsub_rn(nx, (double)u[t]);
      if (geo.window == kWinES) {
        // phi = exp(beta (s - 1)), s = sqrt(1 - y^2/alpha^2); dphi/dy = -phi beta y / (alpha^2 s)
        const double beta = geo.es_beta[t];
        for (int l = 0; l < W; ++l) {
          const double y = c - (double)l, z = 1.0 - (y * y) * geo.es_ia2;
          const double s = z > 0.0 ? sqrt(z) : 0.0;
          const double e = z > 0.0 ? exp(beta * (s - 1.0)) : 0.0;
          w[t][l] = (T)e;
          dw[t][l] = z > 0.0 ? (T)(-e * beta * y * geo.es_ia2 / s * (double)geo.n[t]) : (T)0;
        }
      } else {
        const double ib = 1.0 / geo.b[t];
        for (int l = 0; l < W; ++l) {
          const double y = c - (double)l;
          const double e = exp(-(y * y) * ib);
          w[t][l] = (T)e;
          dw[t][l] = (T)(-2.0 * y * ib * e * (double)geo.n[t]);
        }
      }
    }
    for (int t = d; t < kMaxDim; ++t) {
      w[t][0] = (T)1;
      dw[t][0] = (T)0;
    }
    const int W1 = d >= 2 ? W : 1, W2 = d >= 3 ? W : 1;
    // partial sums: p[t] = sum g * (derivative in dim t, plain weights elsewhere)
    T pr[kMaxDim] = {0, 0, 0}, pi[kMaxDim] = {0, 0, 0};
    for (int l0 = 0; l0 < W; ++l0) {
      const int64_t i0 = wrap_n(u[0] + l0, geo.n[0]);
      for (int l1 = 0; l1 < W1; ++l1) {
        const int64_t i1 = d >= 2 ? wrap_n(u[1] + l1, geo.n[1]) : 0;
        // inner sums over the last dimension: plain and derivative weights
        T ar = 0, ai = 0, br = 0, bi = 0;
        for (int l2 = 0; l2 < W2; ++l2) {
          const int64_t i2 = d >= 3 ? wrap_n(u[2] + l2, geo.n[2]) : 0;
          int64_t gidx = i0;
          if (d >= 2) gidx = gidx * geo.n[1] + i1;
          if (d >= 3) gidx = gidx * geo.n[2] + i2;
          const C v = gi[gidx];
          const T a = d >= 3 ? w[2][l2] : (T)1, b = d >= 3 ? dw[2][l2] : (T)0;
          ar += a * v.x; ai += a * v.y;
          br += b * v.x; bi += b * v.y;
        }
        // (ar, ai): plain in last dim; (br, bi): derivative in dim 2
        const T w1 = d >= 2 ? w[1][l1] : (T)1, dw1 = d >= 2 ? dw[1][l1] : (T)0;
        const T w0 = w[0][l0], dw0 = dw[0][l0];
        pr[0] += dw0 * w1 * ar; pi[0] += dw0 * w1 * ai;
        if (d >= 2) { pr[1] += w0 * dw1 * ar; pi[1] += w0 * dw1 * ai; }
        if (d >= 3) { pr[2] += w0 * w1 * br; pi[2] += w0 * w1 * bi; }
      }
    }
    const C gf = grad_f[j];
    const double nrm = geo.norm;
    for (int t = 0; t < d; ++t)
      grad_x[j * d + t] = nrm * ((double)gf.x * (double)pr[t] + (double)gf.y * (double)pi[t]);
  }
}

cudaError_t launch_interp_grad(const Plan& p, const void* g, const void* grad_f, double* grad_x, cudaStream_t st) {
  if (p.M == 0) return cudaSuccess;
  int64_t b = (p.M + 127) / 128;
  if (b > (int64_t)p.num_sms * 16) b = (int64_t)p.num_sms * 16;
  if (p.prec == kF64)
    k_interp_grad<double><<<(unsigned)b, 128, 0, st>>>(p.x, (const double2*)g, (const double2*)grad_f, grad_x, p.geo,
                                                       p.bins.inst_off, p.M);
  else
    k_interp_grad<float><<<(unsigned)b, 128, 0, st>>>(p.x, (const float2*)g, (const float2*)grad_f, grad_x, p.geo,
                                                      p.bins.inst_off, p.M);
  return cudaGetLastError();
}

}  // namespace cg
