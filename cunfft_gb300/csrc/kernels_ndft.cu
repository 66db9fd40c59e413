// kernels_ndft.cu -- direct NDFT and adjoint NDFT (FP64), shared-memory staged.
//
// Reference: src/cunfft_kernel.cu:1207-1345 (one thread per output, coefficients
// or nodes read from global memory, cos/sin per term).
//   forward  f_j   = sum_k f_hat_k e^{-2 pi i k.x_j}
//   adjoint  f_hat_k = sum_j f_j   e^{+2 pi i k.x_j}
// with k_t in [-N_t/2, N_t - N_t/2), lexicographic k (last dimension fastest).
//
// GB300 form.  Forward: a CTA stages 256 coefficients at a time in shared memory
// and every thread (one node) walks them; along the last dimension the phase is
// advanced by the rotation e^{-2 pi i x_last} and re-evaluated exactly with
// sincospi at each row start and every 64 terms, so the recurrence error stays
// at the 1e-15 level.  Adjoint: a CTA stages 256 nodes (x and f) and every
// thread (one coefficient) evaluates sincospi per term.
#include "runtime.h"

namespace cg {

constexpr int kNdftChunk = 256;
constexpr int kResync = 64;

__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
  return acc;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

__global__ void __launch_bounds__(256) k_ndft_forward(const double* __restrict__ x, const double2* __restrict__ fhat,
                                                      double2* __restrict__ f, Geom geo,
                                                      const int32_t* __restrict__ inst_off) {
  __shared__ double2 sfh[kNdftChunk];
  const int d = geo.d;
  const int inst = blockIdx.y;
  const int64_t j0 = inst_off[inst], j1 = inst_off[inst + 1];
  const double2* fh = fhat + (int64_t)inst * geo.Ntot;
  const int64_t Nlast = geo.N[d - 1];
  for (int64_t jb = j0 + (int64_t)blockIdx.x * blockDim.x; jb < j1; jb += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = jb + threadIdx.x;
    const bool on = j < j1;
    double xj[kMaxDim] = {0.0, 0.0, 0.0};
    if (on)
      for (int t = 0; t < d; ++t) xj[t] = x[j * d + t];
    double sr, cr;
    sincospi(-2.0 * xj[d - 1], &sr, &cr);
    const double2 rot = make_double2(cr, sr);
    double2 acc = make_double2(0.0, 0.0), ph = make_double2(1.0, 0.0);
    // split of the coefficient range over blockIdx.z (partial sums added atomically)
    const int64_t span = ((geo.Ntot + gridDim.z - 1) / gridDim.z + kNdftChunk - 1) / kNdftChunk * kNdftChunk;
    const int64_t c_lo = (int64_t)blockIdx.z * span, c_hi = min(geo.Ntot, c_lo + span);
    int64_t pos = c_lo % Nlast;  // position inside the current row of the last dimension
    for (int64_t c0 = c_lo; c0 < c_hi; c0 += kNdftChunk) {
      const int cn = (int)min((int64_t)kNdftChunk, c_hi - c0);
      __syncthreads();
      if (threadIdx.x < cn) sfh[threadIdx.x] = fh[c0 + threadIdx.x];
      __syncthreads();
      for (int s = 0; s < cn; ++s) {
        const int64_t kl = c0 + s;
        if (pos == 0 || (s & (kResync - 1)) == 0) {
          double kx = 0.0;
          int64_t rem = kl;
          for (int t = d - 1; t >= 0; --t) {
            const int64_t kt = rem % geo.N[t] - geo.N[t] / 2;
            rem /= geo.N[t];
            kx = fma((double)kt, xj[t], kx);
          }
          double sp, cp;
          sincospi(-2.0 * kx, &sp, &cp);
          ph = make_double2(cp, sp);
        }
        acc = cfma(sfh[s], ph, acc);
        ph = cmul(ph, rot);
        if (++pos == Nlast) pos = 0;
      }
    }
    if (on) {
      if (gridDim.z == 1) {
        f[j] = acc;
      } else {
        atomicAdd(&f[j].x, acc.x);
        atomicAdd(&f[j].y, acc.y);
      }
    }
  }
}

// kidx == nullptr: all N_total coefficients of every instance; otherwise the
// nsel coefficient indices kidx[] of instance blockIdx.y, written densely.
__global__ void __launch_bounds__(256) k_ndft_adjoint(const double* __restrict__ x, const double2* __restrict__ f,
                                                      double2* __restrict__ fhat, Geom geo,
                                                      const int32_t* __restrict__ inst_off,
                                                      const int64_t* __restrict__ kidx, int64_t nsel) {
  __shared__ double sx[kNdftChunk * kMaxDim];
  __shared__ double2 sf[kNdftChunk];
  const int d = geo.d;
  const int inst = blockIdx.y;
  const int64_t j0 = inst_off[inst], j1 = inst_off[inst + 1];
  const int64_t nout = kidx ? nsel : geo.Ntot;
  double2* out = fhat + (int64_t)inst * nout;
  for (int64_t kb = (int64_t)blockIdx.x * blockDim.x; kb < nout; kb += (int64_t)gridDim.x * blockDim.x) {
    const int64_t kl = kb + threadIdx.x;
    const bool on = kl < nout;
    double kk[kMaxDim] = {0.0, 0.0, 0.0};
    if (on) {
      int64_t rem = kidx ? kidx[kl] : kl;
      for (int t = d - 1; t >= 0; --t) {
        kk[t] = (double)(rem % geo.N[t] - geo.N[t] / 2);
        rem /= geo.N[t];
      }
    }
    double2 acc = make_double2(0.0, 0.0);
    // split of the node range over blockIdx.z (partial sums added atomically)
    const int64_t span = ((j1 - j0 + gridDim.z - 1) / gridDim.z + kNdftChunk - 1) / kNdftChunk * kNdftChunk;
    const int64_t n_lo = j0 + (int64_t)blockIdx.z * span, n_hi = min(j1, n_lo + span);
    for (int64_t c0 = n_lo; c0 < n_hi; c0 += kNdftChunk) {
      const int cn = (int)min((int64_t)kNdftChunk, n_hi - c0);
      __syncthreads();
      for (int e = threadIdx.x; e < cn * d; e += blockDim.x) sx[e] = x[c0 * d + e];
      if (threadIdx.x < cn) sf[threadIdx.x] = f[c0 + threadIdx.x];
      __syncthreads();
      for (int s = 0; s < cn; ++s) {
        double kx = 0.0;
        for (int t = 0; t < d; ++t) kx = fma(kk[t], sx[s * d + t], kx);
        double sp, cp;
        sincospi(2.0 * kx, &sp, &cp);
        acc = cfma(sf[s], make_double2(cp, sp), acc);
      }
    }
    if (on) {
      if (gridDim.z == 1) {
        out[kl] = acc;
      } else {
        atomicAdd(&out[kl].x, acc.x);
        atomicAdd(&out[kl].y, acc.y);
      }
    }
  }
}

// Few outputs (e.g. a 4096-node check of a large transform) would occupy a few
// SMs only: split the inner sum over up to 4 CTAs per SM, at least 4096 terms each.
static int ndft_splits(const Plan& p, int64_t blocks, int64_t inner) {
  const int64_t want = (int64_t)p.num_sms * 4;
  if (blocks >= want) return 1;
  int64_t s = (want + blocks - 1) / blocks;
  const int64_t cap = (inner + 4095) / 4096;
  if (s > cap) s = cap;
  if (s > 65535) s = 65535;
  return (int)(s < 1 ? 1 : s);
}

cudaError_t launch_ndft_forward(const Plan& p, const double* x, const void* fhat, void* f, cudaStream_t st) {
  int64_t maxM = 0;
  for (int i = 0; i < p.geo.batch; ++i) maxM = p.M_inst[i] > maxM ? p.M_inst[i] : maxM;
  if (maxM == 0) return cudaSuccess;
  int64_t bx = (maxM + 255) / 256;
  if (bx > (int64_t)p.num_sms * 8) bx = (int64_t)p.num_sms * 8;
  const int splits = ndft_splits(p, bx * p.geo.batch, p.geo.Ntot);
  if (splits > 1) {
    const cudaError_t e = cudaMemsetAsync(f, 0, sizeof(double2) * p.M, st);
    if (e != cudaSuccess) return e;
  }
  dim3 grid((unsigned)bx, (unsigned)p.geo.batch, (unsigned)splits);
  k_ndft_forward<<<grid, 256, 0, st>>>(x, (const double2*)fhat, (double2*)f, p.geo, p.bins.inst_off);
  return cudaGetLastError();
}

cudaError_t launch_ndft_adjoint(const Plan& p, const double* x, const void* f, void* fhat, cudaStream_t st,
                                const int64_t* kidx, int64_t nsel) {
  const int64_t nout = kidx ? nsel : p.geo.Ntot;
  if (nout == 0) return cudaSuccess;
  int64_t bx = (nout + 255) / 256;
  if (bx > (int64_t)p.num_sms * 8) bx = (int64_t)p.num_sms * 8;
  int64_t maxM = 0;
  for (int i = 0; i < p.geo.batch; ++i) maxM = p.M_inst[i] > maxM ? p.M_inst[i] : maxM;
  const int splits = ndft_splits(p, bx * p.geo.batch, maxM);
  if (splits > 1) {
    const cudaError_t e = cudaMemsetAsync(fhat, 0, sizeof(double2) * nout * p.geo.batch, st);
    if (e != cudaSuccess) return e;
  }
  dim3 grid((unsigned)bx, (unsigned)p.geo.batch, (unsigned)splits);
  k_ndft_adjoint<<<grid, 256, 0, st>>>(x, (const double2*)f, (double2*)fhat, p.geo, p.bins.inst_off, kidx, nsel);
  return cudaGetLastError();
}

}  // namespace cg
