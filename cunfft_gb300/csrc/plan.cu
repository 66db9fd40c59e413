// plan.cu -- plan life cycle and transform sequencing (host side).
//
// Stage order (reference src/cunfft.cu:196-224, src/cunfft_wrapper.cu):
//   forward:  roll-off + zero-pad  ->  FFT (e^-)  ->  interpolation
//   adjoint:  clear grid -> spreading ->  FFT (e^+) ->  crop + roll-off
// All stages are asynchronous on the plan's stream; no stage synchronises.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "runtime.h"

namespace cg {

int set_status(Plan* p, int code, const char* fmt, ...) {
  if (p) {
    p->last_status = code;
    if (code != CUNFFT_X_SUCCESS && fmt) {
      va_list ap;
      va_start(ap, fmt);
      vsnprintf(p->last_msg, sizeof(p->last_msg), fmt, ap);
      va_end(ap);
    } else if (code == CUNFFT_X_SUCCESS) {
      p->last_msg[0] = 0;
    }
  }
  return code;
}

int check_cuda(Plan* p, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return CUNFFT_X_SUCCESS;
  const int code = e == cudaErrorMemoryAllocation ? CUNFFT_X_ALLOC_FAILED : CUNFFT_X_CUDA_ERROR;
  return set_status(p, code, "%s: %s", what, cudaGetErrorString(e));
}

int check_cufft(Plan* p, cufftResult r, const char* what) {
  if (r == CUFFT_SUCCESS) return CUNFFT_X_SUCCESS;
  return set_status(p, r == CUFFT_ALLOC_FAILED ? CUNFFT_X_ALLOC_FAILED : CUNFFT_X_CUFFT_ERROR,
                    "%s: cuFFT error %d", what, (int)r);
}

// Fault points of the error-path tests: the environment value k (0 or unset: off)
// selects the k-th call of the process, counted from 1.
static long fault_point_env(const char* name) {
  const char* v = getenv(name);
  return v ? atol(v) : 0;
}
static std::atomic<long> g_alloc_calls{0}, g_fft_calls{0};

cudaError_t plan_malloc(void** ptr, size_t bytes) {
  static const long k = fault_point_env("CUNFFT_X_FAULT_ALLOC");
  if (k > 0 && g_alloc_calls.fetch_add(1) + 1 == k) {
    *ptr = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(ptr, bytes);
}

bool plan_fft_fault() {
  static const long k = fault_point_env("CUNFFT_X_FAULT_CUFFT");
  return k > 0 && g_fft_calls.fetch_add(1) + 1 == k;
}

static bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

static size_t elem_bytes(const Plan* p) { return p->prec == kF64 ? 16 : 8; }

static void free_bins(Plan* p) {
  Bins& B = p->bins;
  cudaFree(B.sidx);
  cudaFree(B.soff);
  cudaFree(B.sfrac);
  cudaFree(B.fperm);
  cudaFree(B.tile_rank);
  cudaFree(B.count);
  cudaFree(B.tile_off);
  cudaFree(B.item_off);
  cudaFree(B.items);
  cudaFree(B.scount);
  cudaFree(B.sub_pre);
  cudaFree(B.icount);
  cudaFree(B.iitem_off);
  cudaFree(B.iscratch);
  cudaFree(B.iitems);
  B.sidx = nullptr; B.soff = nullptr; B.sfrac = nullptr; B.tile_rank = nullptr; B.fperm = nullptr;
  B.count = nullptr; B.tile_off = nullptr; B.item_off = nullptr; B.items = nullptr;
  B.scount = nullptr; B.sub_pre = nullptr; B.icount = nullptr; B.iitem_off = nullptr; B.iscratch = nullptr;
  B.iitems = nullptr;
  B.max_iitems = 0;
  p->bins_capacity_M = -1;
  p->bins_capacity_tiles = -1;
  p->bins_capacity_keys = -1;
}

// Default tile extents.  For d >= 2 only the outermost extent T0 is free: the
// inner extents are the kernels' compile-time values (clamped to the grid).
// FP32 3D tiles (8 x 8 x 16) leave room for two CTAs per SM.
static void default_tiles(const Plan* p, int* T) {
  const int d = p->geo.d, W = p->geo.W;
  // 2D FP32 with 2m+2 <= 16: 64 x 64 tiles, the largest the tensor-core spreading covers
  // (E0 = 63 + W rows of its 128-row MMA)
  T[0] = d == 1 ? 2048 : (d == 2 ? (p->prec == kF32 && W <= 16 ? 64 : 32) : (p->prec == kF32 ? 8 : 4));
  if (d == 2) T[1] = fixed_t_last(2, W);
  if (d == 3) {
    T[1] = fixed_t_mid(3, W);
    T[2] = fixed_t_last(3, W);
  }
}

static Tiling make_tiling(const Plan* p, const int* T, int chunk) {
  const int d = p->geo.d, W = p->geo.W;
  Tiling tl{};
  for (int t = 0; t < kMaxDim; ++t) {
    tl.T[t] = t < d ? T[t] : 1;
    tl.nb[t] = t < d ? (int)((p->geo.n[t] + T[t] - 1) / T[t]) : 1;  // the last tile may be partial
    tl.E[t] = t < d ? T[t] + W - 1 : 1;
  }
  // inner strides are the kernels' compile-time values (inner tiles may be
  // smaller than the fixed extents when the grid is small)
  int64_t elems;
  if (d == 1) {
    tl.S = tl.E[0];
    tl.R1 = 1;
    elems = tl.S;
  } else if (d == 2) {
    tl.S = fixed_row_stride(2, W);
    tl.R1 = 1;
    elems = (int64_t)tl.E[0] * tl.S;
  } else {
    tl.S = fixed_row_stride(3, W);
    tl.R1 = fixed_t_mid(3, W) + W - 1;
    elems = (int64_t)tl.E[0] * tl.R1 * tl.S;
  }
  tl.smem_tile = (size_t)elems * elem_bytes(p);
  tl.smem_tile = (tl.smem_tile + 15) / 16 * 16;
  tl.tiles_per_inst = (int64_t)tl.nb[0] * tl.nb[1] * tl.nb[2];
  tl.tiles_total = tl.tiles_per_inst * p->geo.batch;
  tl.threads = 256;
  // 2D FP32 (2m+2 <= 16, the tensor-core spreading): 256-node items keep each tensor-memory
  // accumulation short (its FP32 sums drift with their length; with a tile's nodes ordered
  // by sub-tile, the nodes of one item overlap in most of their windows) and balance the
  // CTAs better.  On the batched 2D workload 512 and 256 spread equally fast, 256 at 0.64
  // times the error against the FP64 form.
  const bool t2 = d == 2 && p->prec == kF32 && W <= 16;
  tl.chunk = chunk > 0 ? chunk : (d == 3 ? 1024 : (t2 ? 256 : 2048));
  tl.use_global = 0;
  tl.ns = 1;  // no sub-bins unless the plan asks for them (plan_choose_tiling)
  return tl;
}

static size_t smem_of(const Plan* p, const Tiling& tl) {
  Plan q = *p;  // shallow copy for the size computation only
  q.tl = tl;
  return gridding_smem_bytes(q);
}

// Spreading kernel for the plan's current tiling under a request (plan_set_spread_kernel).
static int pick_spread_kernel(const Plan& p, int mode) {
  if (p.tl.use_global) return CUNFFT_X_SPREAD_GLOBAL;
  const bool tc = spread_tc_supported(p), reg = spread_reg_supported(p);
  if (mode == CUNFFT_X_SPREAD_TENSOR) return tc ? CUNFFT_X_SPREAD_TENSOR : CUNFFT_X_SPREAD_SHARED;
  if (mode == CUNFFT_X_SPREAD_REGISTER) return reg ? CUNFFT_X_SPREAD_REGISTER : CUNFFT_X_SPREAD_SHARED;
  if (mode == CUNFFT_X_SPREAD_SHARED) return CUNFFT_X_SPREAD_SHARED;
  return tc ? CUNFFT_X_SPREAD_TENSOR : (reg ? CUNFFT_X_SPREAD_REGISTER : CUNFFT_X_SPREAD_SHARED);
}

// Interpolation kernel for the plan's current tiling under a request (plan_set_interp_kernel).
static int pick_interp_kernel(const Plan& p, int mode) {
  if (p.tl.use_global) return CUNFFT_X_INTERP_GLOBAL;
  if (mode == CUNFFT_X_INTERP_SHARED) return CUNFFT_X_INTERP_SHARED;
  return interp_tc_supported(p) ? CUNFFT_X_INTERP_TENSOR : CUNFFT_X_INTERP_SHARED;
}

// Tile extents: the caller's (or the defaults), clamped to the grid.  When the
// padded tile does not fit in shared memory the largest extent is halved until it
// does; when even 1-cell tiles do not fit (wide windows in 3D), the gridding runs
// on the global-memory kernels with the default tiles as work items.
int plan_choose_tiling(Plan* p, const int* Tin, int chunk) {
  const int d = p->geo.d;
  const size_t kMaxSmem = 227 * 1024;
  int T[kMaxDim] = {1, 1, 1};
  default_tiles(p, T);
  if (Tin && Tin[0] > 0) {
    const int tmax = d == 3 ? 1024 : (d == 2 ? 32768 : (1 << 30));  // packed offset: 30/d bits per dim
    if (!is_pow2(Tin[0]) || Tin[0] > tmax)
      return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "tile extent %d is not a power of two <= %d", Tin[0], tmax);
    T[0] = Tin[0];
  }
  for (int t = 0; t < d; ++t)
    while (T[t] > p->geo.n[t]) T[t] >>= 1;  // powers of two, at most the grid size
  Tiling tl = make_tiling(p, T, chunk);
  while (smem_of(p, tl) > kMaxSmem && T[0] > 1) {
    T[0] /= 2;
    tl = make_tiling(p, T, chunk);
  }
  if (smem_of(p, tl) > kMaxSmem) {
    default_tiles(p, T);
    for (int t = 0; t < d; ++t)
      while (T[t] > p->geo.n[t]) T[t] >>= 1;
    tl = make_tiling(p, T, chunk);
    tl.use_global = 1;
    tl.threads = 128;
  }
  if (tl.tiles_total >= (int64_t)1 << 31) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "too many tiles");
  interp2_tc_subbins(*p, tl);
  p->tl = tl;
  p->it_ready = false;  // the interpolation's TMA boxes follow the tile extents: encoded again before use
  p->tl.spread_kernel = pick_spread_kernel(*p, p->spread_mode);
  p->tl.interp_kernel = pick_interp_kernel(*p, p->interp_mode);
  p->bins.valid = 0;
  return CUNFFT_X_SUCCESS;
}

int plan_interp_kernel(const Plan* p) { return p->tl.interp_kernel; }

int plan_set_interp_kernel(Plan* p, int kind) {
  if (kind != CUNFFT_X_INTERP_AUTO && kind != CUNFFT_X_INTERP_SHARED && kind != CUNFFT_X_INTERP_TENSOR)
    return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "unknown interpolation kernel %d", kind);
  if (kind == CUNFFT_X_INTERP_TENSOR && !interp_tc_supported(*p))
    return set_status(p, CUNFFT_X_UNSUPPORTED,
                      "tensor-core interpolation needs FP32 and 2m+2 <= 16, and in 3D an outer tile extent <= 16 "
                      "and n_3 divisible by 8, in 2D an inner tile extent >= 16 and n_2 divisible by 8");
  p->interp_mode = kind;
  p->tl.interp_kernel = pick_interp_kernel(*p, kind);
  ++p->node_gen;
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_spread_kernel(const Plan* p) { return p->tl.spread_kernel; }

// The kernel choice changes only the spreading launch, not the bins; captured
// graphs are invalidated through node_gen.
int plan_set_spread_kernel(Plan* p, int kind) {
  if (kind != CUNFFT_X_SPREAD_AUTO && kind != CUNFFT_X_SPREAD_SHARED && kind != CUNFFT_X_SPREAD_REGISTER &&
      kind != CUNFFT_X_SPREAD_TENSOR)
    return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "unknown spreading kernel %d", kind);
  if (kind == CUNFFT_X_SPREAD_REGISTER && !spread_reg_supported(*p))
    return set_status(p, CUNFFT_X_UNSUPPORTED,
                      "register spreading needs d = 3, FP32, 2m+2 <= 16 and an outer tile extent <= 8");
  if (kind == CUNFFT_X_SPREAD_TENSOR && !spread_tc_supported(*p))
    return set_status(p, CUNFFT_X_UNSUPPORTED,
                      "tensor-core spreading needs FP32, 2m+2 <= 16 and d = 3 with an outer tile extent <= 16 "
                      "or d = 2 with tile extents <= 64");
  p->spread_mode = kind;
  p->tl.spread_kernel = pick_spread_kernel(*p, kind);
  ++p->node_gen;
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

// Gauss-Legendre nodes and weights on [-1, 1]: roots of P_q by Newton's method
// from the asymptotic guess cos(pi (i + 3/4) / (q + 1/2)), P_q and P_q' by the
// three-term recurrence, weights 2 / ((1 - z^2) P_q'(z)^2).
static void gauss_legendre(int q, std::vector<double>& x, std::vector<double>& w) {
  x.assign(q, 0.0);
  w.assign(q, 0.0);
  for (int i = 0; i < (q + 1) / 2; ++i) {
    double z = cos(M_PI * (i + 0.75) / (q + 0.5)), p0 = 1.0, p1 = 0.0;
    for (int it = 0; it < 100; ++it) {
      p0 = 1.0;
      p1 = 0.0;
      for (int j = 1; j <= q; ++j) {
        const double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p2) / j;
      }
      const double dz = p0 / (q * (z * p0 - p1) / (z * z - 1.0));
      z -= dz;
      if (fabs(dz) < 1e-15) break;
    }
    p0 = 1.0;
    p1 = 0.0;
    for (int j = 1; j <= q; ++j) {
      const double p2 = p1;
      p1 = p0;
      p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p2) / j;
    }
    const double dp = q * (z * p0 - p1) / (z * z - 1.0);
    x[i] = -z;
    x[q - 1 - i] = z;
    w[i] = w[q - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Window constants of every dimension.  ES: support alpha = m + 1/2 (every grid
// point closer than alpha to the node is one of the 2m+2 taps of the window-start
// rule), beta_t = 0.97 pi (2 alpha)(1 - 1/(2 sigma_t)) (Barnett, Magland and
// af Klinteberg, SIAM J. Sci. Comput. 41 (2019)); the scaling sits in the roll-off
// factors, so norm = 1.
static void window_constants(Geom& g, int window) {
  g.window = window;
  const double alpha = g.m + 0.5;
  g.es_ia2 = 1.0 / (alpha * alpha);
  g.es_ia2f = (float)g.es_ia2;
  g.norm = 1.0;
  for (int t = 0; t < kMaxDim; ++t) {
    g.es_beta[t] = 0.0;
    g.es_bl[t] = 0.f;
  }
  for (int t = 0; t < g.d; ++t) {
    const double sigma = (double)g.n[t] / (double)g.N[t];
    if (window == kWinES) {
      g.es_beta[t] = 0.97 * M_PI * (2.0 * alpha) * (1.0 - 1.0 / (2.0 * sigma));
      g.es_bl[t] = (float)(g.es_beta[t] * 1.4426950408889634);
    } else {
      g.norm *= sqrt((2.0 * sigma - 1.0) / (2.0 * sigma * (double)g.m));
    }
  }
}

// Per-dimension roll-off factors 1 / phi_hat_t(k / n_t) for k in I_N, the
// dimension's table at offset sum_{s<t} N_s.  Gaussian: exp(fac_t k^2), fac_t =
// pi^2 b_t / n_t^2 (src/cunfft.cu:87; the constant 1/sqrt(pi b) is the kernels'
// norm).  ES: phi_hat(xi) = 2 int_0^alpha phi(y) cos(2 pi xi y) dy by 64-point
// Gauss-Legendre quadrature.
static std::vector<double> roc_factors(const Geom& g) {
  std::vector<double> tab;
  std::vector<double> gx, gw;
  if (g.window == kWinES) gauss_legendre(64, gx, gw);
  const double alpha = g.m + 0.5;
  for (int t = 0; t < g.d; ++t) {
    if (g.window == kWinES) {
      std::vector<double> yq(gx.size()), wq(gx.size());
      for (size_t i = 0; i < gx.size(); ++i) {
        yq[i] = 0.5 * alpha * (gx[i] + 1.0);
        const double z = 1.0 - yq[i] * yq[i] * g.es_ia2;
        wq[i] = alpha * gw[i] * exp(g.es_beta[t] * (sqrt(z > 0.0 ? z : 0.0) - 1.0));  // 2 x (alpha / 2) x w_i x phi
      }
      for (int64_t c = 0; c < g.N[t]; ++c) {
        const double xi = (double)(c - g.N[t] / 2) / (double)g.n[t];
        double ph = 0.0;
        for (size_t i = 0; i < yq.size(); ++i) ph += wq[i] * cos(2.0 * M_PI * xi * yq[i]);
        tab.push_back(1.0 / ph);
      }
    } else {
      const double fac = (M_PI * M_PI * g.b[t]) / (double)(g.n[t] * g.n[t]);
      for (int64_t c = 0; c < g.N[t]; ++c) {
        const double k = (double)(c - g.N[t] / 2);
        tab.push_back(exp(fac * k * k));
      }
    }
  }
  return tab;
}

// Geometry of a plan (parameters, window constants, device attributes); no
// device or host allocation.
int geom_init(Plan* p, int d, const int64_t* N, const int64_t* n, int m, int prec, int batch) {
  if (d < 1 || d > kMaxDim) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "d = %d not in 1..3", d);
  if (m < 1 || 2 * m + 2 > kMaxTaps) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "m = %d not in 1..15", m);
  if (prec != kF64 && prec != kF32) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "unknown precision %d", prec);
  if (batch < 1) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "batch = %d < 1", batch);
  Geom& g = p->geo;
  g.d = d;
  g.m = m;
  g.W = 2 * m + 2;
  g.batch = batch;
  g.Ntot = 1;
  g.ntot = 1;
  g.norm = 1.0;
  for (int t = 0; t < kMaxDim; ++t) {
    g.N[t] = 1;
    g.n[t] = 1;
    g.b[t] = 1.0;
  }
  for (int t = 0; t < d; ++t) {
    if (N[t] < 1) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "N[%d] = %lld < 1", t, (long long)N[t]);
    int64_t nt = n ? n[t] : 0;
    if (nt <= 0) {
      nt = 1;
      while (nt < N[t]) nt <<= 1;
      nt *= 2;
    }
    if (nt < N[t]) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "n[%d] < N[%d]", t, t);
    g.N[t] = N[t];
    g.n[t] = nt;
    const double sigma = (double)nt / (double)N[t];
    g.b[t] = (2.0 * sigma) / (2.0 * sigma - 1.0) * ((double)m / M_PI);
    g.cbf[t] = (float)(1.4426950408889634 / g.b[t]);
    g.Ntot *= N[t];
    g.ntot *= nt;
  }
  if (g.ntot * batch >= ((int64_t)1 << 40)) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "grid too large");
  window_constants(g, kWinGauss);
  p->prec = prec;
  CG_TRY(check_cuda(p, cudaGetDevice(&p->device), "cudaGetDevice"));
  CG_TRY(check_cuda(p, cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device),
                    "cudaDeviceGetAttribute"));
  return CUNFFT_X_SUCCESS;
}

int plan_window(const Plan* p) { return p->geo.window; }

// Switch the window: new tap constants and roll-off factors (same table size);
// captured graphs hold the old constants by value and are re-captured.
int plan_set_window(Plan* p, int window) {
  if (window != kWinGauss && window != kWinES)
    return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "unknown window %d", window);
  if (window != p->geo.window) {
    CG_TRY(check_cuda(p, cudaStreamSynchronize(p->stream), "cudaStreamSynchronize"));  // the old table may be in use
    window_constants(p->geo, window);
    const std::vector<double> tab = roc_factors(p->geo);
    CG_TRY(check_cuda(p, cudaMemcpy(p->roc_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice),
                      "upload roll-off table"));
    ++p->node_gen;
  }
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_init(Plan* p, int d, const int64_t* N, const int64_t* n, int m, int prec, int batch, cudaStream_t stream,
              void* lend_grid) {
  CG_TRY(geom_init(p, d, N, n, m, prec, batch));
  const Geom& g = p->geo;
  if (stream) {
    p->stream = stream;
    p->own_stream = false;
  } else {
    CG_TRY(check_cuda(p, cudaStreamCreate(&p->stream), "cudaStreamCreate"));
    p->own_stream = true;
  }
  for (int i = 0; i < 8; ++i) CG_TRY(check_cuda(p, cudaEventCreate(&p->ev[i]), "cudaEventCreate"));
  p->timing = true;
  // roll-off factor tables, per dimension
  {
    const std::vector<double> tab = roc_factors(g);
    CG_TRY(check_cuda(p, plan_malloc(&p->roc_tab, sizeof(double) * tab.size()), "cudaMalloc roll-off table"));
    CG_TRY(check_cuda(p, cudaMemcpy(p->roc_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice),
                      "upload roll-off table"));
  }
  if (lend_grid) {
    p->g = lend_grid;
    p->own_g = false;
  } else {
    CG_TRY(check_cuda(p, plan_malloc(&p->g, elem_bytes(p) * g.ntot * batch), "cudaMalloc grid"));
    p->own_g = true;
  }
  // batched in-place FFT over the instances' grids
  {
    int nn[kMaxDim];
    for (int t = 0; t < d; ++t) {
      if (g.n[t] > 0x7fffffff) return set_status(p, CUNFFT_X_UNSUPPORTED, "FFT length too large");
      nn[t] = (int)g.n[t];
    }
    cufftHandle h;
    CG_TRY(check_cufft(p, cufftCreate(&h), "cufftCreate"));
    size_t ws = 0;
    long long nll[kMaxDim];
    for (int t = 0; t < d; ++t) nll[t] = nn[t];
    cufftResult r = plan_fft_fault() ? CUFFT_INTERNAL_ERROR
                                     : cufftMakePlanMany64(h, d, nll, nullptr, 1, g.ntot, nullptr, 1, g.ntot,
                                                           prec == kF64 ? CUFFT_Z2Z : CUFFT_C2C, batch, &ws);
    if (r != CUFFT_SUCCESS) {
      cufftDestroy(h);
      return check_cufft(p, r, "cufftMakePlanMany64");
    }
    p->fft = h;
    p->own_fft = true;
  }
  // per-instance node offsets, status flag, work counters
  CG_TRY(check_cuda(p, plan_malloc(&p->bins.inst_off, sizeof(int32_t) * (batch + 1)), "cudaMalloc"));
  CG_TRY(check_cuda(p, plan_malloc(&p->bins.work, sizeof(int32_t) * 2), "cudaMalloc"));
  CG_TRY(check_cuda(p, plan_malloc(&p->bins.num_items, sizeof(int32_t)), "cudaMalloc"));
  CG_TRY(check_cuda(p, plan_malloc(&p->bins.num_iitems, sizeof(int32_t)), "cudaMalloc"));
  CG_TRY(check_cuda(p, plan_malloc(&p->bins.status, sizeof(int32_t)), "cudaMalloc"));
  CG_TRY(check_cuda(p, plan_malloc(&p->bins.fmax, sizeof(uint32_t)), "cudaMalloc"));
  CG_TRY(check_cuda(p, cudaMemset(p->bins.status, 0, sizeof(int32_t)), "cudaMemset"));
  p->M_inst = (int64_t*)calloc((size_t)batch, sizeof(int64_t));
  CG_TRY(plan_choose_tiling(p, nullptr, 0));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

void plan_release(Plan* p) {
  if (!p) return;
  if (p->stream) cudaStreamSynchronize(p->stream);
  plan_host_path_release(p);
  for (int i = 0; i < 2; ++i)
    if (p->gexec[i]) {
      cudaGraphExecDestroy(p->gexec[i]);
      p->gexec[i] = nullptr;
    }
  free_bins(p);
  interp_tc_release(*p);
  cudaFree(p->bins.inst_off);
  cudaFree(p->bins.work);
  cudaFree(p->bins.num_items);
  cudaFree(p->bins.num_iitems);
  cudaFree(p->bins.status);
  cudaFree(p->bins.fmax);
  p->bins.fmax = nullptr;
  p->bins.inst_off = nullptr;
  p->bins.work = nullptr;
  p->bins.num_items = nullptr;
  p->bins.num_iitems = nullptr;
  p->bins.status = nullptr;
  if (p->own_g) cudaFree(p->g);
  p->g = nullptr;
  cudaFree(p->roc_tab);
  p->roc_tab = nullptr;
  if (p->own_fft && p->fft) cufftDestroy(p->fft);
  p->fft = 0;
  for (int i = 0; i < 8; ++i)
    if (p->ev[i]) cudaEventDestroy(p->ev[i]);
  if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
  p->stream = nullptr;
  free(p->M_inst);
  p->M_inst = nullptr;
}

static int ensure_bins(Plan* p, int64_t M) {
  Bins& B = p->bins;
  const int64_t tiles = p->tl.tiles_total;
  const int64_t max_items = tiles + M / std::max(1, p->tl.chunk) + 1;
  // sub-bin keys and their interpolation items (each sub-bin: at most count / kSubItem + 1)
  const int64_t keys = p->tl.sub_on ? tiles * p->tl.ns : 0;
  const int64_t max_iitems = keys > 0 && p->tl.sub_items ? keys + M / kSubItem + 1 : 0;
  const size_t real = elem_bytes(p) / 2;
  if (M > p->bins_capacity_M || tiles > p->bins_capacity_tiles || max_items > B.max_items ||
      keys > p->bins_capacity_keys || max_iitems > B.max_iitems || p->bins_capacity_M < 0) {
    const int64_t capM = std::max<int64_t>(M, 1), capT = tiles;
    free_bins(p);
    CG_TRY(check_cuda(p, plan_malloc(&B.sidx, sizeof(int32_t) * capM), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.soff, sizeof(int32_t) * capM), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.sfrac, real * p->geo.d * capM), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.tile_rank, sizeof(int2) * capM), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.fperm, elem_bytes(p) * capM), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.count, sizeof(int32_t) * (capT + 1)), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.tile_off, sizeof(int32_t) * (capT + 1)), "cudaMalloc bins"));
    CG_TRY(check_cuda(p, plan_malloc(&B.item_off, sizeof(int32_t) * (capT + 1)), "cudaMalloc bins"));
    const int64_t cap_items = capT + capM / std::max(1, p->tl.chunk) + 1;
    CG_TRY(check_cuda(p, plan_malloc(&B.items, sizeof(int4) * cap_items), "cudaMalloc bins"));
    B.max_items = cap_items;
    if (keys > 0) {
      CG_TRY(check_cuda(p, plan_malloc(&B.scount, sizeof(int32_t) * (keys + 1)), "cudaMalloc bins"));
      CG_TRY(check_cuda(p, plan_malloc(&B.sub_pre, sizeof(int32_t) * keys), "cudaMalloc bins"));
    }
    if (max_iitems > 0) {
      const int64_t cap_ii = keys + capM / kSubItem + 1;
      CG_TRY(check_cuda(p, plan_malloc(&B.icount, sizeof(int32_t) * (capT + 1)), "cudaMalloc bins"));
      CG_TRY(check_cuda(p, plan_malloc(&B.iitem_off, sizeof(int32_t) * (capT + 1)), "cudaMalloc bins"));
      CG_TRY(check_cuda(p, plan_malloc(&B.iscratch, sizeof(int32_t) * (capT + 1)), "cudaMalloc bins"));
      CG_TRY(check_cuda(p, plan_malloc(&B.iitems, sizeof(int4) * cap_ii), "cudaMalloc bins"));
      B.max_iitems = cap_ii;
    }
    p->bins_capacity_M = capM;
    p->bins_capacity_tiles = capT;
    p->bins_capacity_keys = keys;
  }
  return CUNFFT_X_SUCCESS;
}

static int rebin(Plan* p) {
  CG_TRY(ensure_bins(p, p->M));
  p->bins.M = p->M;
  if (p->timing) cudaEventRecord(p->ev[6], p->stream);
  CG_TRY(check_cuda(p, launch_binning(*p, p->x, p->stream), "binning kernels"));
  if (p->timing) cudaEventRecord(p->ev[7], p->stream);
  p->bins.valid = 1;
  ++p->node_gen;  // captured graphs hold the old binning by value
  return CUNFFT_X_SUCCESS;
}

int plan_set_nodes(Plan* p, const double* x, const int64_t* M_inst) {
  int64_t M = 0;
  std::vector<int32_t> off((size_t)p->geo.batch + 1, 0);
  bool same = p->inst_off_current;
  for (int i = 0; i < p->geo.batch; ++i) {
    if (M_inst[i] < 0) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "M[%d] < 0", i);
    M += M_inst[i];
    if (M >= ((int64_t)1 << 31) - 1) return set_status(p, CUNFFT_X_UNSUPPORTED, "more than 2^31-2 nodes");
    off[i + 1] = (int32_t)M;
    same = same && p->M_inst[i] == M_inst[i];
  }
  if (M > 0 && !x) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "x is NULL");
  // New per-instance counts: upload the offsets (the host vector must outlive the
  // copy, hence the wait).  Unchanged counts, the usual case of a moving node set,
  // need neither the copy nor the wait, so the stream keeps running.
  if (!same) {
    p->inst_off_current = false;
    CG_TRY(check_cuda(p, cudaMemcpyAsync(p->bins.inst_off, off.data(), sizeof(int32_t) * off.size(),
                                         cudaMemcpyHostToDevice, p->stream), "upload node offsets"));
    CG_TRY(check_cuda(p, cudaStreamSynchronize(p->stream), "cudaStreamSynchronize"));
    for (int i = 0; i < p->geo.batch; ++i) p->M_inst[i] = M_inst[i];
    p->inst_off_current = true;
  }
  p->x = x;
  p->M = M;
  CG_TRY(rebin(p));
  p->nodes_set = true;
  p->t_bin = 0;
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

static cufftResult exec_fft(const Plan* p, cufftHandle h, void* data, int dir) {
  cufftResult r = cufftSetStream(h, p->stream);
  if (r != CUFFT_SUCCESS) return r;
  if (p->prec == kF64) return cufftExecZ2Z(h, (cufftDoubleComplex*)data, (cufftDoubleComplex*)data, dir);
  return cufftExecC2C(h, (cufftComplex*)data, (cufftComplex*)data, dir);
}

static void rec(Plan* p, int i) {
  if (p->timing) cudaEventRecord(p->ev[i], p->stream);
}

// Buffers of the tensor-core interpolation (the grid's split planes and their TMA
// map), created before its first launch.  When they cannot be created and the kernel
// was chosen automatically, the shared-tile interpolation runs instead.
static int prepare_interp(Plan* p) {
  if (p->tl.interp_kernel != CUNFFT_X_INTERP_TENSOR || p->it_ready) return CUNFFT_X_SUCCESS;
  const cudaError_t e = interp_tc_prepare(*p);
  if (e == cudaSuccess) return CUNFFT_X_SUCCESS;
  cudaGetLastError();  // a failed allocation leaves no sticky error
  if (p->interp_mode == CUNFFT_X_INTERP_AUTO) {
    p->tl.interp_kernel = CUNFFT_X_INTERP_SHARED;
    ++p->node_gen;
    return CUNFFT_X_SUCCESS;
  }
  return check_cuda(p, e, "tensor-core interpolation buffers");
}

int plan_forward(Plan* p, const void* fhat, void* f) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "forward: nodes not set");
  if (!p->bins.valid) CG_TRY(rebin(p));
  CG_TRY(prepare_interp(p));
  if (p->timing) p->last_dir = 0;
  rec(p, 0);
  CG_TRY(check_cuda(p, launch_roc_forward(*p, fhat, p->g, p->stream), "roll-off kernel"));
  rec(p, 1);
  CG_TRY(check_cufft(p, exec_fft(p, p->fft_fwd_ext ? p->fft_fwd_ext : p->fft, p->g, CUFFT_FORWARD), "forward FFT"));
  rec(p, 2);
  CG_TRY(check_cuda(p, launch_interp(*p, p->g, f, p->stream), "interpolation kernel"));
  rec(p, 3);
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_adjoint(Plan* p, const void* f, void* fhat) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "adjoint: nodes not set");
  if (!p->bins.valid) CG_TRY(rebin(p));
  if (p->timing) p->last_dir = 1;
  rec(p, 0);
  CG_TRY(check_cuda(p, cudaMemsetAsync(p->g, 0, elem_bytes(p) * p->geo.ntot * p->geo.batch, p->stream),
                    "clear grid"));
  CG_TRY(check_cuda(p, launch_spread(*p, f, p->g, p->stream), "spreading kernel"));
  rec(p, 1);
  CG_TRY(check_cufft(p, exec_fft(p, p->fft_bwd_ext ? p->fft_bwd_ext : p->fft, p->g, CUFFT_INVERSE), "adjoint FFT"));
  rec(p, 2);
  CG_TRY(check_cuda(p, launch_roc_adjoint(*p, p->g, fhat, p->stream), "roll-off kernel"));
  rec(p, 3);
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

// Forward (adjoint = 0) or adjoint (1) through a CUDA graph.  The stage
// sequence (roll-off, FFT, gridding and the small memsets) is captured from the
// plan's stream once per (input, output, node binding) and then replayed with one
// cudaGraphLaunch; the node binning itself stays outside the graph.
int plan_run_graph(Plan* p, int adjoint, const void* in, void* out) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "graph: nodes not set");
  if (!p->bins.valid) CG_TRY(rebin(p));
  const int k = adjoint ? 1 : 0;
  if (!p->gexec[k] || p->g_in[k] != in || p->g_out[k] != out || p->g_gen[k] != p->node_gen) {
    if (p->gexec[k]) {
      cudaGraphExecDestroy(p->gexec[k]);
      p->gexec[k] = nullptr;
    }
    // run once uncaptured so that every kernel attribute and cuFFT resource is set up
    CG_TRY(adjoint ? plan_adjoint(p, in, out) : plan_forward(p, in, out));
    const bool timing = p->timing;
    p->timing = false;
    cudaGraph_t graph = nullptr;
    CG_TRY(check_cuda(p, cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal), "begin capture"));
    const int s = adjoint ? plan_adjoint(p, in, out) : plan_forward(p, in, out);
    const cudaError_t ec = cudaStreamEndCapture(p->stream, &graph);
    p->timing = timing;
    if (s != CUNFFT_X_SUCCESS) {
      if (graph) cudaGraphDestroy(graph);
      return s;
    }
    CG_TRY(check_cuda(p, ec, "end capture"));
    const cudaError_t ei = cudaGraphInstantiate(&p->gexec[k], graph, 0);
    cudaGraphDestroy(graph);
    CG_TRY(check_cuda(p, ei, "instantiate graph"));
    p->g_in[k] = in;
    p->g_out[k] = out;
    p->g_gen[k] = p->node_gen;
    return set_status(p, CUNFFT_X_SUCCESS, nullptr);  // this call's result came from the uncaptured run
  }
  CG_TRY(check_cuda(p, cudaGraphLaunch(p->gexec[k], p->stream), "graph launch"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_interp_only(Plan* p, const void* g, void* f) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "interp: nodes not set");
  if (!p->bins.valid) CG_TRY(rebin(p));
  CG_TRY(prepare_interp(p));
  CG_TRY(check_cuda(p, launch_interp(*p, g, f, p->stream), "interpolation kernel"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_spread_only(Plan* p, const void* f, void* g) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "spread: nodes not set");
  if (!p->bins.valid) CG_TRY(rebin(p));
  CG_TRY(check_cuda(p, launch_spread(*p, f, g, p->stream), "spreading kernel"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_ndft_forward(Plan* p, const void* fhat, void* f) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "ndft: nodes not set");
  CG_TRY(check_cuda(p, launch_ndft_forward(*p, p->x, fhat, f, p->stream), "NDFT kernel"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_ndft_adjoint(Plan* p, const void* f, void* fhat, const int64_t* kidx, int64_t nsel) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "ndft: nodes not set");
  if (kidx && nsel < 0) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "nsel < 0");
  CG_TRY(check_cuda(p, launch_ndft_adjoint(*p, p->x, f, fhat, p->stream, kidx, nsel), "adjoint NDFT kernel"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_node_gradient(Plan* p, const void* fhat, const void* grad_f, double* grad_x) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "gradient: nodes not set");
  CG_TRY(check_cuda(p, launch_roc_forward(*p, fhat, p->g, p->stream), "roll-off kernel"));
  CG_TRY(check_cufft(p, exec_fft(p, p->fft, p->g, CUFFT_FORWARD), "forward FFT"));
  CG_TRY(check_cuda(p, launch_interp_grad(*p, p->g, grad_f, grad_x, p->stream), "gradient kernel"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

// Autotuner: time interpolation and spreading for a few tilings on the bound node
// set, each with every kernel that covers the tiling where no kernel was requested;
// keep the tiling with the fastest sum of the fastest kernels.  Restores the
// previous tiling when no candidate runs.
int plan_autotune(Plan* p, int reps) {
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "autotune: nodes not set");
  if (reps < 1) reps = 1;
  const int d = p->geo.d;
  std::vector<std::vector<int>> cands;
  if (d == 1) {
    for (int t : {512, 1024, 2048, 4096, 8192}) cands.push_back({t, 0, 0});
  } else if (d == 2) {
    for (int a : {8, 16, 32, 64, 128}) cands.push_back({a, 0, 0});
  } else {
    for (int a : {2, 4, 8, 16}) cands.push_back({a, 0, 0});
  }
  const Tiling best0 = p->tl;
  float best = 3.0e38f;
  std::vector<int> best_T(3, 0);
  int best_sk = 0, best_ik = 0;
  const size_t bytes = elem_bytes(p);
  void* scratch_f = nullptr;
  if (check_cuda(p, plan_malloc(&scratch_f, bytes * std::max<int64_t>(p->M, 1)), "autotune scratch")) return p->last_status;
  // non-zero data so that the spreading flush does real work while timed
  cudaMemsetAsync(scratch_f, 0x3c, bytes * std::max<int64_t>(p->M, 1), p->stream);
  cudaMemsetAsync(p->g, 0x3c, bytes * p->geo.ntot * p->geo.batch, p->stream);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const bool timing = p->timing;
  p->timing = false;
  bool failed = false;
  // device time of reps launches of one gridding kernel (after one warm-up); < 0 on failure
  auto time_kernel = [&](bool spread) -> float {
    if (!spread && p->tl.interp_kernel == CUNFFT_X_INTERP_TENSOR && interp_tc_prepare(*p) != cudaSuccess) {
      cudaGetLastError();
      return -1.f;
    }
    auto run = [&]() {
      return spread ? launch_spread(*p, scratch_f, p->g, p->stream) : launch_interp(*p, p->g, scratch_f, p->stream);
    };
    if (run() != cudaSuccess) return -1.f;
    cudaEventRecord(a, p->stream);
    for (int r = 0; r < reps; ++r) run();
    cudaEventRecord(b, p->stream);
    if (cudaEventSynchronize(b) != cudaSuccess) {
      failed = true;
      return -1.f;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  };
  for (auto& c : cands) {
    int T[3] = {c[0], c[1], c[2]};
    bool fits = true;
    for (int t = 0; t < d; ++t) fits = fits && T[t] <= p->geo.n[t];
    if (!fits) continue;
    if (plan_choose_tiling(p, T, p->chunk_override) != CUNFFT_X_SUCCESS) continue;
    if (rebin(p) != CUNFFT_X_SUCCESS) break;
    // every kernel that covers the tiling, where the choice is open; interpolation
    // and spreading are timed separately and the fastest of each kept
    std::vector<int> skinds{p->tl.spread_kernel}, ikinds{p->tl.interp_kernel};
    if (p->spread_mode == CUNFFT_X_SPREAD_AUTO) {
      if (p->tl.spread_kernel != CUNFFT_X_SPREAD_REGISTER && spread_reg_supported(*p))
        skinds.push_back(CUNFFT_X_SPREAD_REGISTER);
      if (p->tl.spread_kernel != CUNFFT_X_SPREAD_GLOBAL && p->tl.spread_kernel != CUNFFT_X_SPREAD_SHARED)
        skinds.push_back(CUNFFT_X_SPREAD_SHARED);
    }
    if (p->interp_mode == CUNFFT_X_INTERP_AUTO && p->tl.interp_kernel == CUNFFT_X_INTERP_TENSOR)
      ikinds.push_back(CUNFFT_X_INTERP_SHARED);
    float bs = 3.0e38f, bi = 3.0e38f;
    int sk = skinds[0], ik = ikinds[0];
    for (int kind : skinds) {
      p->tl.spread_kernel = kind;
      const float ms = time_kernel(true);
      if (failed) break;
      if (ms >= 0.f && ms < bs) {
        bs = ms;
        sk = kind;
      }
    }
    for (int kind : ikinds) {
      if (failed) break;
      p->tl.interp_kernel = kind;
      const float ms = time_kernel(false);
      if (ms >= 0.f && ms < bi) {
        bi = ms;
        ik = kind;
      }
    }
    if (failed) break;
    if (bs < 3.0e38f && bi < 3.0e38f && bs + bi < best) {
      best = bs + bi;
      best_T = {T[0], T[1], T[2]};
      best_sk = sk;
      best_ik = ik;
    }
  }
  p->timing = timing;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(scratch_f);
  cudaGetLastError();
  if (best_T[0] == 0) {
    p->tl = best0;
    p->it_ready = false;
    p->bins.valid = 0;
    return set_status(p, CUNFFT_X_CUDA_ERROR, "autotune: no candidate ran");
  }
  int T[3] = {best_T[0], best_T[1], best_T[2]};
  CG_TRY(plan_choose_tiling(p, T, p->chunk_override));
  p->tl.spread_kernel = best_sk;
  p->tl.interp_kernel = best_ik;
  CG_TRY(rebin(p));
  // the grid holds garbage from the timing runs; transforms rewrite it fully
  p->autotuned = true;
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

}  // namespace cg
