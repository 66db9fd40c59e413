/*
 * cunfft_oracle.c -- CPU restatement of the CUNFFT method (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * the parity tests, the smoke check and the benchmark's CPU-baseline leg call
 * it; the product (libcunfft.so) never links, loads or falls back to it.
 *
 * It restates, from the mathematics and in code of its own, the algorithm of
 * sukunis/CUNFFT 1.0 (Gaussian window, fast Gaussian gridding, FP64):
 *   - plan parameters       src/cunfft.cu:282-378 (n = 2*next_pow2(N),
 *                           sigma = n/N, b = 2 sigma/(2 sigma-1) * m/pi),
 *                           src/cunfft.cu:60-90 (fg_exp_l table, fac = pi^2 b/n^2)
 *   - window start index    src/cunfft_kernel.cu:175-182
 *                           (u = llrint(n x) - signbit(x) - m)
 *   - tap weights (FGG)     src/cunfft_kernel.cu:162-166, 491-505
 *   - roll-off correction   src/cunfft_kernel.cu:240-467 (k at grid index k mod n,
 *                           factor exp(sum_t fac_t k_t^2), no 1/n^d scaling)
 *   - interpolation         src/cunfft_kernel.cu:514-535, 667-712, 918-972
 *   - spreading             src/cunfft_kernel.cu:608-631, 842-878, 1098-1149
 *   - FFT sign convention   src/cunfft_wrapper.cu:288-329 (forward e^-, adjoint e^+,
 *                           both unnormalised)
 *   - direct NDFT / adjoint src/cunfft_kernel.cu:1207-1345
 *   - example data          src/cuda_util.cpp:151-171, 204-212 (drand48 order)
 *   - error norm            src/cuda_util.cpp:237-258
 *
 * A second window, not in the reference, checks the extension API's ES option:
 * exponential of semicircle phi(y) = exp(beta (sqrt(1 - y^2/alpha^2) - 1)) on
 * |y| < alpha = m + 1/2, beta = 0.97 pi (2m+1)(1 - 1/(2 sigma)) (Barnett, Magland,
 * af Klinteberg, SIAM J. Sci. Comput. 41 (2019)), roll-off 1/phi_hat(k/n) with
 * phi_hat by composite Simpson quadrature (orc_set_window(1)).  Its accuracy is
 * pinned against the direct NDFT, not against the reference.
 *
 * Parity is pinned against the E_inf known answers of the reference's own
 * result logs (Tests/Runtime/*.txt), which the reference produced from
 * drand48's default state; see tests/golden/.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (oracle/build.py).
 * -ffp-contract=off keeps x86 and Arm results identical.
 *
 * Layout conventions (match the reference's plan arrays):
 *   x     [M][d] row-major doubles
 *   fhat  row-major over I_N, dim 0 slowest, index sum_t (k_t + N_t/2) * prod_{s>t} N_s
 *   g     row-major n0 x n1 x n2, frequency k stored at grid index k mod n
 *   complex arrays are interleaved (re, im) doubles.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORC_MAXD 3

/* ------------------------------------------------------------------------ */
/* drand48: the POSIX 48-bit linear congruential generator                  */
/* X_{k+1} = (a X_k + c) mod 2^48, a = 0x5DEECE66D, c = 0xB, value X/2^48.  */
/* glibc (the reference's platform) starts an unseeded stream at X_0 = 0,   */
/* so the first value is 11/2^48; the reference drivers never seed it.      */
/* ------------------------------------------------------------------------ */
uint64_t orc_drand48_default_state(void) { return 0ULL; }

void orc_drand48_fill(uint64_t *state, double *out, int64_t count)
{
    const uint64_t a = 0x5DEECE66DULL, c = 0xBULL, mask = (1ULL << 48) - 1ULL;
    uint64_t s = *state;
    for (int64_t i = 0; i < count; ++i) {
        s = (a * s + c) & mask;
        out[i] = (double)s * 0x1p-48;
    }
    *state = s;
}

/* Reference example data (src/cuda_util.cpp:151-171): coef[k] = (drand48, drand48)
 * for k < ncoef, then x[i] = drand48() - 0.5 for i < M*d. */
void orc_example_data(uint64_t *state, int64_t ncoef, double *coef, int64_t nx, double *x)
{
    orc_drand48_fill(state, coef, 2 * ncoef);
    orc_drand48_fill(state, x, nx);
    for (int64_t i = 0; i < nx; ++i) x[i] = x[i] - 0.5;
}

/* ------------------------------------------------------------------------ */
/* Parameters                                                                */
/* ------------------------------------------------------------------------ */
int64_t orc_next_pow2(int64_t N)
{
    int64_t p = 1;
    while (p < N) p <<= 1;
    return p;
}

void orc_params(int d, const int64_t *N, const int64_t *n, int m,
                double *sigma, double *b, double *fac)
{
    for (int t = 0; t < d; ++t) {
        sigma[t] = (double)n[t] / (double)N[t];
        b[t] = (2.0 * sigma[t]) / (2.0 * sigma[t] - 1.0) * ((double)m / M_PI);
        fac[t] = (M_PI * M_PI * b[t]) / (double)(n[t] * n[t]);
    }
}

/* fg_exp_l[l] = exp(-l^2/b), l = 0..W-1, by the recurrence of src/cunfft.cu:60-76. */
void orc_fg_exp_l(double *out, double b, int W)
{
    double b0 = exp(-1.0 / b), b0sq = b0 * b0, b1 = 1.0, b2;
    out[0] = 1.0;
    for (int l = 1; l < W; ++l) {
        b2 = b1 * b0;
        b1 *= b0sq;
        out[l] = out[l - 1] * b2;
    }
}

/* u = llrint(n x) - signbit(x) - m (round to nearest even, signbit of -0.0 is 1). */
int64_t orc_window_start(double x, int64_t n, int m)
{
    return (int64_t)llrint(x * (double)n) - (signbit(x) ? 1 : 0) - (int64_t)m;
}

static inline int64_t wrap(int64_t i, int64_t n)
{
    int64_t r = i % n;
    return r < 0 ? r + n : r;
}

/* Tap weights of one node in one dimension, FGG form:
 * psi_0 = phi(c), psi_l = phi(c) * E^l * fg[l], E = exp(2c/b),
 * phi(c) = sqrt(b') exp(-pi b' c^2), b' = (2 sigma - 1)/(2 sigma m). */
static void node_weights(double c, double sigma, double b, int m, const double *fg, int W, double *w)
{
    double bp = (2.0 * sigma - 1.0) / (2.0 * sigma * (double)m);
    double phi = exp(-(c * c) * bp * M_PI) * sqrt(bp);
    double E = exp(2.0 * c / b);
    double e = 1.0;
    w[0] = phi;
    for (int l = 1; l < W; ++l) {
        e = e * E;
        w[l] = phi * e * fg[l];
    }
}

/* Window of the restated method: 0 the reference's Gaussian, 1 ES (see above). */
static int orc_win = 0;
void orc_set_window(int w) { orc_win = w; }
int orc_get_window(void) { return orc_win; }

typedef struct {
    int win;
    double es_beta[ORC_MAXD];
    int d, m, W;
    int64_t N[ORC_MAXD], n[ORC_MAXD];
    int64_t Ntot, ntot;
    double sigma[ORC_MAXD], b[ORC_MAXD], fac[ORC_MAXD];
    double fg[ORC_MAXD][64];
} oplan;

static int plan_setup(oplan *p, int d, const int64_t *N, const int64_t *n, int m)
{
    if (d < 1 || d > ORC_MAXD || m < 1 || 2 * m + 2 > 64) return -1;
    p->d = d; p->m = m; p->W = 2 * m + 2;
    p->Ntot = 1; p->ntot = 1;
    for (int t = 0; t < d; ++t) {
        p->N[t] = N[t]; p->n[t] = n[t];
        p->Ntot *= N[t]; p->ntot *= n[t];
    }
    orc_params(d, N, n, m, p->sigma, p->b, p->fac);
    for (int t = 0; t < d; ++t) orc_fg_exp_l(p->fg[t], p->b[t], p->W);
    p->win = orc_win;
    for (int t = 0; t < d; ++t)
        p->es_beta[t] = 0.97 * M_PI * (2.0 * m + 1.0) * (1.0 - 1.0 / (2.0 * p->sigma[t]));
    return 0;
}

static double es_phi(double y, double beta, double alpha)
{
    double z = 1.0 - (y / alpha) * (y / alpha);
    return z > 0.0 ? exp(beta * (sqrt(z) - 1.0)) : 0.0;
}

/* 1 / phi_hat_t(k / n_t) for k = c - N_t/2, c = 0..N_t-1: phi_hat(xi) =
 * 2 int_0^alpha phi(y) cos(2 pi xi y) dy, composite Simpson on 40000 intervals. */
static double *es_roc_table(const oplan *p, int t)
{
    const int K = 40000;
    const double alpha = p->m + 0.5, h = alpha / K;
    double *ph = (double *)malloc(sizeof(double) * (K + 1));
    double *tab = (double *)malloc(sizeof(double) * (size_t)p->N[t]);
    for (int i = 0; i <= K; ++i) {
        double sw = (i == 0 || i == K) ? 1.0 : ((i % 2) ? 4.0 : 2.0);
        ph[i] = sw * es_phi(i * h, p->es_beta[t], alpha);
    }
    for (int64_t c = 0; c < p->N[t]; ++c) {
        double xi = (double)(c - p->N[t] / 2) / (double)p->n[t], acc = 0.0;
        for (int i = 0; i <= K; ++i) acc += ph[i] * cos(2.0 * M_PI * xi * (i * h));
        tab[c] = 1.0 / (2.0 * acc * h / 3.0);
    }
    free(ph);
    return tab;
}

/* Node -> (u_t, weights) for all dims. */
static void node_setup(const oplan *p, const double *xj, int64_t *u, double w[][64])
{
    for (int t = 0; t < p->d; ++t) {
        u[t] = orc_window_start(xj[t], p->n[t], p->m);
        double c = (double)p->n[t] * xj[t] - (double)u[t];
        if (p->win == 1) {
            for (int l = 0; l < p->W; ++l) w[t][l] = es_phi(c - (double)l, p->es_beta[t], p->m + 0.5);
        } else {
            node_weights(c, p->sigma[t], p->b[t], p->m, p->fg[t], p->W, w[t]);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Roll-off correction                                                      */
/* ------------------------------------------------------------------------ */
static void coef_index_to_k(const oplan *p, int64_t idx, int64_t *k)
{
    for (int t = p->d - 1; t >= 0; --t) {
        k[t] = idx % p->N[t] - p->N[t] / 2;
        idx /= p->N[t];
    }
}

static int64_t grid_index_of_k(const oplan *p, const int64_t *k)
{
    int64_t gi = 0;
    for (int t = 0; t < p->d; ++t) gi = gi * p->n[t] + wrap(k[t], p->n[t]);
    return gi;
}

static double roc_factor(const oplan *p, const int64_t *k)
{
    double s = 0.0;
    for (int t = 0; t < p->d; ++t) s += p->fac[t] * (double)k[t] * (double)k[t];
    return exp(s);
}

static double es_roc_factor(const oplan *p, double *const *tab, const int64_t *k)
{
    double f = 1.0;
    for (int t = 0; t < p->d; ++t) f *= tab[t][k[t] + p->N[t] / 2];
    return f;
}

/* g = 0 outside I_N; g[k mod n] = fhat[k] * exp(sum fac k^2) (Gaussian), or
 * fhat[k] * prod_t 1/phi_hat_t(k_t/n_t) (ES). */
void orc_roc_forward(int d, const int64_t *N, const int64_t *n, int m,
                     const double *fhat, double *g)
{
    oplan p;
    if (plan_setup(&p, d, N, n, m)) return;
    double *es_tab[ORC_MAXD] = {NULL, NULL, NULL};
    if (p.win == 1)
        for (int t = 0; t < d; ++t) es_tab[t] = es_roc_table(&p, t);
    memset(g, 0, sizeof(double) * 2 * (size_t)p.ntot);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p.Ntot; ++i) {
        int64_t k[ORC_MAXD];
        coef_index_to_k(&p, i, k);
        int64_t gi = grid_index_of_k(&p, k);
        double f = p.win == 1 ? es_roc_factor(&p, es_tab, k) : roc_factor(&p, k);
        g[2 * gi] = fhat[2 * i] * f;
        g[2 * gi + 1] = fhat[2 * i + 1] * f;
    }
    for (int t = 0; t < d; ++t) free(es_tab[t]);
}

/* fhat[k] = g[k mod n] * exp(sum fac k^2). */
void orc_roc_adjoint(int d, const int64_t *N, const int64_t *n, int m,
                     const double *g, double *fhat)
{
    oplan p;
    if (plan_setup(&p, d, N, n, m)) return;
    double *es_tab[ORC_MAXD] = {NULL, NULL, NULL};
    if (p.win == 1)
        for (int t = 0; t < d; ++t) es_tab[t] = es_roc_table(&p, t);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p.Ntot; ++i) {
        int64_t k[ORC_MAXD];
        coef_index_to_k(&p, i, k);
        int64_t gi = grid_index_of_k(&p, k);
        double f = p.win == 1 ? es_roc_factor(&p, es_tab, k) : roc_factor(&p, k);
        fhat[2 * i] = g[2 * gi] * f;
        fhat[2 * i + 1] = g[2 * gi + 1] * f;
    }
    for (int t = 0; t < d; ++t) free(es_tab[t]);
}

/* ------------------------------------------------------------------------ */
/* FFT: unnormalised multi-dimensional complex FFT, X[l] = sum_k x[k] e^{sign 2 pi i kl/n}. */
/* Radix-2 iterative for power-of-two lengths, direct DFT otherwise.        */
/* ------------------------------------------------------------------------ */
static void fft1d_pow2(double *a, int64_t len, int64_t stride, const double *tw, int sign)
{
    /* bit reversal */
    for (int64_t i = 1, j = 0; i < len; ++i) {
        int64_t bit = len >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = a[2 * i * stride], ti = a[2 * i * stride + 1];
            a[2 * i * stride] = a[2 * j * stride];
            a[2 * i * stride + 1] = a[2 * j * stride + 1];
            a[2 * j * stride] = tr;
            a[2 * j * stride + 1] = ti;
        }
    }
    for (int64_t half = 1; half < len; half <<= 1) {
        int64_t step = len / (2 * half);
        for (int64_t s = 0; s < len; s += 2 * half) {
            for (int64_t k = 0; k < half; ++k) {
                double wr = tw[2 * (k * step)], wi = sign * tw[2 * (k * step) + 1];
                double *pa = a + 2 * (s + k) * stride, *pb = a + 2 * (s + k + half) * stride;
                double br = pb[0] * wr - pb[1] * wi, bi = pb[0] * wi + pb[1] * wr;
                pb[0] = pa[0] - br; pb[1] = pa[1] - bi;
                pa[0] = pa[0] + br; pa[1] = pa[1] + bi;
            }
        }
    }
}

static void dft1d(double *a, int64_t len, int64_t stride, int sign, double *tmp)
{
    for (int64_t l = 0; l < len; ++l) {
        double sr = 0.0, si = 0.0;
        for (int64_t k = 0; k < len; ++k) {
            double ang = sign * 2.0 * M_PI * (double)((k * l) % len) / (double)len;
            double c = cos(ang), s = sin(ang);
            double xr = a[2 * k * stride], xi = a[2 * k * stride + 1];
            sr += xr * c - xi * s;
            si += xr * s + xi * c;
        }
        tmp[2 * l] = sr; tmp[2 * l + 1] = si;
    }
    for (int64_t l = 0; l < len; ++l) {
        a[2 * l * stride] = tmp[2 * l];
        a[2 * l * stride + 1] = tmp[2 * l + 1];
    }
}

void orc_fft(int d, const int64_t *n, double *a, int sign)
{
    int64_t total = 1;
    for (int t = 0; t < d; ++t) total *= n[t];
    for (int t = 0; t < d; ++t) {
        int64_t len = n[t], stride = 1;
        for (int s = t + 1; s < d; ++s) stride *= n[s];
        int64_t outer = total / (len * stride);
        int pow2 = (len & (len - 1)) == 0;
        double *tw = NULL;
        if (pow2) {
            tw = (double *)malloc(sizeof(double) * 2 * (size_t)(len / 2 + 1));
            for (int64_t k = 0; k <= len / 2; ++k) {
                double ang = -2.0 * M_PI * (double)k / (double)len; /* sign applied in butterfly */
                tw[2 * k] = cos(ang);
                tw[2 * k + 1] = -sin(ang); /* +sin(2 pi k/len); butterfly multiplies by sign */
            }
        }
        int64_t lines = outer * stride;
#pragma omp parallel
        {
            double *tmp = pow2 ? NULL : (double *)malloc(sizeof(double) * 2 * (size_t)len);
#pragma omp for schedule(static)
            for (int64_t line = 0; line < lines; ++line) {
                int64_t o = line / stride, s = line % stride;
                double *base = a + 2 * (o * len * stride + s);
                if (pow2) fft1d_pow2(base, len, stride, tw, sign);
                else dft1d(base, len, stride, sign, tmp);
            }
            free(tmp);
        }
        free(tw);
    }
}

/* ------------------------------------------------------------------------ */
/* Gridding                                                                  */
/* ------------------------------------------------------------------------ */
/* f_j = sum_l g[(u+l) mod n] prod_t psi_t(l_t); nesting and multiplication order
 * as in the reference kernels (innermost dimension summed first). */
void orc_interp(int d, const int64_t *N, const int64_t *n, int m, int64_t M,
                const double *x, const double *g, double *f)
{
    oplan p;
    if (plan_setup(&p, d, N, n, m)) return;
    const int W = p.W;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t j = 0; j < M; ++j) {
        int64_t u[ORC_MAXD], ix[ORC_MAXD][64];
        double w[ORC_MAXD][64];
        node_setup(&p, x + j * d, u, w);
        for (int t = 0; t < d; ++t)
            for (int l = 0; l < W; ++l) ix[t][l] = wrap(u[t] + l, p.n[t]);
        double sr = 0.0, si = 0.0;
        if (d == 1) {
            for (int l0 = 0; l0 < W; ++l0) {
                const double *gp = g + 2 * ix[0][l0];
                sr += gp[0] * w[0][l0];
                si += gp[1] * w[0][l0];
            }
        } else if (d == 2) {
            for (int l0 = 0; l0 < W; ++l0) {
                const double *row = g + 2 * ix[0][l0] * p.n[1];
                double ar = 0.0, ai = 0.0;
                for (int l1 = 0; l1 < W; ++l1) {
                    const double *gp = row + 2 * ix[1][l1];
                    ar += gp[0] * w[1][l1];
                    ai += gp[1] * w[1][l1];
                }
                sr += ar * w[0][l0];
                si += ai * w[0][l0];
            }
        } else {
            for (int l0 = 0; l0 < W; ++l0) {
                double ar = 0.0, ai = 0.0;
                for (int l1 = 0; l1 < W; ++l1) {
                    const double *row = g + 2 * (ix[0][l0] * p.n[1] + ix[1][l1]) * p.n[2];
                    double br = 0.0, bi = 0.0;
                    for (int l2 = 0; l2 < W; ++l2) {
                        const double *gp = row + 2 * ix[2][l2];
                        br += gp[0] * w[2][l2];
                        bi += gp[1] * w[2][l2];
                    }
                    ar += br * w[1][l1];
                    ai += bi * w[1][l1];
                }
                sr += ar * w[0][l0];
                si += ai * w[0][l0];
            }
        }
        f[2 * j] = sr;
        f[2 * j + 1] = si;
    }
}

static void spread_node(const oplan *p, const double *xj, const double *fj, double *g)
{
    int64_t u[ORC_MAXD], ix[ORC_MAXD][64];
    double w[ORC_MAXD][64];
    const int W = p->W, d = p->d;
    node_setup(p, xj, u, w);
    for (int t = 0; t < d; ++t)
        for (int l = 0; l < W; ++l) ix[t][l] = wrap(u[t] + l, p->n[t]);
    if (d == 1) {
        for (int l0 = 0; l0 < W; ++l0) {
            double *gp = g + 2 * ix[0][l0];
            gp[0] += fj[0] * w[0][l0];
            gp[1] += fj[1] * w[0][l0];
        }
    } else if (d == 2) {
        for (int l0 = 0; l0 < W; ++l0) {
            double *row = g + 2 * ix[0][l0] * p->n[1];
            for (int l1 = 0; l1 < W; ++l1) {
                double *gp = row + 2 * ix[1][l1];
                gp[0] += fj[0] * w[1][l1] * w[0][l0];
                gp[1] += fj[1] * w[1][l1] * w[0][l0];
            }
        }
    } else {
        for (int l0 = 0; l0 < W; ++l0) {
            for (int l1 = 0; l1 < W; ++l1) {
                double *row = g + 2 * (ix[0][l0] * p->n[1] + ix[1][l1]) * p->n[2];
                const double a0 = fj[0] * w[0][l0] * w[1][l1], a1 = fj[1] * w[0][l0] * w[1][l1];
                for (int l2 = 0; l2 < W; ++l2) {
                    double *gp = row + 2 * ix[2][l2];
                    gp[0] += a0 * w[2][l2];
                    gp[1] += a1 * w[2][l2];
                }
            }
        }
    }
}

/* g += sum_j f_j prod_t psi_t (g is NOT cleared here).  Deterministic parallel
 * schedule: nodes are bucketed by slab of their dim-0 window start; slabs are at
 * least W planes wide, even slabs run in parallel, then odd slabs, each slab's
 * nodes in index order. */
void orc_spread(int d, const int64_t *N, const int64_t *n, int m, int64_t M,
                const double *x, const double *f, double *g)
{
    oplan p;
    if (plan_setup(&p, d, N, n, m)) return;
    int64_t nslab = p.n[0] / p.W;
    if (nslab % 2) nslab -= 1;
    if (nslab < 2 || M < 2) {
        for (int64_t j = 0; j < M; ++j) spread_node(&p, x + j * d, f + 2 * j, g);
        return;
    }
    int64_t *cnt = (int64_t *)calloc((size_t)nslab + 1, sizeof(int64_t));
    int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)M);
    int64_t *slab_of = (int64_t *)malloc(sizeof(int64_t) * (size_t)M);
    for (int64_t j = 0; j < M; ++j) {
        int64_t s0 = wrap(orc_window_start(x[j * d], p.n[0], p.m), p.n[0]);
        slab_of[j] = s0 * nslab / p.n[0];
        cnt[slab_of[j] + 1]++;
    }
    for (int64_t s = 0; s < nslab; ++s) cnt[s + 1] += cnt[s];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)nslab);
    memcpy(fill, cnt, sizeof(int64_t) * (size_t)nslab);
    for (int64_t j = 0; j < M; ++j) order[fill[slab_of[j]]++] = j;
    for (int color = 0; color < 2; ++color) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t s = color; s < nslab; s += 2) {
            for (int64_t q = cnt[s]; q < cnt[s + 1]; ++q) {
                int64_t j = order[q];
                spread_node(&p, x + j * d, f + 2 * j, g);
            }
        }
    }
    free(cnt); free(order); free(slab_of); free(fill);
}

/* ------------------------------------------------------------------------ */
/* NFFT forward / adjoint                                                    */
/* ------------------------------------------------------------------------ */
void orc_nfft_forward(int d, const int64_t *N, const int64_t *n, int m, int64_t M,
                      const double *x, const double *fhat, double *f)
{
    int64_t ntot = 1;
    for (int t = 0; t < d; ++t) ntot *= n[t];
    double *g = (double *)malloc(sizeof(double) * 2 * (size_t)ntot);
    orc_roc_forward(d, N, n, m, fhat, g);
    orc_fft(d, n, g, -1);
    orc_interp(d, N, n, m, M, x, g, f);
    free(g);
}

void orc_nfft_adjoint(int d, const int64_t *N, const int64_t *n, int m, int64_t M,
                      const double *x, const double *f, double *fhat)
{
    int64_t ntot = 1;
    for (int t = 0; t < d; ++t) ntot *= n[t];
    double *g = (double *)calloc(2 * (size_t)ntot, sizeof(double));
    orc_spread(d, N, n, m, M, x, f, g);
    orc_fft(d, n, g, +1);
    orc_roc_adjoint(d, N, n, m, g, fhat);
    free(g);
}

/* ------------------------------------------------------------------------ */
/* Direct NDFT (src/cunfft_kernel.cu:1207-1345)                             */
/* f_j = sum_k fhat_k e^{-2 pi i k.x_j},  fhat_k = sum_j f_j e^{+2 pi i k.x_j} */
/* phase omega = sum_t k_t (2 pi x_t), accumulated in dimension order.       */
/* ------------------------------------------------------------------------ */
void orc_ndft_forward(int d, const int64_t *N, int64_t M, const double *x,
                      const double *fhat, double *f)
{
    int64_t Ntot = 1;
    for (int t = 0; t < d; ++t) Ntot *= N[t];
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t j = 0; j < M; ++j) {
        double X[ORC_MAXD];
        int64_t k[ORC_MAXD];
        for (int t = 0; t < d; ++t) { X[t] = 2.0 * M_PI * x[j * d + t]; k[t] = -N[t] / 2; }
        double sr = 0.0, si = 0.0;
        for (int64_t kl = 0; kl < Ntot; ++kl) {
            double om = 0.0;
            for (int t = 0; t < d; ++t) om = (double)k[t] * X[t] + om;
            double c = cos(-om), s = sin(-om);
            double ar = fhat[2 * kl], ai = fhat[2 * kl + 1];
            sr += ar * c - ai * s;
            si += ar * s + ai * c;
            /* odometer, last dimension fastest */
            for (int t = d - 1; t >= 0; --t) {
                if (++k[t] < N[t] - N[t] / 2) break;
                k[t] = -N[t] / 2;
            }
        }
        f[2 * j] = sr;
        f[2 * j + 1] = si;
    }
}

void orc_ndft_adjoint(int d, const int64_t *N, int64_t M, const double *x,
                      const double *f, double *fhat)
{
    int64_t Ntot = 1;
    for (int t = 0; t < d; ++t) Ntot *= N[t];
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t kl = 0; kl < Ntot; ++kl) {
        int64_t k[ORC_MAXD], rem = kl;
        for (int t = d - 1; t >= 0; --t) { k[t] = rem % N[t] - N[t] / 2; rem /= N[t]; }
        double sr = 0.0, si = 0.0;
        for (int64_t j = 0; j < M; ++j) {
            double om = 0.0;
            for (int t = 0; t < d; ++t) om += (double)k[t] * (2.0 * M_PI) * x[j * d + t];
            double c = cos(om), s = sin(om);
            double ar = f[2 * j], ai = f[2 * j + 1];
            sr += ar * c - ai * s;
            si += ar * s + ai * c;
        }
        fhat[2 * kl] = sr;
        fhat[2 * kl + 1] = si;
    }
}

/* Forward NDFT restricted to a subset of nodes (idx[q], q < nsel): used for
 * error checks on subsamples of large node sets. */
void orc_ndft_forward_subset(int d, const int64_t *N, int64_t nsel, const int64_t *idx,
                             const double *x, const double *fhat, double *f)
{
    double *xs = (double *)malloc(sizeof(double) * (size_t)(nsel * d + 1));
    for (int64_t q = 0; q < nsel; ++q)
        for (int t = 0; t < d; ++t) xs[q * d + t] = x[idx[q] * d + t];
    orc_ndft_forward(d, N, nsel, xs, fhat, f);
    free(xs);
}

/* Adjoint NDFT evaluated only at the coefficient indices kidx[q], q < nsel. */
void orc_ndft_adjoint_subset(int d, const int64_t *N, int64_t M, const double *x,
                             const double *f, int64_t nsel, const int64_t *kidx, double *out)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t q = 0; q < nsel; ++q) {
        int64_t k[ORC_MAXD], rem = kidx[q];
        for (int t = d - 1; t >= 0; --t) { k[t] = rem % N[t] - N[t] / 2; rem /= N[t]; }
        double sr = 0.0, si = 0.0;
        for (int64_t j = 0; j < M; ++j) {
            double om = 0.0;
            for (int t = 0; t < d; ++t) om += (double)k[t] * (2.0 * M_PI) * x[j * d + t];
            double c = cos(om), s = sin(om);
            sr += f[2 * j] * c - f[2 * j + 1] * s;
            si += f[2 * j] * s + f[2 * j + 1] * c;
        }
        out[2 * q] = sr;
        out[2 * q + 1] = si;
    }
}

/* ------------------------------------------------------------------------ */
/* Error norm (src/cuda_util.cpp:237-258): ||x - y||_inf / ||x||_inf, |.| the complex modulus. */
/* ------------------------------------------------------------------------ */
double orc_error_l_infty(const double *x, const double *y, int64_t n)
{
    double num = 0.0, den = 0.0;
    for (int64_t k = 0; k < n; ++k) {
        double a = hypot(x[2 * k], x[2 * k + 1]);
        double e = hypot(x[2 * k] - y[2 * k], x[2 * k + 1] - y[2 * k + 1]);
        if (a > den) den = a;
        if (e > num) num = e;
    }
    return num / den;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
