// Host check of coord_pow2 (cunfft_gb300/csrc/bin_coord.h) against the reference's FP64
// rule u = llrint(n x) - signbit(x) - m, c = n x - u (src/cunfft_kernel.cu:175-182) on
// power-of-two n: window starts must agree exactly, FP32 fractions to one FP32 ulp plus
// 2^-49 (the FP64 rule rounds c to FP64 before its FP32 rounding, the integer form
// rounds the exact value once).  Prints a summary line; exit status 0
// when both hold.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bin_coord.h"

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static uint64_t next_u64() {  // splitmix64
  uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double uniform(double lo, double hi) { return lo + (hi - lo) * ((next_u64() >> 11) * 0x1.0p-53); }

static int32_t fbits(float f) {
  int32_t i;
  std::memcpy(&i, &f, 4);
  return i;
}

int main() {
  long long checked = 0, fallback = 0, u_bad = 0, f_exact = 0, f_bad = 0;
  for (int k = 1; k <= 24; ++k) {
    const double n = std::ldexp(1.0, k);
    std::vector<double> xs;
    for (int i = 0; i < 20000; ++i) xs.push_back(uniform(-0.5, 0.5));
    for (int i = 0; i < 2000; ++i) xs.push_back(uniform(-4.0, 4.0));
    for (int i = 0; i < 2000; ++i) {  // exact grid points, exact ties and their neighbours
      const double j = std::floor(uniform(-n / 2, n / 2));
      for (double t : {j / n, (j + 0.5) / n}) {
        xs.push_back(t);
        xs.push_back(std::nextafter(t, 1.0));
        xs.push_back(std::nextafter(t, -1.0));
      }
    }
    for (double t : {-0.5, 0.0, -0.0, std::nextafter(0.5, 0.0), 1e-300, -1e-300, 1e-3, -1e-3, 0.25, -0.25})
      xs.push_back(t);
    for (int m = 1; m <= 15; m += 7) {
      for (double x : xs) {
        const double nx = x * n;
        const int64_t u_ref = (int64_t)std::llrint(nx) - (std::signbit(x) ? 1 : 0) - m;
        const double c = nx - (double)u_ref;
        const float f_ref = (float)(c - (double)m);
        cg::CoordPow2 cp;
        if (!cg::coord_pow2(x, k, m, cp)) {
          ++fallback;
          continue;
        }
        ++checked;
        if (cp.u != u_ref) {
          if (u_bad < 5) std::printf("u mismatch: k %d m %d x %.17g: %lld vs %lld\n", k, m, x, (long long)cp.u, (long long)u_ref);
          ++u_bad;
        }
        // the FP64 rule rounds c = n x - u (|c| < 16) to 2^-49 or finer before its FP32
        // rounding; the integer form rounds the exact value once
        const float f = cg::coord_pow2_frac(cp);
        const double big = std::fmax(std::fabs((double)f), std::fabs((double)f_ref));
        const double tol = std::ldexp(1.0, std::ilogb(big > 0 ? big : 1.0) - 23) + std::ldexp(1.0, -49);
        if (fbits(f) == fbits(f_ref)) ++f_exact;
        else if (std::fabs((double)f - (double)f_ref) > tol) {
          if (f_bad < 5) std::printf("fraction mismatch: k %d m %d x %.17g: %.9g vs %.9g\n", k, m, x, f, f_ref);
          ++f_bad;
        }
      }
    }
  }
  std::printf("checked %lld fallback %lld u_mismatch %lld frac_exact %lld frac_beyond_tol %lld\n", checked, fallback,
              u_bad, f_exact, f_bad);
  return (u_bad == 0 && f_bad == 0 && checked > 0) ? 0 : 1;
}
