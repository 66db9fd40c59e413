// Host check of the tensor-core kernels' static resource rules for every supported
// (W, T0): shared memory within the 227 KB a CTA may use, 16-byte aligned regions,
// tensor-memory columns within 512, and the M-tile / row mappings covering the tile.
// Prints one line per failure; exit status 0 when none.
#include <cstdio>

#include "kernels_interp2_tc.cuh"
#include "kernels_interp_tc.cuh"
#include "kernels_spread2_tm.cuh"
#include "kernels_spread_tm.cuh"

using namespace cg;

static int fails = 0;
#define CHECK(c, ...)              \
  do {                             \
    if (!(c)) {                    \
      std::printf(__VA_ARGS__);    \
      std::printf("\n");           \
      ++fails;                     \
    }                              \
  } while (0)

int main() {
  const unsigned kMaxSmem = 227u * 1024u;
  for (int W = 4; W <= 16; W += 2) {
    for (int T0 = 1; T0 <= 16; T0 *= 2) {
      const int E0 = T0 + W - 1, E1 = tm_e1(W);
      if (spread_tc_ok(3, W, T0)) {
        const TcLayout L = tc_layout(W, E0);
        CHECK(L.total <= kMaxSmem, "tc W %d T0 %d: shared %u", W, T0, L.total);
        CHECK(L.mt * 128 >= E0 * E1, "tc W %d T0 %d: M-tiles", W, T0);
        CHECK(L.nacc * L.mt * kTcN <= 512 && L.tmem_cols <= 512, "tc W %d T0 %d: tmem", W, T0);
        CHECK(L.bar_off % 16 == 0 && L.wx_off % 16 == 0 && L.wb_off % 16 == 0, "tc W %d T0 %d: align", W, T0);
      }
      if (spread_tm_ok(3, W, T0, E0)) {
        const TmLayout L = tm_layout(W, E0);
        CHECK(L.total <= kMaxSmem, "tm W %d T0 %d: shared %u", W, T0, L.total);
        CHECK(L.mt <= kTmMaxMt && L.mt * tm_ap(W) >= E0 && tm_ap(W) * E1 <= 128, "tm W %d T0 %d: rows", W, T0);
        CHECK(kTmACol0 + kTmStages * kTmAStageCols <= 512 && (unsigned)(L.mt * kTcN) <= kTmACol0,
              "tm W %d T0 %d: tmem", W, T0);
        CHECK(L.rec_off % 16 == 0 && L.wx_off % 16 == 0 && L.wb_off % 16 == 0 && L.bar_off % 16 == 0 &&
                  L.stg_off % 16 == 0,
              "tm W %d T0 %d: align", W, T0);
        CHECK(2 * (fixed_t_last(3, W) + W - 1) <= kTcN, "tm W %d T0 %d: columns", W, T0);
      }
      if (interp_tc_ok(3, W, T0, 256)) {
        const ItLayout L = it_layout();
        CHECK(L.dyn <= kMaxSmem, "interp W %d T0 %d: shared %u", W, T0, L.dyn);
        CHECK(it_pairs(W) <= kItHalf && it_ch(W) >= 1, "interp W %d T0 %d: chunk", W, T0);
      }
    }
  }
  {
    const T2Layout L = t2_layout();
    CHECK(L.total <= kMaxSmem && L.total > 228u * 1024u / 2u, "spread2: shared %u (one CTA per SM)", L.total);
    CHECK(L.rec_off % 16 == 0 && L.bar_off % 16 == 0 && L.stg_off % 16 == 0 && (kT2StgStride * 4) % 16 == 0 &&
              kT2SlotBytes % 16 == 0 && kT2SlotVal % 8 == 0,
          "spread2: align");
    CHECK(kT2ACol0 + kT2Stages * 16u <= 512u, "spread2: tmem");
    CHECK(kT2Ahead < kT2Ring && kT2OpSet1 % 4 == 0 && kT2EpiWarp0 % 4 == 0 && kT2MmaWarp < kT2EpiWarp0,
          "spread2: roles");
    for (int W = 4; W <= 16; W += 2)
      CHECK(2 * (64 + W - 1) <= kT2N && kT2MaxT0 + W - 1 <= 128, "spread2 W %d: extents", W);
  }
  {
    const I2Layout L = i2_layout();
    CHECK(L.dyn <= kMaxSmem, "interp2: shared %u", L.dyn);
    CHECK(L.b_off % 1024 == 0 && kI2Part % 512 == 0 && kI2Stage % 1024 == 0 && L.a_off % 1024 == 0 &&
              kItAPart % 1024 == 0 && L.bar_off % 16 == 0,
          "interp2: align (64-byte swizzle atoms, core matrices)");
    CHECK(L.bar_off + 8u * (2 * kI2ABufs + 2 * kI2Stages + 2 * kI2Acc) + 8u <= L.total, "interp2: barriers");
    CHECK(kI2Acc * kI2N <= 512 && kI2N % 16 == 0 && kI2N <= 256, "interp2: tmem / MMA N");
    CHECK(kI2Threads == (kI2RWarp0 + 4 * kI2Sets) * 32 && kI2Threads <= 1024 && kI2RWarp0 % 4 == 2 &&
              kI2ABufs % kI2Sets == 0,
          "interp2: roles");
    for (int W = 4; W <= 16; W += 2)
      CHECK(kI2Sub + W - 1 <= kI2K && kI2Sub + W - 1 <= kI2Rows && interp2_tc_ok(2, W, 64, 512) &&
                !interp2_tc_ok(2, W, 8, 512) && !interp2_tc_ok(2, W, 64, 90),
            "interp2 W %d: extents", W);
  }
  std::printf("layout check: %d failures\n", fails);
  return fails == 0 ? 0 : 1;
}
