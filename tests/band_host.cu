// Host check of the band variants of the register row and column passes
// (dtmm_gb300/csrc/dtmm_regkern.cuh): for every side with a register
// transform and every band limit, the variant that row_band_pick selects
// loads every entry a lane may need -- an entry t + N1 m with |f| <= lim
// always has m < KB or m >= N2 - KB -- and the variants it may select exist
// (2 KB < N2).  Prints "checked <side> <limits>" lines and "OK" at the end.
#include <cstdio>

#include "dtmm_regkern.cuh"

using namespace dtmm;

template <int N>
static bool check_side() {
  constexpr int N1 = reg_lanes(N), N2 = N / N1;
  bool ok = true;
  int tested = 0;
  for (int lim = -1; lim <= N / 2; ++lim) {
    const int b = row_band_pick(N, lim);
    if (b == 0) continue;  // dense variant: loads every entry
    ++tested;
    const int KB = row_band_slots(N2, b);
    if (!row_band_ok(N2, b) || lim >= KB * N1) {
      std::printf("FAIL side %d lim %d: variant %d (KB %d) not valid\n", N, lim, b, KB);
      ok = false;
      continue;
    }
    for (int t = 0; t < N1; ++t)
      for (int m = 0; m < N2; ++m) {
        const int xk = t + N1 * m;
        const int fx = xk < (N + 1) / 2 ? xk : N - xk;
        if (fx <= lim && !(m < KB || m >= N2 - KB)) {
          std::printf("FAIL side %d lim %d: entry %d (lane %d, m %d) in band but not loaded\n", N, lim, xk, t, m);
          ok = false;
        }
      }
  }
  std::printf("checked %d %d\n", N, tested);
  return ok;
}

int main() {
  bool ok = true;
#define DTMM_CHECK_SIDE(N) ok = check_side<N>() && ok;
  DTMM_REG_SIDES(DTMM_CHECK_SIDE)
#undef DTMM_CHECK_SIDE
  std::printf(ok ? "OK\n" : "FAILED\n");
  return ok ? 0 : 1;
}
