// Host check of the library's integer FP64 -> FP32 conversion (f32_rn in
// dtmm_common.cuh) against the host's IEEE conversion (round to nearest
// even): random bit patterns over the whole double range, values on and
// next to every rounding tie, the float normal / subnormal / overflow
// boundaries, signed zeros, infinities and NaN.  Prints the number of
// mismatches and "OK" when there are none.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "dtmm_common.cuh"

static uint64_t g_checked = 0, g_bad = 0;

static void check(double d) {
  const float want = (float)d, got = dtmm::f32_rn(d);
  uint32_t a, b;
  std::memcpy(&a, &want, 4);
  std::memcpy(&b, &got, 4);
  ++g_checked;
  const bool both_nan = std::isnan(want) && std::isnan(got);
  if (a != b && !both_nan) {
    if (g_bad < 10) std::printf("mismatch %.17g: want %08x got %08x\n", d, a, b);
    ++g_bad;
  }
}

static double from_bits(uint64_t u) {
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}

int main() {
  std::mt19937_64 rng(12345);
  for (int i = 0; i < 4000000; ++i) check(from_bits(rng()));  // every exponent, sign, NaN payloads
  std::uniform_real_distribution<double> ue(-160.0, 160.0);
  for (int i = 0; i < 4000000; ++i) {  // the normal float range and both of its edges
    const double m = std::ldexp(1.0, (int)std::floor(ue(rng)));
    check(m * (1.0 + (double)(rng() >> 12) * 0x1p-52) * ((rng() & 1) ? 1.0 : -1.0));
  }
  // exact ties and their neighbours: float mantissa f plus half an ulp
  for (int i = 0; i < 2000000; ++i) {
    const int e = (int)(rng() % 300) - 150;
    const uint64_t f = rng() & 0x7fffffu;
    const double base = std::ldexp(1.0 + (double)f * 0x1p-23, e);
    const double half = std::ldexp(0x1p-24, e);
    check(base + half);
    check(std::nextafter(base + half, 0.0));
    check(std::nextafter(base + half, 1e300));
    check(-(base + half));
  }
  const double specials[] = {0.0, -0.0, std::numeric_limits<double>::infinity(),
                             -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::quiet_NaN(),
                             (double)std::numeric_limits<float>::max(), (double)std::numeric_limits<float>::min(),
                             (double)std::numeric_limits<float>::denorm_min(), 3.4028235677973366e38,
                             3.4028235677973362e38, 1.1754942807573643e-38, 1.1754943508222875e-38,
                             std::numeric_limits<double>::denorm_min(), std::numeric_limits<double>::min(),
                             std::numeric_limits<double>::max(), 1.0, -1.0, 0.1, 1e-45, 7e-46};
  for (double d : specials) {
    check(d);
    check(-d);
    check(std::nextafter(d, 0.0));
    check(std::nextafter(d, 1e308));
  }
  std::printf("checked %llu mismatches %llu\n", (unsigned long long)g_checked, (unsigned long long)g_bad);
  std::printf(g_bad == 0 ? "OK\n" : "FAILED\n");
  return g_bad == 0 ? 0 : 1;
}
