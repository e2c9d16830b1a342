// Host check of the register transforms (dtmm_gb300/csrc/dtmm_regfft.cuh):
// compile-time twiddles against the C library, in-register DFTs and the
// two-step line transform (lanes run one after another, the lane barrier
// between the steps) against a direct O(N^2) DFT, both directions, in
// complex128.  Prints "max_err <name> <value>" lines and "OK" at the end.
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

#include "dtmm_regfft.cuh"

using namespace dtmm;
using C = std::complex<double>;

static double g_worst = 0.0;

static void report(const char* what, int n, double err, double tol) {
  std::printf("max_err %s %d %.3e\n", what, n, err);
  if (!(err <= tol)) {
    std::printf("FAIL %s %d\n", what, n);
    g_worst = 1.0;
  }
}

static std::vector<C> direct(const std::vector<C>& x, bool inv) {
  const int n = (int)x.size();
  std::vector<C> X(n);
  for (int k = 0; k < n; ++k) {
    C s = 0;
    for (int j = 0; j < n; ++j) {
      const long long e = (long long)j * k % n;
      const double a = (inv ? 2.0 : -2.0) * M_PI * (double)e / n;
      s += x[j] * C(std::cos(a), std::sin(a));
    }
    X[k] = s;
  }
  return X;
}

static std::vector<C> input(int n, int seed) {
  std::vector<C> x(n);
  unsigned s = 12345u + 7919u * seed + 104729u * n;
  for (int i = 0; i < n; ++i) {
    s = s * 1664525u + 1013904223u;
    const double a = (s >> 8) / 16777216.0 - 0.5;
    s = s * 1664525u + 1013904223u;
    const double b = (s >> 8) / 16777216.0 - 0.5;
    x[i] = C(a, b);
  }
  return x;
}

static double rel_err(const std::vector<C>& a, const std::vector<C>& b) {
  double num = 0, den = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    num += std::norm(a[i] - b[i]);
    den += std::norm(b[i]);
  }
  return std::sqrt(num / den);
}

template <int N, bool INV>
static void check_dft() {
  std::vector<C> x = input(N, INV);
  cpx<double> v[N];
  for (int i = 0; i < N; ++i) v[i] = mk<double>(x[i].real(), x[i].imag());
  RegDFTg<double, N, INV>::run(v);
  std::vector<C> got(N);
  for (int i = 0; i < N; ++i) got[i] = C(v[i].re, v[i].im);
  report(INV ? "regdft_inv" : "regdft_fwd", N, rel_err(got, direct(x, INV)), 1e-14);
}

template <int N>
static void check_dft_both() {
  check_dft<N, false>();
  check_dft<N, true>();
}

template <int N1, int N2, bool INV>
static void check_two_step() {
  using TS = TwoStep<N1, N2>;
  constexpr int N = N1 * N2;
  std::vector<C> x = input(N, 3 + INV);
  std::vector<cpx<double>> xch(N), out(N), tw(N), twt(N);
  for (int e = 0; e < N; ++e) {
    const double a = -2.0 * M_PI * e / N;
    tw[e] = mk<double>(std::cos(a), std::sin(a));
  }
  for (int e = 0; e < N; ++e) twt[e] = TS::twiddle_entry(tw.data(), e);  // lane-major table
  for (int t = 0; t < N1; ++t) {  // step 1, every lane
    cpx<double> v[N2];
    for (int m = 0; m < N2; ++m) v[m] = mk<double>(x[t + N1 * m].real(), x[t + N1 * m].imag());
    TS::template step1<double, INV>(v, xch.data(), 1, nullptr, twt.data(), t);
  }
  for (int t = 0; t < N1; ++t) {  // step 2, every lane
    cpx<double> u[TS::J][N1];
    TS::template step2<double, INV>(u, xch.data(), 1, t);
    TS::template store<double>(u, out.data(), 1, t, 1.0);
  }
  std::vector<C> got(N);
  for (int i = 0; i < N; ++i) got[i] = C(out[i].re, out[i].im);
  report(INV ? "two_step_inv" : "two_step_fwd", N, rel_err(got, direct(x, INV)), 1e-13);
}

// DFT of an input that is zero outside the band mask (entries m < KB, m >= N - KB)
template <int N, int KB, bool INV>
static void check_sparse() {
  constexpr unsigned M = band_mask(N, KB);
  std::vector<C> x = input(N, 7 + INV);
  for (int m = 0; m < N; ++m)
    if (!((M >> m) & 1u)) x[m] = 0;
  cpx<double> v[N];
  for (int i = 0; i < N; ++i) v[i] = mk<double>(x[i].real(), x[i].imag());
  RegDFTs<double, N, INV, M>::run(v);
  std::vector<C> got(N);
  for (int i = 0; i < N; ++i) got[i] = C(v[i].re, v[i].im);
  report(INV ? "sparse_dft_inv" : "sparse_dft_fwd", N * 100 + KB, rel_err(got, direct(x, INV)), 1e-14);
}

template <int N>
static void check_sparse_all() {
  check_sparse<N, 1, false>(); check_sparse<N, 1, true>();
  if constexpr (N > 4) { check_sparse<N, 2, false>(); check_sparse<N, 2, true>(); }
  if constexpr (N > 8) { check_sparse<N, N / 4, false>(); check_sparse<N, N / 4, true>(); }
  if constexpr (N > 16) { check_sparse<N, N / 8, false>(); check_sparse<N, N / 8, true>(); }
}

// two-step inverse transform of a band-limited line (|f| < KB N1) with the
// sparse step 1, lanes loading only their band entries
template <int N1, int N2, int KB>
static void check_band_line() {
  using TS = TwoStep<N1, N2>;
  constexpr int N = N1 * N2;
  std::vector<C> x = input(N, 11);
  for (int k = 0; k < N; ++k) {
    const int f = k < (N + 1) / 2 ? k : N - k;
    if (f >= KB * N1) x[k] = 0;
  }
  std::vector<cpx<double>> xch(N), out(N), tw(N), twt(N);
  for (int e = 0; e < N; ++e) {
    const double a = -2.0 * M_PI * e / N;
    tw[e] = mk<double>(std::cos(a), std::sin(a));
  }
  for (int e = 0; e < N; ++e) twt[e] = TS::twiddle_entry(tw.data(), e);
  for (int t = 0; t < N1; ++t) {
    cpx<double> v[N2];
    for (int m = 0; m < N2; ++m)
      v[m] = (m < KB || m >= N2 - KB) ? mk<double>(x[t + N1 * m].real(), x[t + N1 * m].imag()) : mk<double>(0, 0);
    TS::template step1<double, true, band_mask(N2, KB)>(v, xch.data(), 1, nullptr, twt.data(), t);
  }
  for (int t = 0; t < N1; ++t) {
    cpx<double> u[TS::J][N1];
    TS::template step2<double, true>(u, xch.data(), 1, t);
    TS::template store<double>(u, out.data(), 1, t, 1.0);
  }
  std::vector<C> got(N);
  for (int i = 0; i < N; ++i) got[i] = C(out[i].re, out[i].im);
  report("band_line_inv", N * 100 + KB, rel_err(got, direct(x, true)), 1e-13);
}

template <int N>
static void check_band() {
  constexpr int N1 = reg_lanes(N), N2 = N / N1;
  constexpr int K1 = N2 / 8 > 1 ? N2 / 8 : 1, K2 = N2 / 4 > 1 ? N2 / 4 : 1;
  if constexpr (2 * K1 < N2) check_band_line<N1, N2, K1>();
  if constexpr (2 * K2 < N2) check_band_line<N1, N2, K2>();
}

template <int N>
static void check_line() {
  constexpr int N1 = reg_lanes(N);
  static_assert(N1 > 0, "size without a register transform");
  check_two_step<N1, N / N1, false>();
  check_two_step<N1, N / N1, true>();
}

int main() {
  double worst = 0;
  for (int d = 1; d <= 4096; d = d * 3 + 1)
    for (int n = -d; n <= 2 * d; ++n) {
      // reference in long double on the reduced angle
      const long long r = ((n % d) + d) % d;
      const long double a = 2.0L * 3.14159265358979323846264338327950288L * (long double)r / (long double)d;
      worst = std::fmax(worst, std::fabs(ct::cos2pi(n, d) - (double)std::cos(a)));
      worst = std::fmax(worst, std::fabs(ct::sin2pi(n, d) - (double)std::sin(a)));
    }
  report("cos2pi_sin2pi", 0, worst, 4e-16);
  check_dft_both<2>(); check_dft_both<3>(); check_dft_both<4>(); check_dft_both<5>();
  check_dft_both<6>(); check_dft_both<7>(); check_dft_both<8>(); check_dft_both<9>();
  check_dft_both<10>(); check_dft_both<12>(); check_dft_both<14>(); check_dft_both<15>();
  check_dft_both<16>(); check_dft_both<18>(); check_dft_both<20>(); check_dft_both<21>();
  check_dft_both<24>(); check_dft_both<25>(); check_dft_both<27>(); check_dft_both<28>();
  check_dft_both<30>(); check_dft_both<32>();
  check_line<64>(); check_line<80>(); check_line<96>(); check_line<112>(); check_line<128>();
  check_line<144>(); check_line<160>(); check_line<192>(); check_line<224>(); check_line<240>();
  check_line<256>(); check_line<288>(); check_line<320>(); check_line<336>(); check_line<384>();
  check_line<400>(); check_line<432>(); check_line<448>(); check_line<480>(); check_line<512>();
  check_line<1024>();
  check_sparse_all<4>(); check_sparse_all<5>(); check_sparse_all<6>(); check_sparse_all<7>();
  check_sparse_all<8>(); check_sparse_all<9>(); check_sparse_all<10>(); check_sparse_all<12>();
  check_sparse_all<14>(); check_sparse_all<15>(); check_sparse_all<16>(); check_sparse_all<18>();
  check_sparse_all<20>(); check_sparse_all<21>(); check_sparse_all<24>(); check_sparse_all<25>();
  check_sparse_all<27>(); check_sparse_all<28>(); check_sparse_all<30>(); check_sparse_all<32>();
  check_band<64>(); check_band<80>(); check_band<96>(); check_band<112>(); check_band<128>();
  check_band<144>(); check_band<160>(); check_band<192>(); check_band<224>(); check_band<240>();
  check_band<256>(); check_band<288>(); check_band<320>(); check_band<336>(); check_band<384>();
  check_band<400>(); check_band<432>(); check_band<448>(); check_band<480>(); check_band<512>();
  check_band<1024>();
  std::printf(g_worst == 0.0 ? "OK\n" : "FAILED\n");
  return g_worst == 0.0 ? 0 : 1;
}
