// Register-resident line transforms for any 7-smooth length.
//
// A line of N = N1 * N2 points is transformed by a group of N1 lanes
// (N1 a power of two, N1 <= 32, so a group never straddles a warp):
//
//   step 1  lane t holds x[t + N1 m], m < N2, and computes the N2-point DFT
//           over m in registers, then multiplies entry k1 by W_N^(t k1);
//   swap    every lane writes its N2 values to the line's exchange buffer;
//   step 2  the N2 DFTs of length N1 (one per k1) are spread over the lanes,
//           lane t taking k1 = t, t + N1, ... < N2; entry k2 of the DFT for
//           k1 is X[k1 + N2 k2].
//
// Every DFT of up to 32 points runs in registers as a mixed-radix
// decimation in time (radix 4 first, then 2, 3, 5, 7) whose twiddles are
// compile-time constants; multiplications by 1, -1 and +-i are exact swaps
// and negations.  The constants come from `ct::cos2pi`, a Taylor series
// evaluated by the compiler after an exact octant reduction in integers.
//
// The two steps are separate functions so that a caller (or a host test)
// can place the lane barrier between them; both are __host__ __device__.
#pragma once

#include "dtmm_common.cuh"

namespace dtmm {

// ---------------------------------------------------------------------------
// compile-time trigonometry of rational multiples of 2 pi
// ---------------------------------------------------------------------------
namespace ct {

__host__ __device__ constexpr double taylor_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k <= 11; ++k) {
    term = -term * x2 / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}

__host__ __device__ constexpr double taylor_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k <= 11; ++k) {
    term = -term * x2 / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}

// cos(2 pi n / d): the angle is folded into [0, pi/4] with integer arithmetic
// (2 pi - a, pi - a, pi/2 - a), so the series only sees |x| <= pi/4
__host__ __device__ constexpr double cos2pi(long long n, long long d) {
  n %= d;
  if (n < 0) n += d;
  if (2 * n > d) n = d - n;  // cos(2 pi - a) = cos(a)
  double sign = 1.0;
  long long num = n, den = d;
  if (4 * num > den) {       // cos(a) = -cos(pi - a), pi - a = 2 pi (d - 2n) / (2d)
    num = den - 2 * num;
    den = 2 * den;
    sign = -1.0;
  }
  const double two_pi = 6.28318530717958647692528676655900577;
  if (8 * num > den)         // cos(a) = sin(pi/2 - a), pi/2 - a = 2 pi (den - 4 num) / (4 den)
    return sign * taylor_sin(two_pi * (double)(den - 4 * num) / (double)(4 * den));
  return sign * taylor_cos(two_pi * (double)num / (double)den);
}

// sin(2 pi n / d) = cos(2 pi (4n - d) / (4d))
__host__ __device__ constexpr double sin2pi(long long n, long long d) { return cos2pi(4 * n - d, 4 * d); }

}  // namespace ct

// v * exp(s 2 pi i E / N), s = -1 forward, +1 inverse
template <typename R, long long E, long long N, bool INV>
__host__ __device__ __forceinline__ cpx<R> rotc(cpx<R> v) {
  constexpr long long e = ((E % N) + N) % N;
  if constexpr (e == 0) {
    return v;
  } else if constexpr (2 * e == N) {
    return mk<R>(-v.re, -v.im);
  } else if constexpr (4 * e == N) {
    return INV ? mk<R>(-v.im, v.re) : mk<R>(v.im, -v.re);
  } else if constexpr (4 * e == 3 * N) {
    return INV ? mk<R>(v.im, -v.re) : mk<R>(-v.im, v.re);
  } else {
    constexpr R c = (R)ct::cos2pi(e, N);
    constexpr R s = INV ? (R)ct::sin2pi(e, N) : (R)-ct::sin2pi(e, N);
    return mk<R>(v.re * c - v.im * s, v.re * s + v.im * c);
  }
}

// ---------------------------------------------------------------------------
// small DFTs: 2, 4 and odd primes (symmetric pairs: X_s, X_{P-s} = a -+ i b)
// ---------------------------------------------------------------------------
template <typename R, int P, bool INV, int S, int J>
__host__ __device__ __forceinline__ void prime_acc(const cpx<R>* x, cpx<R>& a, cpx<R>& b) {
  if constexpr (J <= (P - 1) / 2) {
    constexpr R c = (R)ct::cos2pi((long long)J * S, P);
    constexpr R s = (R)ct::sin2pi((long long)J * S, P);
    const cpx<R> sp = x[J] + x[P - J], dm = x[J] - x[P - J];
    a = mk<R>(a.re + c * sp.re, a.im + c * sp.im);
    b = mk<R>(b.re + s * dm.re, b.im + s * dm.im);
    prime_acc<R, P, INV, S, J + 1>(x, a, b);
  }
}

template <typename R, int P, bool INV, int S>
__host__ __device__ __forceinline__ void prime_out(const cpx<R>* x, cpx<R>* X) {
  if constexpr (S <= (P - 1) / 2) {
    cpx<R> a = x[0], b = mk<R>((R)0, (R)0);
    prime_acc<R, P, INV, S, 1>(x, a, b);
    const cpx<R> ib = mk<R>(-b.im, b.re);  // i b
    X[S] = INV ? a + ib : a - ib;
    X[P - S] = INV ? a - ib : a + ib;
    prime_out<R, P, INV, S + 1>(x, X);
  }
}

template <typename R, int P, bool INV>
struct SmallDFT {
  __host__ __device__ static __forceinline__ void run(cpx<R>* v) {
    if constexpr (P == 1) {
    } else if constexpr (P == 2) {
      const cpx<R> a = v[0], b = v[1];
      v[0] = a + b;
      v[1] = a - b;
    } else if constexpr (P == 4) {
      const cpx<R> s02 = v[0] + v[2], d02 = v[0] - v[2], s13 = v[1] + v[3], d13 = v[1] - v[3];
      const cpx<R> jd = INV ? mk<R>(-d13.im, d13.re) : mk<R>(d13.im, -d13.re);
      v[0] = s02 + s13;
      v[2] = s02 - s13;
      v[1] = d02 + jd;
      v[3] = d02 - jd;
    } else {
      cpx<R> x[P];
#pragma unroll
      for (int i = 0; i < P; ++i) x[i] = v[i];
      cpx<R> s0 = x[0];
#pragma unroll
      for (int i = 1; i < P; ++i) s0 = s0 + x[i];
      prime_out<R, P, INV, 1>(x, v);
      v[0] = s0;
    }
  }
};

template <int N>
__host__ __device__ constexpr int first_radix() {
  return N % 4 == 0 ? 4 : (N % 2 == 0 ? 2 : (N % 3 == 0 ? 3 : (N % 5 == 0 ? 5 : (N % 7 == 0 ? 7 : N))));
}

// N-point DFT in registers, natural order in and out.  N = P Q, P the first
// radix: Y_p = DFT_Q(x[p + P m]); X[k + Q r] = sum_p W_N^(p k) Y_p[k] W_P^(p r).
template <typename R, int N, bool INV>
struct RegDFTg {
  static constexpr int P = first_radix<N>();
  static constexpr int Q = N / P;

  template <int K, int I>
  __host__ __device__ static __forceinline__ void gather(cpx<R> (&t)[P], const cpx<R> (&y)[P][Q]) {
    if constexpr (I < P) {
      t[I] = rotc<R, (long long)I * K, N, INV>(y[I][K]);
      gather<K, I + 1>(t, y);
    }
  }
  template <int K>
  __host__ __device__ static __forceinline__ void combine(cpx<R>* v, const cpx<R> (&y)[P][Q]) {
    if constexpr (K < Q) {
      cpx<R> t[P];
      gather<K, 0>(t, y);
      SmallDFT<R, P, INV>::run(t);
#pragma unroll
      for (int r = 0; r < P; ++r) v[K + Q * r] = t[r];
      combine<K + 1>(v, y);
    }
  }
  __host__ __device__ static __forceinline__ void run(cpx<R>* v) {
    if constexpr (Q == 1) {
      SmallDFT<R, P, INV>::run(v);
    } else {
      cpx<R> y[P][Q];
#pragma unroll
      for (int p = 0; p < P; ++p)
#pragma unroll
        for (int m = 0; m < Q; ++m) y[p][m] = v[p + P * m];
#pragma unroll
      for (int p = 0; p < P; ++p) RegDFTg<R, Q, INV>::run(y[p]);
      combine<0>(v, y);
    }
  }
};

// ---------------------------------------------------------------------------
// DFT of an input known to be zero outside a compile-time mask (bit m set:
// x[m] may be non-zero).  The decimation of RegDFTg is followed, but a
// sub-transform whose inputs are all zero is left out, one with a single
// non-zero input x[m0] becomes the rotations x[m0] W_N^(m0 k), and the
// combining DFTs only see the sub-transforms that exist.  A band-limited
// line (entries m < KB and m >= N - KB) costs about half the butterflies of
// the dense transform in its first stage.  Entries outside the mask must
// hold zeros (a dense prime-length stage still reads them).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr unsigned full_mask(int n) { return n >= 32 ? 0xffffffffu : ((1u << n) - 1u); }

// entries m < kb and m >= n - kb of an n-point line
__host__ __device__ constexpr unsigned band_mask(int n, int kb) {
  unsigned s = 0;
  for (int m = 0; m < n; ++m)
    if (m < kb || m >= n - kb) s |= 1u << m;
  return s;
}

// mask of the Q entries p + P m of a mask
__host__ __device__ constexpr unsigned stride_mask(unsigned mask, int p, int P, int Q) {
  unsigned s = 0;
  for (int m = 0; m < Q; ++m)
    if ((mask >> (p + P * m)) & 1u) s |= 1u << m;
  return s;
}

__host__ __device__ constexpr int mask_count(unsigned m) {
  int c = 0;
  for (; m; m &= m - 1) ++c;
  return c;
}

__host__ __device__ constexpr int mask_low(unsigned m) {
  int i = 0;
  while (!((m >> i) & 1u)) ++i;
  return i;
}

template <typename R, int N, bool INV, unsigned MASK>
struct RegDFTs {
  static constexpr int P = first_radix<N>();
  static constexpr int Q = N / P;

  // which of the P sub-transforms have a non-zero input
  __host__ __device__ static constexpr unsigned pmask() {
    unsigned s = 0;
    for (int p = 0; p < P; ++p)
      if (stride_mask(MASK, p, P, Q)) s |= 1u << p;
    return s;
  }

  template <int M0, int K>
  __host__ __device__ static __forceinline__ void rotations(cpx<R>* v, const cpx<R> x) {
    if constexpr (K < N) {
      v[K] = rotc<R, (long long)M0 * K, N, INV>(x);
      rotations<M0, K + 1>(v, x);
    }
  }

  template <int I>
  __host__ __device__ static __forceinline__ void subs(cpx<R> (&y)[P][Q], const cpx<R>* v) {
    if constexpr (I < P) {
      constexpr unsigned sm = stride_mask(MASK, I, P, Q);
      if constexpr (sm != 0) {
#pragma unroll
        for (int m = 0; m < Q; ++m) y[I][m] = v[I + P * m];
        RegDFTs<R, Q, INV, sm>::run(y[I]);
      }
      subs<I + 1>(y, v);
    }
  }

  template <int K, int I>
  __host__ __device__ static __forceinline__ void gather(cpx<R> (&t)[P], const cpx<R> (&y)[P][Q]) {
    if constexpr (I < P) {
      if constexpr ((pmask() >> I) & 1u)
        t[I] = rotc<R, (long long)I * K, N, INV>(y[I][K]);
      else
        t[I] = mk<R>((R)0, (R)0);
      gather<K, I + 1>(t, y);
    }
  }

  template <int K>
  __host__ __device__ static __forceinline__ void combine(cpx<R>* v, const cpx<R> (&y)[P][Q]) {
    if constexpr (K < Q) {
      cpx<R> t[P];
      gather<K, 0>(t, y);
      RegDFTs<R, P, INV, pmask()>::run(t);
#pragma unroll
      for (int r = 0; r < P; ++r) v[K + Q * r] = t[r];
      combine<K + 1>(v, y);
    }
  }

  __host__ __device__ static __forceinline__ void run(cpx<R>* v) {
    if constexpr (MASK == full_mask(N) || Q == 1) {
      RegDFTg<R, N, INV>::run(v);  // dense, or a prime length (reads the zeros)
    } else if constexpr (mask_count(MASK) == 1) {
      rotations<mask_low(MASK), 0>(v, v[mask_low(MASK)]);
    } else {
      cpx<R> y[P][Q];
      subs<0>(y, v);
      combine<0>(v, y);
    }
  }
};

// ---------------------------------------------------------------------------
// Two-step line transform, N = N1 * N2 (see the file comment).  Exchange
// element (k1, s) lives at xch[(k1 * N1 + (s ^ (k1 & (N1 - 1)))) * xs]: the
// writes of one k1 (lanes s) and the reads of one k1 (entries s) both touch
// N1 distinct consecutive slots.
// ---------------------------------------------------------------------------
template <int N1, int N2>
struct TwoStep {
  static_assert((N1 & (N1 - 1)) == 0 && N1 >= 1 && N1 <= 32, "lanes per line: power of two up to 32");
  static constexpr int N = N1 * N2;
  static constexpr int J = (N2 + N1 - 1) / N1;  // step-2 transforms per lane (the last round may be partial)
  static constexpr bool EVEN = N2 % N1 == 0;

  __host__ __device__ static __forceinline__ int slot(int k1, int s) { return k1 * N1 + (s ^ (k1 & (N1 - 1))); }

  // Twiddle table in lane-major order: twt[k1 * N1 + t] = W_N^(t k1), so the
  // N1 lanes of a group read N1 consecutive entries (no bank conflicts)
  template <typename R>
  __host__ __device__ static __forceinline__ cpx<R> twiddle_entry(const cpx<R>* tw_natural, int e) {
    return tw_natural[(e % N1) * (e / N1)];
  }

  // step 1: v[m] = x[t + N1 m] in; DFT over m, twiddle, write to the exchange.
  // Twiddles W_N^(t k1) come from `trow` (registers) or the lane-major table `twt`.
  // MASK: the entries m that may be non-zero (the others hold zeros).
  template <typename R, bool INV, unsigned MASK = full_mask(N2)>
  __host__ __device__ static __forceinline__ void step1(cpx<R> (&v)[N2], cpx<R>* xch, int xs, const cpx<R>* trow,
                                                        const cpx<R>* twt, int t) {
    RegDFTs<R, N2, INV, MASK>::run(v);
#pragma unroll
    for (int k1 = 1; k1 < N2; ++k1) {
      cpx<R> w = trow ? trow[k1] : twt[k1 * N1 + t];
      if (INV) w.im = -w.im;
      v[k1] = v[k1] * w;
    }
#pragma unroll
    for (int k1 = 0; k1 < N2; ++k1) xch[slot(k1, t) * xs] = v[k1];
  }

  // step 2 into registers: u[j][k2] = X[(t + N1 j) + N2 k2] for t + N1 j < N2
  template <typename R, bool INV>
  __host__ __device__ static __forceinline__ void step2(cpx<R> (&u)[J][N1], const cpx<R>* xch, int xs, int t) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int k1 = t + N1 * j;
      if (EVEN || k1 < N2) {
#pragma unroll
        for (int s = 0; s < N1; ++s) u[j][s] = xch[slot(k1, s) * xs];
        RegDFTg<R, N1, INV>::run(u[j]);
      }
    }
  }

  // write step 2's results in natural order: out[e * os] = X[e] * scale
  template <typename R>
  __host__ __device__ static __forceinline__ void store(const cpx<R> (&u)[J][N1], cpx<R>* out, int os, int t, R scale) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int k1 = t + N1 * j;
      if (EVEN || k1 < N2) {
#pragma unroll
        for (int k2 = 0; k2 < N1; ++k2) out[(k1 + N2 * k2) * os] = u[j][k2] * scale;
      }
    }
  }
  // store without a scale
  template <typename R>
  __host__ __device__ static __forceinline__ void store(const cpx<R> (&u)[J][N1], cpx<R>* out, int os, int t) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int k1 = t + N1 * j;
      if (EVEN || k1 < N2) {
#pragma unroll
        for (int k2 = 0; k2 < N1; ++k2) out[(k1 + N2 * k2) * os] = u[j][k2];
      }
    }
  }

  // EVEN only: step 2's results in the input's register order,
  // v[m] = X[t + N1 m] (k1 = t + N1 j, m = j + J k2)
  template <typename R>
  __host__ __device__ static __forceinline__ void to_lane_order(const cpx<R> (&u)[J][N1], cpx<R> (&v)[N2]) {
    static_assert(EVEN, "lane order needs N2 % N1 == 0");
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
      for (int k2 = 0; k2 < N1; ++k2) v[j + J * k2] = u[j][k2];
  }
};

// Register transform shape of an N-point line: lanes per line N1 (0 when N
// has no register transform); N2 = N / N1 <= 32 points per lane.
__host__ __device__ constexpr int reg_lanes(int n) {
  switch (n) {
    case 64: return 8;
    case 80: return 4;
    case 96: return 4;
    case 112: return 4;
    case 128: return 8;
    case 144: return 8;
    case 160: return 8;
    case 192: return 8;
    case 224: return 8;
    case 240: return 8;
    case 256: return 16;
    case 288: return 16;
    case 320: return 16;
    case 336: return 16;
    case 384: return 16;
    case 400: return 16;
    case 432: return 16;
    case 448: return 16;
    case 480: return 16;
    case 512: return 16;
    case 1024: return 32;
    default: return 0;
  }
}

__host__ __device__ constexpr bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

}  // namespace dtmm
