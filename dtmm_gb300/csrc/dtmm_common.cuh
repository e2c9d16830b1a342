// Shared device helpers of the dtmm_gb300 field-transfer kernels:
// interleaved complex arithmetic and an in-place mixed-radix FFT over lines
// held in shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dtmm {

// Interleaved complex number, bit-compatible with numpy complex64/complex128.
template <typename R>
struct __align__(2 * sizeof(R)) cpx {
  R re, im;
};

template <typename R>
__host__ __device__ __forceinline__ cpx<R> mk(R re, R im) {
  cpx<R> c;
  c.re = re;
  c.im = im;
  return c;
}
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator+(cpx<R> a, cpx<R> b) { return mk<R>(a.re + b.re, a.im + b.im); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator-(cpx<R> a, cpx<R> b) { return mk<R>(a.re - b.re, a.im - b.im); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator-(cpx<R> a) { return mk<R>(-a.re, -a.im); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator*(cpx<R> a, cpx<R> b) {
  return mk<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator*(cpx<R> a, R s) { return mk<R>(a.re * s, a.im * s); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator*(R s, cpx<R> a) { return mk<R>(a.re * s, a.im * s); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> conj(cpx<R> a) { return mk<R>(a.re, -a.im); }
// a * b + c
template <typename R>
__host__ __device__ __forceinline__ cpx<R> cfma(cpx<R> a, cpx<R> b, cpx<R> c) {
  return mk<R>(fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im)));
}
template <typename R>
__host__ __device__ __forceinline__ R norm2(cpx<R> a) { return a.re * a.re + a.im * a.im; }

// FP64 -> FP32 with round to nearest even, in integer arithmetic.  The
// hardware conversion issues at the FP64 rate (about 1/64 of the FP32 rate on
// this part), which bounds kernels that store FP64 results as FP32.  Every
// value whose result is a normal float (or whose input is a signed zero) is
// converted here with INT32 operations: rebias the exponent, keep the top 23
// mantissa bits and round on the 29 bits dropped (a carry out of the
// mantissa correctly bumps the exponent, up to infinity).  Results that are
// float subnormals, overflow, infinities and NaN take the hardware path.
__host__ __device__ __forceinline__ float f32_rn(double d) {
#ifdef __CUDA_ARCH__
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
#else
  unsigned long long u;
  __builtin_memcpy(&u, &d, sizeof(u));
#endif
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // FP32 biased exponent
  unsigned bits;
  if (e >= 1 && e <= 254) {
    bits = ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    bits += (rest > 0x10000000u || (rest == 0x10000000u && (bits & 1u))) ? 1u : 0u;
  } else if ((hi & 0x7fffffffu) == 0 && lo == 0) {
    bits = 0;
  } else {
    return (float)d;
  }
  bits |= hi & 0x80000000u;
#ifdef __CUDA_ARCH__
  return __uint_as_float(bits);
#else
  float f;
  __builtin_memcpy(&f, &bits, sizeof(f));
  return f;
#endif
}

// a double in the bulk precision R
template <typename R>
__host__ __device__ __forceinline__ R to_r(double d);
template <>
__host__ __device__ __forceinline__ double to_r<double>(double d) {
  return d;
}
template <>
__host__ __device__ __forceinline__ float to_r<float>(double d) {
  return f32_rn(d);
}

#ifdef __CUDACC__
// An FP32 value widened to FP64 exactly, in integer arithmetic (normal
// floats; others take the hardware conversion, which issues at the FP64 rate)
__device__ __forceinline__ double f64_of(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned long long u = ((unsigned long long)(b & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)u);
}

// Square root of x > 0 for results stored in FP32: the FP32 reciprocal square
// root of x (its input truncated to FP32 in integer arithmetic) refined by
// one Newton-Raphson step for 1/sqrt(x), y <- y (3 - x y^2) / 2, whose error
// is about 1.5 e^2 for a seed error e (<= 1e-6 here, so <= 2e-12), then
// sqrt(x) = x y: five FP64 operations.  Arguments outside the float range
// (and non-positive ones) take the library square root.
__device__ __forceinline__ double sqrt_pos_fast(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32);
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // FP32 biased exponent
  if ((hi & 0x80000000u) || e < 2 || e > 252) return sqrt(x);
  const float xf = __uint_as_float(((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | ((unsigned)u >> 29));
  const double y0 = f64_of(rsqrtf(xf));
  const double hy = (0.5 * x) * y0;
  const double y = y0 * fma(-hy, y0, 1.5);
  return x * y;
}

// Square root of x > 0 in three FP64 operations from an FP32 seed: with y0
// the FP32 reciprocal square root of x (input truncated to FP32 in integer
// arithmetic), r0 = x y0, hy0 = y0 / 2 and e = x - r0^2, sqrt(x) is
// fma(hy0, e, r0): one Newton-Raphson step for the square root, relative
// error about 1.5 s^2 for a seed error s (<= 3e-7 here, so <= 2e-13).  The
// parts are returned so that a caller can fold a term into the last fma.
// Arguments outside the float range, and non-positive ones, take the library
// square root (r0 = sqrt(x), hy0 = e = 0).
__device__ __forceinline__ void sqrt_newton(double x, double& r0, double& hy0, double& e) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32);
  const int ex = (int)((hi >> 20) & 0x7ffu) - 896;  // FP32 biased exponent
  if ((hi & 0x80000000u) || ex < 2 || ex > 252) {
    r0 = sqrt(x);
    hy0 = 0.0;
    e = 0.0;
    return;
  }
  const float xf = __uint_as_float(((unsigned)ex << 23) | ((hi & 0xfffffu) << 3) | ((unsigned)u >> 29));
  const float yf = rsqrtf(xf);
  r0 = x * f64_of(yf);
  hy0 = f64_of(0.5f * yf);
  e = fma(-r0, r0, x);
}

// 1 / x for a normal x from the FP32 reciprocal of x (input truncated to FP32
// in integer arithmetic) and two Newton-Raphson steps y <- y + y (1 - x y):
// four FP64 operations; the seed error (<= 2e-7) squares twice, so the result
// is within a few FP64 roundings of 1 / x.
// Arguments outside the float range take the FP64 division.
__device__ __forceinline__ double rcp_newton(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32);
  const int ex = (int)((hi >> 20) & 0x7ffu) - 896;
  if (ex < 2 || ex > 252) return 1.0 / x;
  const float xf = __uint_as_float((hi & 0x80000000u) | ((unsigned)ex << 23) | ((hi & 0xfffffu) << 3) |
                                   ((unsigned)u >> 29));
  double y = f64_of(__frcp_rn(xf));
  y = fma(y, fma(-x, y, 1.0), y);
  return fma(y, fma(-x, y, 1.0), y);
}

// d == 0 (either sign), in integer arithmetic
__device__ __forceinline__ bool is_zero_d(double d) { return (__double_as_longlong(d) << 1) == 0; }
#endif

__device__ __forceinline__ cpx<double> cvt_d(cpx<float> a) { return mk<double>(a.re, a.im); }
__device__ __forceinline__ cpx<double> cvt_d(cpx<double> a) { return a; }
template <typename R>
__device__ __forceinline__ cpx<R> cvt(cpx<double> a) { return mk<R>(to_r<R>(a.re), to_r<R>(a.im)); }

// Complex division and principal square root in FP64 (used by the
// eigen-solve).  Division scales by the larger component (Smith's method);
// the square root follows the textbook formula on the half-plane.
__device__ __forceinline__ cpx<double> cdiv(cpx<double> a, cpx<double> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    if (b.re == 0.0 && b.im == 0.0) {
      const double nan_ = __longlong_as_double(0x7ff8000000000000ULL);
      return mk<double>(nan_, nan_);
    }
    double r = b.im / b.re, den = b.re + b.im * r;
    return mk<double>((a.re + a.im * r) / den, (a.im - a.re * r) / den);
  } else {
    double r = b.re / b.im, den = b.re * r + b.im;
    return mk<double>((a.re * r + a.im) / den, (a.im * r - a.re) / den);
  }
}
__device__ __forceinline__ cpx<double> csqrt_d(cpx<double> z) {
  if (z.im == 0.0) {
    if (z.re >= 0.0) return mk<double>(sqrt(z.re), z.im);
    return mk<double>(0.0, copysign(sqrt(-z.re), z.im));
  }
  double m = hypot(z.re, z.im);
  double t = sqrt(0.5 * (m + fabs(z.re)));
  if (z.re >= 0.0) return mk<double>(t, z.im / (2.0 * t));
  return mk<double>(fabs(z.im) / (2.0 * t), copysign(t, z.im));
}
__device__ __forceinline__ cpx<double> cexp_i(cpx<double> z) {  // exp(i z)
  double s, c;
  sincos(z.re, &s, &c);
  double e = exp(-z.im);
  return mk<double>(e * c, e * s);
}
__device__ __forceinline__ cpx<float> cexp_i(cpx<float> z) {
  float s, c;
  sincosf(z.re, &s, &c);
  float e = expf(-z.im);
  return mk<float>(e * c, e * s);
}

// ---------------------------------------------------------------------------
// In-place mixed-radix FFT of lines stored in shared memory.
//
// A plan factors N into radices r[0..nr-1] (2, 3, 4, 5, 7, 8, or a prime from
// 11 to 31: those take a generic O(r^2) butterfly as a call).  The
// decimation-in-time form (`fft_dit`) takes its input in digit-reversed order
// and leaves the spectrum in natural order; the transposed network
// (`fft_dif`) takes natural order and leaves digit-reversed order.  Both run
// every butterfly in place (a butterfly reads and writes the same R slots), so
// one buffer suffices; `perm[n]` is the digit-reversed slot of element n, used
// by the global<->shared copies.  Twiddles come from `tw[t] = exp(-2 pi i t/N)`
// (conjugated for the inverse transform).
// Line l, element n lives at s[l * ls + n * es].  With `line_fastest`
// consecutive threads take consecutive lines (conflict-free for tiles whose
// lines are interleaved columns); otherwise consecutive butterflies of a line.
// ---------------------------------------------------------------------------
// at most kMaxPasses radices (every side up to 16384 needs fewer)
constexpr int kMaxPasses = 12;
struct FFTPlan {
  int n;
  int nr;
  int r[kMaxPasses];
  unsigned long long rbits;  // r[i] in bits [5i, 5i+5): read without dynamic indexing
};

__device__ __forceinline__ int plan_radix(const FFTPlan& p, int i) { return (int)((p.rbits >> (5 * i)) & 31ull); }

template <typename R, bool INV>
__device__ __forceinline__ cpx<R> twid(const cpx<R>* tw, int idx) {
  cpx<R> w = tw[idx];
  if (INV) w.im = -w.im;
  return w;
}

// R-point DFT in registers (R compile-time)
template <typename R, int RAD, bool INV>
__device__ __forceinline__ void dft_reg(cpx<R>* v, const cpx<R>* tw, int n) {
  if constexpr (RAD == 2) {
    cpx<R> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else if constexpr (RAD == 4) {
    cpx<R> s02 = v[0] + v[2], d02 = v[0] - v[2], s13 = v[1] + v[3], d13 = v[1] - v[3];
    // forward: W4 = -i ; inverse: W4 = +i
    cpx<R> jd = INV ? mk<R>(-d13.im, d13.re) : mk<R>(d13.im, -d13.re);
    v[0] = s02 + s13;
    v[2] = s02 - s13;
    v[1] = d02 + jd;
    v[3] = d02 - jd;
  } else if constexpr (RAD == 8) {
    // two 4-point DFTs (even / odd samples) joined by W8^k = exp(-+ i pi k / 4)
    cpx<R> e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft_reg<R, 4, INV>(e, tw, n);
    dft_reg<R, 4, INV>(o, tw, n);
    const R h = (R)0.70710678118654752440084436210485;  // 1 / sqrt(2)
    const cpx<R> a = o[1], b = o[2], c = o[3];
    if (INV) {
      o[1] = mk<R>(h * (a.re - a.im), h * (a.re + a.im));
      o[2] = mk<R>(-b.im, b.re);
      o[3] = mk<R>(-h * (c.re + c.im), h * (c.re - c.im));
    } else {
      o[1] = mk<R>(h * (a.re + a.im), h * (a.im - a.re));
      o[2] = mk<R>(b.im, -b.re);
      o[3] = mk<R>(h * (c.im - c.re), -h * (c.re + c.im));
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = e[k] + o[k];
      v[k + 4] = e[k] - o[k];
    }
  } else {
    cpx<R> in[RAD];
#pragma unroll
    for (int i = 0; i < RAD; ++i) in[i] = v[i];
    const int step = n / RAD;
#pragma unroll
    for (int q = 0; q < RAD; ++q) {
      cpx<R> acc = in[0];
#pragma unroll
      for (int i = 1; i < RAD; ++i) acc = cfma(in[i], twid<R, INV>(tw, ((q * i) % RAD) * step), acc);
      v[q] = acc;
    }
  }
}

// one butterfly of one pass; `ns` = length of the sub-transforms combined so far
template <typename R, int RAD, bool INV, bool DIT>
__device__ __forceinline__ void butterfly(cpx<R>* line, int es, int b, int ns, int nsh, int tstep, const cpx<R>* tw,
                                          int n) {
  int k, g;
  if (nsh >= 0) {
    k = b & (ns - 1);
    g = b >> nsh;
  } else {
    g = b / ns;
    k = b - g * ns;
  }
  cpx<R>* ptr = line + (g * ns * RAD + k) * es;
  const int stride = ns * es;
  cpx<R> v[RAD];
  if (DIT) {
    v[0] = ptr[0];
#pragma unroll
    for (int r = 1; r < RAD; ++r) v[r] = ptr[r * stride] * twid<R, INV>(tw, k * r * tstep);
    dft_reg<R, RAD, INV>(v, tw, n);
#pragma unroll
    for (int r = 0; r < RAD; ++r) ptr[r * stride] = v[r];
  } else {
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[r] = ptr[r * stride];
    dft_reg<R, RAD, INV>(v, tw, n);
    ptr[0] = v[0];
#pragma unroll
    for (int r = 1; r < RAD; ++r) ptr[r * stride] = v[r] * twid<R, INV>(tw, k * r * tstep);
  }
}

// radix-8 butterflies as a call: its 8 live complex values then cost
// registers only inside the call, not in every kernel that can take the pass
template <typename R, bool INV, bool DIT>
__device__ __noinline__ void butterfly8(cpx<R>* line, int es, int b, int ns, int nsh, int tstep, const cpx<R>* tw,
                                        int n) {
  butterfly<R, 8, INV, DIT>(line, es, b, ns, nsh, tstep, tw, n);
}

// butterfly of a prime radix 11 .. 31 (runtime), as a call: the r-point DFT
// sum_i v_i W_r^(q i) by direct summation
template <typename R, bool INV, bool DIT>
__device__ __noinline__ void butterfly_prime(cpx<R>* line, int es, int b, int ns, int tstep, const cpx<R>* tw, int n,
                                             int rad) {
  const int g = b / ns, k = b - g * ns;
  cpx<R>* ptr = line + (g * ns * rad + k) * es;
  const int stride = ns * es;
  const int step = n / rad;
  cpx<R> v[31];
  for (int r = 0; r < rad; ++r) v[r] = (DIT && r > 0) ? ptr[r * stride] * twid<R, INV>(tw, k * r * tstep) : ptr[r * stride];
  for (int q = 0; q < rad; ++q) {
    cpx<R> acc = v[0];
    int e = 0;  // (q * i) mod rad
    for (int i = 1; i < rad; ++i) {
      e += q;
      if (e >= rad) e -= rad;
      acc = cfma(v[i], twid<R, INV>(tw, e * step), acc);
    }
    ptr[q * stride] = (!DIT && q > 0) ? acc * twid<R, INV>(tw, k * q * tstep) : acc;
  }
}

__device__ __forceinline__ int log2_or_neg(int x) { return (x & (x - 1)) == 0 ? __ffs(x) - 1 : -1; }

// One pass over `nlines` lines by a group of `nthr` threads (thread index `tid`).
// line_fastest: consecutive threads take consecutive lines.
template <typename R, bool INV, bool DIT>
__device__ __forceinline__ void fft_pass(cpx<R>* s, int es, int ls, int nlines, bool line_fastest, const cpx<R>* tw,
                                         int n, int rad, int ns, int tid, int nthr) {
  const int nb = n / rad;
  const int total = nb * nlines;
  const int tstep = n / (ns * rad);
  const int nsh = log2_or_neg(ns);
  if (line_fastest && nthr % nlines == 0) {
    // each thread keeps one line; butterflies advance by nthr / nlines
    const int line = tid % nlines;
    const int bstep = nthr / nlines;
    cpx<R>* ln = s + line * ls;
    for (int b = tid / nlines; b < nb; b += bstep) {
      switch (rad) {
        case 4: butterfly<R, 4, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
        case 2: butterfly<R, 2, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
        case 3: butterfly<R, 3, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
        case 5: butterfly<R, 5, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
        case 8: butterfly8<R, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
        case 7: butterfly<R, 7, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
        default: butterfly_prime<R, INV, DIT>(ln, es, b, ns, tstep, tw, n, rad); break;
      }
    }
    return;
  }
  for (int t = tid; t < total; t += nthr) {
    int line, b;
    if (line_fastest) {
      line = t % nlines;
      b = t / nlines;
    } else {
      b = t % nb;
      line = t / nb;
    }
    cpx<R>* ln = s + line * ls;
    switch (rad) {
      case 4: butterfly<R, 4, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
      case 2: butterfly<R, 2, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
      case 3: butterfly<R, 3, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
      case 5: butterfly<R, 5, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
      case 8: butterfly8<R, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
      case 7: butterfly<R, 7, INV, DIT>(ln, es, b, ns, nsh, tstep, tw, n); break;
      default: butterfly_prime<R, INV, DIT>(ln, es, b, ns, tstep, tw, n, rad); break;
    }
  }
}

// decimation in time over the whole block: digit-reversed in, natural out
template <typename R, bool INV>
__device__ void fft_dit(cpx<R>* s, int es, int ls, int nlines, bool line_fastest, const cpx<R>* tw,
                        const FFTPlan& p) {
  int ns = 1;
  for (int ip = 0; ip < p.nr; ++ip) {
    const int rad = plan_radix(p, ip);
    fft_pass<R, INV, true>(s, es, ls, nlines, line_fastest, tw, p.n, rad, ns, threadIdx.x, blockDim.x);
    ns *= rad;
    __syncthreads();
  }
}

// transposed network over the whole block: natural in, digit-reversed out
template <typename R, bool INV>
__device__ void fft_dif(cpx<R>* s, int es, int ls, int nlines, bool line_fastest, const cpx<R>* tw,
                        const FFTPlan& p) {
  int ns = p.n;
  for (int ip = p.nr - 1; ip >= 0; --ip) {
    const int rad = plan_radix(p, ip);
    ns /= rad;
    fft_pass<R, INV, false>(s, es, ls, nlines, line_fastest, tw, p.n, rad, ns, threadIdx.x, blockDim.x);
    __syncthreads();
  }
}

// the same, one warp per line: warp w transforms lines w, w + nwarps, ...
// (only warp-level synchronisation between passes)
template <typename R, bool INV, bool DIT>
__device__ void fft_lines_warp(cpx<R>* s, int ls, int nlines, const cpx<R>* tw, const FFTPlan& p) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int l = warp; l < nlines; l += nwarps) {
    cpx<R>* ln = s + l * ls;
    if (DIT) {
      int ns = 1;
      for (int ip = 0; ip < p.nr; ++ip) {
        const int rad = plan_radix(p, ip);
        fft_pass<R, INV, true>(ln, 1, 0, 1, false, tw, p.n, rad, ns, lane, 32);
        ns *= rad;
        __syncwarp();
      }
    } else {
      int ns = p.n;
      for (int ip = p.nr - 1; ip >= 0; --ip) {
        const int rad = plan_radix(p, ip);
        ns /= rad;
        fft_pass<R, INV, false>(ln, 1, 0, 1, false, tw, p.n, rad, ns, lane, 32);
        __syncwarp();
      }
    }
  }
}

}  // namespace dtmm
