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

__device__ __forceinline__ cpx<double> cvt_d(cpx<float> a) { return mk<double>(a.re, a.im); }
__device__ __forceinline__ cpx<double> cvt_d(cpx<double> a) { return a; }
template <typename R>
__device__ __forceinline__ cpx<R> cvt(cpx<double> a) { return mk<R>((R)a.re, (R)a.im); }

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
// A plan factors N into radices r[0..nr-1] (each 2, 3, 4, 5 or 7).  The
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
struct FFTPlan {
  int n;
  int nr;
  int r[14];
};

template <typename R, bool INV>
__device__ __forceinline__ cpx<R> twid(const cpx<R>* tw, int idx) {
  cpx<R> w = tw[idx];
  if (INV) w.im = -w.im;
  return w;
}

template <typename R, bool INV>
__device__ __forceinline__ void dft_small(cpx<R>* v, int rad, const cpx<R>* tw, int n) {
  if (rad == 2) {
    cpx<R> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else if (rad == 4) {
    cpx<R> s02 = v[0] + v[2], d02 = v[0] - v[2], s13 = v[1] + v[3], d13 = v[1] - v[3];
    // forward: W4 = -i ; inverse: W4 = +i
    cpx<R> jd = INV ? mk<R>(-d13.im, d13.re) : mk<R>(d13.im, -d13.re);
    v[0] = s02 + s13;
    v[2] = s02 - s13;
    v[1] = d02 + jd;
    v[3] = d02 - jd;
  } else {
    cpx<R> in[7];
    for (int i = 0; i < rad; ++i) in[i] = v[i];
    const int step = n / rad;
    for (int q = 0; q < rad; ++q) {
      cpx<R> acc = in[0];
      for (int i = 1; i < rad; ++i) acc = cfma(in[i], twid<R, INV>(tw, ((q * i) % rad) * step), acc);
      v[q] = acc;
    }
  }
}

// decimation in time: digit-reversed in, natural out
template <typename R, bool INV>
__device__ void fft_dit(cpx<R>* s, int es, int ls, int nlines, bool line_fastest, const cpx<R>* tw,
                        const FFTPlan& p) {
  const int n = p.n;
  int ns = 1;
  for (int ip = 0; ip < p.nr; ++ip) {
    const int rad = p.r[ip];
    const int nb = n / rad;
    const int total = nb * nlines;
    const int tstep = n / (ns * rad);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int line, b;
      if (line_fastest) {
        line = t % nlines;
        b = t / nlines;
      } else {
        b = t % nb;
        line = t / nb;
      }
      const int k = b % ns;
      const int base = (b / ns) * ns * rad + k;
      cpx<R>* ptr = s + line * ls + base * es;
      cpx<R> v[7];
      v[0] = ptr[0];
      for (int r = 1; r < rad; ++r) v[r] = ptr[r * ns * es] * twid<R, INV>(tw, k * r * tstep);
      dft_small<R, INV>(v, rad, tw, n);
      for (int r = 0; r < rad; ++r) ptr[r * ns * es] = v[r];
    }
    ns *= rad;
    __syncthreads();
  }
}

// transposed network: natural in, digit-reversed out
template <typename R, bool INV>
__device__ void fft_dif(cpx<R>* s, int es, int ls, int nlines, bool line_fastest, const cpx<R>* tw,
                        const FFTPlan& p) {
  const int n = p.n;
  int ns = n;
  for (int ip = p.nr - 1; ip >= 0; --ip) {
    const int rad = p.r[ip];
    ns /= rad;
    const int nb = n / rad;
    const int total = nb * nlines;
    const int tstep = n / (ns * rad);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int line, b;
      if (line_fastest) {
        line = t % nlines;
        b = t / nlines;
      } else {
        b = t % nb;
        line = t / nb;
      }
      const int k = b % ns;
      const int base = (b / ns) * ns * rad + k;
      cpx<R>* ptr = s + line * ls + base * es;
      cpx<R> v[7];
      for (int r = 0; r < rad; ++r) v[r] = ptr[r * ns * es];
      dft_small<R, INV>(v, rad, tw, n);
      ptr[0] = v[0];
      for (int r = 1; r < rad; ++r) ptr[r * ns * es] = v[r] * twid<R, INV>(tw, k * r * tstep);
    }
    __syncthreads();
  }
}

}  // namespace dtmm
