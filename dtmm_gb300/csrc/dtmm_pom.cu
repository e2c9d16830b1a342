// POM image formation on transferred fields (the consumer of transfer_field's
// output in dtmm's field viewer): polarizer / window / analyzer on the field
// (calculate_pom_field, dtmm/field_viewer.py:70-143, real-space path without
// refocus), the normal Poynting component per pixel and wavelength
// (field2specter / field2spectersum, dtmm/field.py:784-847) and the specter ->
// XYZ -> sRGB or gray -> transfer-curve conversion (specter2color,
// dtmm/color.py:52-224), separately and fused into one pass per pixel.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "../../include/dtmm_gb300.h"
#include "dtmm_common.cuh"

using namespace dtmm;

namespace dtmm {
std::string& last_error_slot();  // the text dtmm_last_error returns (dtmm_capi.cu)
}

namespace {

int pom_fail(int code, const char* msg) {
  last_error_slot() = msg;
  return code;
}

// sRGB primaries with the D65 white point (dtmm/color.py:41-43)
__constant__ double kXYZ2RGB[3][3] = {{3.2404542, -1.5371385, -0.4985314},
                                      {-0.9692660, 1.8760108, 0.0415560},
                                      {0.0556434, -0.2040259, 1.0572252}};
__constant__ float kXYZ2RGBf[3][3] = {{3.2404542f, -1.5371385f, -0.4985314f},
                                      {-0.9692660f, 1.8760108f, 0.0415560f},
                                      {0.0556434f, -0.2040259f, 1.0572252f}};
template <typename R>
__device__ __forceinline__ R xyz2rgb_coef(int k, int j);
template <>
__device__ __forceinline__ double xyz2rgb_coef<double>(int k, int j) { return kXYZ2RGB[k][j]; }
template <>
__device__ __forceinline__ float xyz2rgb_coef<float>(int k, int j) { return kXYZ2RGBf[k][j]; }

struct PomArgs {
  int H, W, nlam, nset, npol;
  double j0r, j0i, j1r, j1i;  // jones vector
  const cpx<double>* pmat;    // 4x4 or null
  const double* window;       // H x W or null
};

// Per-block copies of the small operands in the bulk precision R: every
// conversion from their FP64 inputs happens once per block, not per pixel
// (a float <-> double conversion issues at the FP64 rate, about 1/64 of the
// FP32 rate on this part, and would otherwise bound the kernel).
constexpr int kStagedLam = 1024;  // colour-matching rows staged in shared memory

template <typename R>
struct PomStage {
  cpx<R> pm[16];
  cpx<R> c, s;  // jones vector
  int has_pm;
};

template <typename R>
__device__ __forceinline__ void pom_stage(const PomArgs& a, PomStage<R>& st) {
  if (threadIdx.x < 16) st.pm[threadIdx.x] = a.pmat ? cvt<R>(a.pmat[threadIdx.x]) : mk<R>((R)0, (R)0);
  if (threadIdx.x == 0) {
    st.c = mk<R>((R)a.j0r, (R)a.j0i);
    st.s = mk<R>((R)a.j1r, (R)a.j1i);
    st.has_pm = a.pmat != nullptr;
  }
}

// one image's field at pixel p, after polarizer, window (w, already in R)
// and analyzer, in the bulk precision R (complex64 fields: FP32 arithmetic)
template <typename R>
__device__ __forceinline__ void pom_pixel(const PomArgs& a, const PomStage<R>& st, const cpx<R>* __restrict__ f,
                                          int set, int lam, long long p, bool windowed, R w, cpx<R> g[4]) {
  const long long HW = (long long)a.H * a.W;
  if (a.npol == 2) {
    const cpx<R>* fx = f + (((long long)set * 2 + 0) * a.nlam + lam) * 4 * HW + p;
    const cpx<R>* fy = f + (((long long)set * 2 + 1) * a.nlam + lam) * 4 * HW + p;
    cpx<R> x[4], y[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      x[k] = fx[k * HW];
      y[k] = fy[k * HW];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = x[k] * st.c + y[k] * st.s;
  } else {
    const cpx<R>* fi = f + ((long long)set * a.nlam + lam) * 4 * HW + p;
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = fi[k * HW];
  }
  if (windowed) {
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = g[k] * w;
  }
  if (st.has_pm) {
    cpx<R> o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      cpx<R> acc = mk<R>((R)0, (R)0);
#pragma unroll
      for (int j = 0; j < 4; ++j) acc = acc + st.pm[i * 4 + j] * g[j];
      o[i] = acc;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = o[k];
  }
}

template <typename R>
__device__ __forceinline__ R poynting(const cpx<R> g[4]) {
  return (g[0].re * g[1].re + g[0].im * g[1].im) - (g[2].re * g[3].re + g[2].im * g[3].im);
}

// out[set][lam][4][H][W]
template <typename R>
__global__ void k_pom_field(PomArgs a, const cpx<R>* __restrict__ f, cpx<R>* __restrict__ out) {
  __shared__ PomStage<R> st;
  pom_stage<R>(a, st);
  __syncthreads();
  const long long HW = (long long)a.H * a.W;
  const int sl = blockIdx.y, set = sl / a.nlam, lam = sl - set * a.nlam;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < HW; p += (long long)gridDim.x * blockDim.x) {
    cpx<R> g[4];
    const R w = a.window ? (R)a.window[p] : (R)1;
    pom_pixel<R>(a, st, f, set, lam, p, a.window != nullptr, w, g);
    cpx<R>* o = out + ((long long)set * a.nlam + lam) * 4 * HW + p;
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k * HW] = g[k];
  }
}

// spec[s][y][x][lam], s < nset (or one summed set)
template <typename R>
__global__ void k_field2specter(int H, int W, int nlam, int nset, int sum, const cpx<R>* __restrict__ f,
                                double* __restrict__ spec) {
  const long long HW = (long long)H * W;
  const int so = blockIdx.y;  // output set
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < HW; p += (long long)gridDim.x * blockDim.x) {
    for (int lam = 0; lam < nlam; ++lam) {
      double acc = 0.0;
      const int s0 = sum ? 0 : so, s1 = sum ? nset : so + 1;
      for (int s = s0; s < s1; ++s) {
        const cpx<R>* fi = f + ((long long)s * nlam + lam) * 4 * HW + p;
        cpx<double> g[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) g[k] = cvt_d(fi[k * HW]);
        acc += poynting<double>(g);
      }
      spec[((long long)so * HW + p) * nlam + lam] = acc;
    }
  }
}

// XYZ -> normalise -> linear RGB or gray -> transfer curve
// norm_div: divisor (0 = none); gamma: 0 none, < 0 sRGB, > 0 power 1/gamma
// v^e for v > 0: FP32 through the SFU (__powf, 2^(e log2 v)), whose error is
// a few ulp, far below the float32 image's resolution; FP64 through pow
__device__ __forceinline__ float pos_pow(float v, float e) { return __powf(v, e); }
__device__ __forceinline__ double pos_pow(double v, double e) { return pow(v, e); }
template <typename R>
__device__ __forceinline__ R srgb_curve(R v) {
  if (v < (R)0.0031308) return v < (R)0 ? (R)0 : (R)12.92 * v;
  return v > (R)1 ? (R)1 : ((R)1 + (R)0.055) * pos_pow(v, (R)1 / (R)2.4) - (R)0.055;
}
template <typename R>
__device__ __forceinline__ R power_curve(R v, R gamma) {
  if (v > (R)1) return (R)1;
  if (v <= (R)0) return (R)0;
  return pos_pow(v, (R)1 / gamma);
}
template <typename R>
__device__ __forceinline__ void xyz_to_out(R xyz[3], R norm_div, int gray, R gamma, R rgb[3]) {
  if (norm_div != (R)0)
    for (int k = 0; k < 3; ++k) xyz[k] = xyz[k] / norm_div;
  if (gray) {
    rgb[0] = rgb[1] = rgb[2] = xyz[1];
  } else {
    for (int k = 0; k < 3; ++k)
      rgb[k] = xyz2rgb_coef<R>(k, 0) * xyz[0] + xyz2rgb_coef<R>(k, 1) * xyz[1] + xyz2rgb_coef<R>(k, 2) * xyz[2];
  }
  if (gamma < (R)0) {
    for (int k = 0; k < 3; ++k) rgb[k] = srgb_curve<R>(rgb[k]);
  } else if (gamma > (R)0) {
    for (int k = 0; k < 3; ++k) rgb[k] = power_curve<R>(rgb[k], gamma);
  }
}

// xyz (or, with `convert`, the final colour) of every pixel of a specter
template <typename T>
__global__ void k_specter2color(long long npix, int nlam, const double* __restrict__ spec,
                                const double* __restrict__ cmf, double norm_div, int gray, double gamma, int convert,
                                T* __restrict__ out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    double xyz[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < nlam; ++i) {
      const double s = spec[p * nlam + i];
      for (int k = 0; k < 3; ++k) xyz[k] = xyz[k] + cmf[i * 3 + k] * s;
    }
    double rgb[3];
    if (convert) {
      xyz_to_out<double>(xyz, norm_div, gray, gamma, rgb);
    } else {
      rgb[0] = xyz[0];
      rgb[1] = xyz[1];
      rgb[2] = xyz[2];
    }
    for (int k = 0; k < 3; ++k) out[p * 3 + k] = (T)rgb[k];
  }
}

// normalisation by the image maximum (norm=True): one block finds the
// maximum of every XYZ value, then converts every pixel in place (the
// maximum is exact whatever the reduction order); arithmetic in R
template <typename T, typename R>
__global__ void __launch_bounds__(1024) k_color_by_max(long long npix, int gray, double gamma, T* __restrict__ io) {
  __shared__ R red[1024];
  R m = -INFINITY;
  for (long long i = threadIdx.x; i < npix * 3; i += blockDim.x) m = fmax(m, (R)io[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const R mx = red[0];
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    R xyz[3] = {(R)io[p * 3], (R)io[p * 3 + 1], (R)io[p * 3 + 2]};
    R rgb[3];
    xyz_to_out<R>(xyz, mx, gray, (R)gamma, rgb);
    for (int k = 0; k < 3; ++k) io[p * 3 + k] = (T)rgb[k];
  }
}

// fused: polarizer / window / analyzer, Poynting summed over sets, XYZ,
// colour; every step in the bulk precision R (FP32 for complex64 fields)
template <typename R, typename T>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 1)
    k_pom_image(PomArgs a, const cpx<R>* __restrict__ f, const double* __restrict__ cmf, double norm_div, int gray,
                double gamma, int convert, T* __restrict__ out) {
  __shared__ PomStage<R> st;
  __shared__ R s_cmf[kStagedLam * 3];
  pom_stage<R>(a, st);
  const int staged = min(a.nlam, kStagedLam);
  for (int i = threadIdx.x; i < staged * 3; i += blockDim.x) s_cmf[i] = (R)cmf[i];
  __syncthreads();
  const R nd = (R)norm_div, gm = (R)gamma;
  const long long HW = (long long)a.H * a.W;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < HW; p += (long long)gridDim.x * blockDim.x) {
    const R w = a.window ? (R)a.window[p] : (R)1;
    R xyz[3] = {(R)0, (R)0, (R)0};
    for (int lam = 0; lam < a.nlam; ++lam) {
      R s = (R)0;
      for (int set = 0; set < a.nset; ++set) {
        cpx<R> g[4];
        pom_pixel<R>(a, st, f, set, lam, p, a.window != nullptr, w, g);
        s += poynting<R>(g);
      }
      if (lam < kStagedLam) {
        for (int k = 0; k < 3; ++k) xyz[k] = xyz[k] + s_cmf[lam * 3 + k] * s;
      } else {
        for (int k = 0; k < 3; ++k) xyz[k] = xyz[k] + (R)cmf[lam * 3 + k] * s;
      }
    }
    R rgb[3];
    if (convert) {
      xyz_to_out<R>(xyz, nd, gray, gm, rgb);
    } else {
      rgb[0] = xyz[0];
      rgb[1] = xyz[1];
      rgb[2] = xyz[2];
    }
    for (int k = 0; k < 3; ++k) out[p * 3 + k] = (T)rgb[k];
  }
}

int check_pom(const dtmm_pom_desc* d) {
  if (!d) return pom_fail(DTMM_EINVAL, "null descriptor");
  if (d->height < 1 || d->width < 1) return pom_fail(DTMM_EINVAL, "grid must be at least 1x1");
  if (d->nlam < 1 || d->nset < 1) return pom_fail(DTMM_EINVAL, "empty wavelength or set axis");
  if (d->npol != 1 && d->npol != 2) return pom_fail(DTMM_EINVAL, "npol must be 1 or 2");
  if ((long long)d->nset * d->nlam > 65535) return pom_fail(DTMM_EINVAL, "too many images");
  if (d->precision != DTMM_PRECISION_MIXED && d->precision != DTMM_PRECISION_DOUBLE)
    return pom_fail(DTMM_EINVAL, "invalid precision");
  return DTMM_OK;
}

PomArgs args_of(const dtmm_pom_desc* d) {
  PomArgs a;
  a.H = d->height;
  a.W = d->width;
  a.nlam = d->nlam;
  a.nset = d->nset;
  a.npol = d->npol;
  a.j0r = d->jvec[0];
  a.j0i = d->jvec[1];
  a.j1r = d->jvec[2];
  a.j1i = d->jvec[3];
  a.pmat = (const cpx<double>*)d->pmat;
  a.window = d->window;
  return a;
}

unsigned blocks_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 1216); }

int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    last_error_slot() = std::string(what) + ": " + cudaGetErrorString(e);
    return DTMM_ECUDA;
  }
  return DTMM_OK;
}

}  // namespace

extern "C" {

int dtmm_pom_field(const dtmm_pom_desc* d, const void* field, void* out, void* stream) {
  last_error_slot().clear();
  int rc = check_pom(d);
  if (rc) return rc;
  if (!field || !out) return pom_fail(DTMM_EINVAL, "null field");
  const PomArgs a = args_of(d);
  dim3 grid(blocks_for((long long)a.H * a.W), a.nset * a.nlam);
  cudaStream_t st = (cudaStream_t)stream;
  if (d->precision == DTMM_PRECISION_DOUBLE)
    k_pom_field<double><<<grid, 256, 0, st>>>(a, (const cpx<double>*)field, (cpx<double>*)out);
  else
    k_pom_field<float><<<grid, 256, 0, st>>>(a, (const cpx<float>*)field, (cpx<float>*)out);
  return launched("k_pom_field");
}

int dtmm_field2specter(int height, int width, int nlam, int nset, int sum_sets, int precision, const void* field,
                       double* spec, void* stream) {
  last_error_slot().clear();
  if (height < 1 || width < 1 || nlam < 1 || nset < 1) return pom_fail(DTMM_EINVAL, "empty axis");
  if (nset > 65535) return pom_fail(DTMM_EINVAL, "too many sets");
  if (!field || !spec) return pom_fail(DTMM_EINVAL, "null pointer");
  if (precision != DTMM_PRECISION_MIXED && precision != DTMM_PRECISION_DOUBLE)
    return pom_fail(DTMM_EINVAL, "invalid precision");
  dim3 grid(blocks_for((long long)height * width), sum_sets ? 1 : nset);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == DTMM_PRECISION_DOUBLE)
    k_field2specter<double><<<grid, 256, 0, st>>>(height, width, nlam, nset, sum_sets, (const cpx<double>*)field,
                                                   spec);
  else
    k_field2specter<float><<<grid, 256, 0, st>>>(height, width, nlam, nset, sum_sets, (const cpx<float>*)field,
                                                  spec);
  return launched("k_field2specter");
}

int dtmm_specter2color(long long npix, int nlam, const double* spec, const double* cmf, int norm_mode,
                       double norm_value, double gamma, int gray, double* rgb, void* stream) {
  last_error_slot().clear();
  if (npix < 1 || nlam < 1) return pom_fail(DTMM_EINVAL, "empty specter");
  if (!spec || !cmf || !rgb) return pom_fail(DTMM_EINVAL, "null pointer");
  if (norm_mode < 0 || norm_mode > 2) return pom_fail(DTMM_EINVAL, "invalid norm mode");
  cudaStream_t st = (cudaStream_t)stream;
  const double div = norm_mode == 1 ? norm_value : 0.0;
  k_specter2color<double><<<blocks_for(npix), 256, 0, st>>>(npix, nlam, spec, cmf, div, gray, gamma,
                                                            norm_mode != 2, rgb);
  int rc = launched("k_specter2color");
  if (rc || norm_mode != 2) return rc;
  k_color_by_max<double, double><<<1, 1024, 0, st>>>(npix, gray, gamma, rgb);
  return launched("k_color_by_max");
}

int dtmm_pom_image(const dtmm_pom_desc* d, const void* field, const double* cmf, int norm_mode, double norm_value,
                   double gamma, int gray, float* rgb, void* stream) {
  last_error_slot().clear();
  int rc = check_pom(d);
  if (rc) return rc;
  if (!field || !cmf || !rgb) return pom_fail(DTMM_EINVAL, "null pointer");
  if (norm_mode < 0 || norm_mode > 2) return pom_fail(DTMM_EINVAL, "invalid norm mode");
  const PomArgs a = args_of(d);
  const long long hw = (long long)a.H * a.W;
  const double div = norm_mode == 1 ? norm_value : 0.0;
  cudaStream_t st = (cudaStream_t)stream;
  if (d->precision == DTMM_PRECISION_DOUBLE)
    k_pom_image<double, float><<<blocks_for(hw), 256, 0, st>>>(a, (const cpx<double>*)field, cmf, div, gray, gamma,
                                                                norm_mode != 2, rgb);
  else
    k_pom_image<float, float><<<blocks_for(hw), 256, 0, st>>>(a, (const cpx<float>*)field, cmf, div, gray, gamma,
                                                               norm_mode != 2, rgb);
  rc = launched("k_pom_image");
  if (rc || norm_mode != 2) return rc;
  if (d->precision == DTMM_PRECISION_DOUBLE)
    k_color_by_max<float, double><<<1, 1024, 0, st>>>(hw, gray, gamma, rgb);
  else
    k_color_by_max<float, float><<<1, 1024, 0, st>>>(hw, gray, gamma, rgb);
  return launched("k_color_by_max");
}

}  // extern "C"
