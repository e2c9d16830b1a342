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

struct PomArgs {
  int H, W, nlam, nset, npol;
  double j0r, j0i, j1r, j1i;  // jones vector
  const cpx<double>* pmat;    // 4x4 or null
  const double* window;       // H x W or null
};

// one image's field at pixel p, after polarizer, window and analyzer, in
// the bulk precision R (complex64 fields: FP32 arithmetic)
template <typename R>
__device__ __forceinline__ void pom_pixel(const PomArgs& a, const cpx<R>* __restrict__ f, int set, int lam,
                                          long long p, cpx<R> g[4]) {
  const long long HW = (long long)a.H * a.W;
  if (a.npol == 2) {
    const cpx<R>* fx = f + (((long long)set * 2 + 0) * a.nlam + lam) * 4 * HW + p;
    const cpx<R>* fy = f + (((long long)set * 2 + 1) * a.nlam + lam) * 4 * HW + p;
    const cpx<R> c = mk<R>((R)a.j0r, (R)a.j0i), s = mk<R>((R)a.j1r, (R)a.j1i);
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = fx[k * HW] * c + fy[k * HW] * s;
  } else {
    const cpx<R>* fi = f + ((long long)set * a.nlam + lam) * 4 * HW + p;
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = fi[k * HW];
  }
  if (a.window) {
    const R w = (R)a.window[p];
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = g[k] * w;
  }
  if (a.pmat) {
    cpx<R> o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      cpx<R> acc = mk<R>((R)0, (R)0);
#pragma unroll
      for (int j = 0; j < 4; ++j) acc = acc + cvt<R>(a.pmat[i * 4 + j]) * g[j];
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
  const long long HW = (long long)a.H * a.W;
  const int sl = blockIdx.y, set = sl / a.nlam, lam = sl - set * a.nlam;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < HW; p += (long long)gridDim.x * blockDim.x) {
    cpx<R> g[4];
    pom_pixel<R>(a, f, set, lam, p, g);
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
__device__ __forceinline__ double srgb_curve(double v) {
  if (v < 0.0031308) return v < 0.0 ? 0.0 : 12.92 * v;
  return v > 1.0 ? 1.0 : (1.0 + 0.055) * pow(v, 1.0 / 2.4) - 0.055;
}
__device__ __forceinline__ double power_curve(double v, double gamma) {
  if (v > 1.0) return 1.0;
  if (v < 0.0) return 0.0;
  return pow(v, 1.0 / gamma);
}
__device__ __forceinline__ void xyz_to_out(double xyz[3], double norm_div, int gray, double gamma, double rgb[3]) {
  if (norm_div != 0.0)
    for (int k = 0; k < 3; ++k) xyz[k] = xyz[k] / norm_div;
  if (gray) {
    rgb[0] = rgb[1] = rgb[2] = xyz[1];
  } else {
    for (int k = 0; k < 3; ++k) rgb[k] = kXYZ2RGB[k][0] * xyz[0] + kXYZ2RGB[k][1] * xyz[1] + kXYZ2RGB[k][2] * xyz[2];
  }
  if (gamma < 0.0) {
    for (int k = 0; k < 3; ++k) rgb[k] = srgb_curve(rgb[k]);
  } else if (gamma > 0.0) {
    for (int k = 0; k < 3; ++k) rgb[k] = power_curve(rgb[k], gamma);
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
      xyz_to_out(xyz, norm_div, gray, gamma, rgb);
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
// maximum is exact whatever the reduction order)
template <typename T>
__global__ void __launch_bounds__(1024) k_color_by_max(long long npix, int gray, double gamma, T* __restrict__ io) {
  __shared__ double red[1024];
  double m = -INFINITY;
  for (long long i = threadIdx.x; i < npix * 3; i += blockDim.x) m = fmax(m, (double)io[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const double mx = red[0];
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    double xyz[3] = {(double)io[p * 3], (double)io[p * 3 + 1], (double)io[p * 3 + 2]};
    double rgb[3];
    xyz_to_out(xyz, mx, gray, gamma, rgb);
    for (int k = 0; k < 3; ++k) io[p * 3 + k] = (T)rgb[k];
  }
}

// fused: polarizer / window / analyzer, Poynting summed over sets, XYZ, colour
template <typename R, typename T>
__global__ void k_pom_image(PomArgs a, const cpx<R>* __restrict__ f, const double* __restrict__ cmf,
                            double norm_div, int gray, double gamma, int convert, T* __restrict__ out) {
  const long long HW = (long long)a.H * a.W;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < HW; p += (long long)gridDim.x * blockDim.x) {
    double xyz[3] = {0.0, 0.0, 0.0};
    for (int lam = 0; lam < a.nlam; ++lam) {
      double s = 0.0;
      for (int set = 0; set < a.nset; ++set) {
        cpx<R> g[4];
        pom_pixel<R>(a, f, set, lam, p, g);
        s += (double)poynting<R>(g);
      }
      for (int k = 0; k < 3; ++k) xyz[k] = xyz[k] + cmf[lam * 3 + k] * s;
    }
    double rgb[3];
    if (convert) {
      xyz_to_out(xyz, norm_div, gray, gamma, rgb);
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
  k_color_by_max<double><<<1, 1024, 0, st>>>(npix, gray, gamma, rgb);
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
  k_color_by_max<float><<<1, 1024, 0, st>>>(hw, gray, gamma, rgb);
  return launched("k_color_by_max");
}

}  // extern "C"
