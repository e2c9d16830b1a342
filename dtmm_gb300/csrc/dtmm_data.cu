// Optical data from a director field on the device (director2data,
// dtmm/data.py:277-320): per voxel the order parameter is the square root of
// the director's length (director2order, dtmm/data.py:963-973), the
// eigenvalues are the uniaxial order of (no^2, no^2, ne^2) scaled by it
// (_uniaxial_order, dtmm/data.py:1214-1233), host voxels outside the mask get
// nhost^2, and the Euler angles are (0, atan2(|d_xy|, d_z), atan2(d_y, d_x))
// (director2angles, dtmm/data.py:975-990).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "../../include/dtmm_gb300.h"

namespace dtmm {
std::string& last_error_slot();  // the text dtmm_last_error returns (dtmm_capi.cu)
}

namespace {

template <typename D>
__global__ void k_director2data(long long n, const D* __restrict__ dir, const unsigned char* __restrict__ mask,
                                double eo, double ee, double eh, double scale, double* __restrict__ epsv,
                                double* __restrict__ epsa) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x = (double)dir[3 * i], y = (double)dir[3 * i + 1], z = (double)dir[3 * i + 2];
    const double xy = sqrt(x * x + y * y);
    epsa[3 * i] = 0.0;
    epsa[3 * i + 1] = atan2(xy, z);
    epsa[3 * i + 2] = atan2(y, x);
    double e1, e3;
    if (mask != nullptr && !mask[i]) {
      e1 = e3 = eh;
    } else {
      const double order = sqrt(sqrt(x * x + y * y + z * z)) / scale;
      const double m = (eo + eo + ee) / 3.0;
      const double delta = ee - (eo + eo) / 2.0;
      if (order == 0.0) {
        e1 = e3 = m;
      } else {
        e1 = m - 1.0 / 3.0 * order * delta;
        e3 = m + 2.0 / 3.0 * order * delta;
      }
    }
    epsv[3 * i] = e1;
    epsv[3 * i + 1] = e1;
    epsv[3 * i + 2] = e3;
  }
}

}  // namespace

extern "C" int dtmm_director2data(long long nvox, const void* director, int director_double, const void* mask,
                                  double no, double ne, double nhost, double scale_factor, double* epsv,
                                  double* epsa, void* stream) {
  dtmm::last_error_slot().clear();
  if (nvox < 1) {
    dtmm::last_error_slot() = "empty director";
    return DTMM_EINVAL;
  }
  if (!director || !epsv || !epsa) {
    dtmm::last_error_slot() = "null pointer";
    return DTMM_EINVAL;
  }
  if (!(scale_factor != 0.0)) {
    dtmm::last_error_slot() = "scale_factor must be non-zero";
    return DTMM_EINVAL;
  }
  const unsigned blocks = (unsigned)std::min<long long>((nvox + 255) / 256, 4864);
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned char* m = (const unsigned char*)mask;
  if (director_double)
    k_director2data<double><<<blocks, 256, 0, st>>>(nvox, (const double*)director, m, no * no, ne * ne, nhost * nhost,
                                                     scale_factor, epsv, epsa);
  else
    k_director2data<float><<<blocks, 256, 0, st>>>(nvox, (const float*)director, m, no * no, ne * ne, nhost * nhost,
                                                    scale_factor, epsv, epsa);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    dtmm::last_error_slot() = std::string("k_director2data: ") + cudaGetErrorString(e);
    return DTMM_ECUDA;
  }
  return DTMM_OK;
}

// ---------------------------------------------------------------------------
// Synthetic twisted-nematic Euler angles (the benchmark's seeded director
// fields, dtmm_gb300.samples.twisted_nematic): per pixel two smooth
// perturbations d_phi, d_tilt (sums of cosine modes cos(ax x + ay y + c),
// scaled), then for every layer l
//   epsa[l][y][x] = (0, pi/2 - (d_tilt + tilt), l * twist / L + d_phi).
// The modes arrive by value, so building a request needs no upload.
// ---------------------------------------------------------------------------
namespace {

constexpr int kMaxModes = 16;
struct ModeSet {
  int n;
  double ax[kMaxModes], ay[kMaxModes], c[kMaxModes];
  double scale;
};

__device__ double mode_sum(const ModeSet& m, double x, double y) {
  double s = 0.0;
  for (int i = 0; i < m.n; ++i) s += cos(m.ax[i] * x + m.ay[i] * y + m.c[i]);
  return s * m.scale;
}

__global__ void k_twisted_angles(int L, int H, int W, ModeSet mphi, ModeSet mtilt, double twist, double tilt,
                                 double* __restrict__ epsa) {
  const long long HW = (long long)H * W;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < HW; p += (long long)gridDim.x * blockDim.x) {
    const double y = (double)(p / W), x = (double)(p % W);
    const double dphi = mode_sum(mphi, x, y);
    const double th = M_PI / 2 - (mode_sum(mtilt, x, y) + tilt);
    for (int l = 0; l < L; ++l) {
      double* e = epsa + ((long long)l * HW + p) * 3;
      e[0] = 0.0;
      e[1] = th;
      e[2] = (double)l * twist / L + dphi;
    }
  }
}

}  // namespace

extern "C" int dtmm_twisted_nematic_angles(int nlayers, int height, int width, const double* modes, int nmodes,
                                           double amp_phi, double amp_tilt, double twist, double tilt, double* epsa,
                                           void* stream) {
  dtmm::last_error_slot().clear();
  if (nlayers < 1 || height < 1 || width < 1) {
    dtmm::last_error_slot() = "empty grid";
    return DTMM_EINVAL;
  }
  if (!modes || !epsa) {
    dtmm::last_error_slot() = "null pointer";
    return DTMM_EINVAL;
  }
  if (nmodes < 1 || nmodes > kMaxModes) {
    dtmm::last_error_slot() = "nmodes must be 1..16";
    return DTMM_EINVAL;
  }
  ModeSet mp, mt;
  mp.n = mt.n = nmodes;
  mp.scale = amp_phi;
  mt.scale = amp_tilt;
  for (int i = 0; i < nmodes; ++i) {
    mp.ax[i] = modes[3 * i];
    mp.ay[i] = modes[3 * i + 1];
    mp.c[i] = modes[3 * i + 2];
    mt.ax[i] = modes[3 * (nmodes + i)];
    mt.ay[i] = modes[3 * (nmodes + i) + 1];
    mt.c[i] = modes[3 * (nmodes + i) + 2];
  }
  const long long hw = (long long)height * width;
  const unsigned blocks = (unsigned)std::min<long long>((hw + 255) / 256, 152LL * 8);
  k_twisted_angles<<<blocks, 256, 0, (cudaStream_t)stream>>>(nlayers, height, width, mp, mt, twist, tilt, epsa);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    dtmm::last_error_slot() = std::string("k_twisted_angles: ") + cudaGetErrorString(e);
    return DTMM_ECUDA;
  }
  return DTMM_OK;
}
