// Optical data from a director field on the device (director2data,
// dtmm/data.py:277-320): per voxel the order parameter is the square root of
// the director's length (director2order, dtmm/data.py:963-973), the
// eigenvalues are the uniaxial order of (no^2, no^2, ne^2) scaled by it
// (_uniaxial_order, dtmm/data.py:1214-1233), host voxels outside the mask get
// nhost^2, and the Euler angles are (0, atan2(|d_xy|, d_z), atan2(d_y, d_x))
// (director2angles, dtmm/data.py:975-990).
#include <cuda_runtime.h>

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
