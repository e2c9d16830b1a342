// Optical data from a Q-tensor field on the device (Q2data,
// dtmm/data.py:322-371).  Per voxel:
//
//   eps = epsa_s * Q + epsm * I                      (Q2eps, dtmm/data.py:432-487)
//   eigenvalues / eigenvectors of eps by the non-iterative eigensolver of
//   D. Eberly, "A Robust Eigensolver for 3x3 Symmetric Matrices" (Geometric
//   Tools), as the reference applies it (dtmm/linalg.py:44-300): scale by the
//   largest element, roots of the characteristic cubic from acos of the
//   half determinant, the eigenvector of the best-separated root from the
//   longest cross product of two rows of A - e I, the second by a 2x2
//   minimisation in the plane orthogonal to it, the third by a cross product;
//   then a cyclic permutation that puts the most distinct eigenvalue last
//   (dtmm/linalg.py:171-218)
//   Euler angles of the eigenvector matrix (columns = eigenvectors)
//                                                    (dtmm/rotation.py:154-174)
//   uniaxial order 1 of the eigenvalues unless biaxial (dtmm/data.py:1215-1233)
//   nhost^2 on the diagonal outside the mask.
//
// The file is compiled without FMA contraction, so that every sum and
// product rounds as the reference's double arithmetic does: for a tensor
// with two equal eigenvalues the eigenvector pair of that eigenvalue is
// chosen by rounding, and contraction would change it where the reference
// does not.  Operand order follows the reference expression by expression.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "../../include/dtmm_gb300.h"

namespace dtmm {
std::string& last_error_slot();  // the text dtmm_last_error returns (dtmm_capi.cu)
}

namespace {

__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
  const double c0 = a[1] * b[2] - a[2] * b[1];
  const double c1 = a[2] * b[0] - a[0] * b[2];
  const double c2 = a[0] * b[1] - a[1] * b[0];
  c[0] = c0;
  c[1] = c1;
  c[2] = c2;
}

__device__ __forceinline__ double sq3(const double* v) {
  double s = 0.0;
  s = s + v[0] * v[0];
  s = s + v[1] * v[1];
  s = s + v[2] * v[2];
  return s;
}

// eigenvector of the root `ev`: the longest of the three row cross products
// of A - ev I, normalised
__device__ void eigvec_first(double a00, double a11, double a22, double a01, double a02, double a12, double ev,
                             double* out) {
  const double r0[3] = {a00 - ev, a01, a02};
  const double r1[3] = {a01, a11 - ev, a12};
  const double r2[3] = {a02, a12, a22 - ev};
  double c01[3], c12[3], c02[3];
  cross3(r0, r1, c01);
  cross3(r1, r2, c12);
  cross3(r0, r2, c02);
  const double d0 = sq3(c01), d1 = sq3(c02), d2 = sq3(c12);
  const double* best = c01;
  double dmax = d0;
  if (d1 > dmax) {
    dmax = d1;
    best = c02;
  }
  if (d2 > dmax) best = c12;
  const double norm = 1.0 / sqrt(best[0] * best[0] + best[1] * best[1] + best[2] * best[2]);
  out[0] = best[0] * norm;
  out[1] = best[1] * norm;
  out[2] = best[2] * norm;
}

// eigenvector of `ev` orthogonal to the unit vector w
__device__ void eigvec_second(double a00, double a11, double a22, double a01, double a02, double a12, const double* w,
                              double ev, double* out) {
  double u[3];
  if (fabs(w[0]) > fabs(w[1])) {
    u[0] = -w[2];
    u[1] = 0.0;
    u[2] = w[0];
  } else {
    u[0] = 0.0;
    u[1] = w[2];
    u[2] = -w[1];
  }
  const double sc = 1.0 / sqrt(sq3(u));
  u[0] *= sc;
  u[1] *= sc;
  u[2] *= sc;
  double v[3];
  cross3(w, u, v);
  const double au0 = a00 * u[0] + a01 * u[1] + a02 * u[2];
  const double au1 = a01 * u[0] + a11 * u[1] + a12 * u[2];
  const double au2 = a02 * u[0] + a12 * u[1] + a22 * u[2];
  double m00 = u[0] * au0 + u[1] * au1 + u[2] * au2 - ev;
  const double av0 = a00 * v[0] + a01 * v[1] + a02 * v[2];
  const double av1 = a01 * v[0] + a11 * v[1] + a12 * v[2];
  const double av2 = a02 * v[0] + a12 * v[1] + a22 * v[2];
  double m01 = u[0] * av0 + u[1] * av1 + u[2] * av2;
  double m11 = v[0] * av0 + v[1] * av1 + v[2] * av2 - ev;
  const double am00 = fabs(m00), am01 = fabs(m01), am11 = fabs(m11);
  double cu = 1.0, cv = 0.0;  // out = cu u - cv v (u itself when the 2x2 block is zero)
  if (am00 >= am11) {
    if (fmax(am00, am01) > 0.0) {
      if (am00 >= am01) {
        m01 /= m00;
        m00 = 1.0 / sqrt(1.0 + m01 * m01);
        m01 *= m00;
      } else {
        m00 /= m01;
        m01 = 1.0 / sqrt(1.0 + m00 * m00);
        m00 *= m01;
      }
      cu = m01;
      cv = m00;
    }
  } else if (fmax(am11, am01) > 0.0) {
    if (am11 >= am01) {
      m01 /= m11;
      m11 = 1.0 / sqrt(1.0 + m01 * m01);
      m01 *= m11;
    } else {
      m11 /= m01;
      m01 = 1.0 / sqrt(1.0 + m11 * m11);
      m11 *= m01;
    }
    cu = m11;
    cv = m01;
  }
  for (int i = 0; i < 3; ++i) out[i] = cu * u[i] - cv * v[i];
}

// eigenvalues e[3] and eigenvectors (rows of vec) of one symmetric tensor,
// sorted so that e[2] is the most distinct
__device__ void tensor_eig(const double* t, double* e, double (*vec)[3]) {
  const double t00 = t[0], t11 = t[1], t22 = t[2], t01 = t[3], t02 = t[4], t12 = t[5];
  const double scale = fmax(fmax(fmax(fabs(t00), fabs(t11)), fmax(fabs(t22), fabs(t01))), fmax(fabs(t02), fabs(t12)));
  double ev[3], vv[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  if (scale == 0.0) {
    ev[0] = ev[1] = ev[2] = 0.0;
  } else {
    const double s = 1.0 / scale;
    const double a00 = t00 * s, a11 = t11 * s, a22 = t22 * s, a01 = t01 * s, a02 = t02 * s, a12 = t12 * s;
    const double q = (a00 + a11 + a22) / 3.0;
    const double b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const double norm = a01 * a01 + a02 * a02 + a12 * a12;
    if (fabs(norm) > 1e-12) {
      const double p = sqrt((b00 * b00 + b11 * b11 + b22 * b22 + 2.0 * norm) / 6.0);
      const double c00 = b11 * b22 - a12 * a12;
      const double c01 = a01 * b22 - a12 * a02;
      const double c02 = a01 * a12 - b11 * a02;
      double half_det = (b00 * c00 - a01 * c01 + a02 * c02) / (p * p * p * 2.0);
      half_det = fmin(fmax(half_det, -1.0), 1.0);
      const double phi = acos(half_det) / 3.0;
      double e0 = cos(phi + 2.09439510239319549) * 2.0;  // 2 pi / 3 rounded to double
      double e2 = cos(phi) * 2.0;
      double e1 = -(e0 + e2);
      e0 = e0 * p + q;
      e1 = e1 * p + q;
      e2 = e2 * p + q;
      if (half_det >= 0.0) {
        eigvec_first(a00, a11, a22, a01, a02, a12, e2, vv[2]);
        eigvec_second(a00, a11, a22, a01, a02, a12, vv[2], e1, vv[1]);
        cross3(vv[1], vv[2], vv[0]);
      } else {
        eigvec_first(a00, a11, a22, a01, a02, a12, e0, vv[0]);
        eigvec_second(a00, a11, a22, a01, a02, a12, vv[0], e1, vv[1]);
        cross3(vv[0], vv[1], vv[2]);
      }
      ev[0] = e0 * scale;
      ev[1] = e1 * scale;
      ev[2] = e2 * scale;
    } else {
      ev[0] = a00 * scale;
      ev[1] = a11 * scale;
      ev[2] = a22 * scale;
    }
  }
  const double m2 = fabs(ev[1] - ev[0]), m1 = fabs(ev[2] - ev[0]), m0 = fabs(ev[2] - ev[1]);
  int i = 0, j = 1, k = 2;
  if (m2 > m1 || m2 > m0) {
    if (m1 > m0) {
      i = 1, j = 2, k = 0;
    } else {
      i = 2, j = 0, k = 1;
    }
  }
  const int perm[3] = {i, j, k};
  for (int a = 0; a < 3; ++a) {
    e[a] = ev[perm[a]];
    for (int b = 0; b < 3; ++b) vec[a][b] = vv[perm[a]][b];
  }
}

// Q tensors [n, 6] (Q00, Q11, Q22, Q01, Q02, Q12) -> epsv [n, 3], epsa [n, 3]
__global__ void k_q2data(long long n, const double* __restrict__ qt, const unsigned char* __restrict__ mask,
                         double epsa_s, double epsm, double eh, int biaxial, double* __restrict__ epsv,
                         double* __restrict__ epsa) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double t[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) t[c] = epsa_s * qt[6 * i + c] + epsm;
#pragma unroll
    for (int c = 3; c < 6; ++c) t[c] = epsa_s * qt[6 * i + c];
    double e[3], vec[3][3];
    tensor_eig(t, e, vec);
    // rotation matrix R: eigenvectors in its columns, R[r][c] = vec[c][r]
    const double r22 = fmax(-1.0, fmin(1.0, vec[2][2]));
    const double theta = acos(r22);
    double psi, phi;
    if ((vec[2][1] == 0.0 && vec[2][0] == 0.0) || theta == 0.0) {
      psi = 0.0;
      phi = acos(fmax(-1.0, fmin(1.0, vec[1][1])));
    } else {
      phi = atan2(vec[2][1], vec[2][0]);
      psi = atan2(vec[1][2], -vec[0][2]);
    }
    epsa[3 * i] = psi;
    epsa[3 * i + 1] = theta;
    epsa[3 * i + 2] = phi;
    if (mask != nullptr && !mask[i]) {
      e[0] = e[1] = e[2] = eh;
    } else if (!biaxial) {
      const double m = (e[0] + e[1] + e[2]) / 3.0;
      const double delta = e[2] - (e[0] + e[1]) / 2.0;
      const double e1 = m - 1.0 / 3.0 * 1.0 * delta;
      const double e3 = m + 2.0 / 3.0 * 1.0 * delta;
      e[0] = e[1] = e1;
      e[2] = e3;
    }
    epsv[3 * i] = e[0];
    epsv[3 * i + 1] = e[1];
    epsv[3 * i + 2] = e[2];
  }
}

}  // namespace

extern "C" int dtmm_q2data(long long nvox, const double* qtensor, const void* mask, double no, double ne, double nhost,
                           double scale_factor, int biaxial, double* epsv, double* epsa, void* stream) {
  dtmm::last_error_slot().clear();
  if (nvox < 1) {
    dtmm::last_error_slot() = "empty Q tensor field";
    return DTMM_EINVAL;
  }
  if (!qtensor || !epsv || !epsa) {
    dtmm::last_error_slot() = "null pointer";
    return DTMM_EINVAL;
  }
  if (!(scale_factor != 0.0)) {
    dtmm::last_error_slot() = "scale_factor must be non-zero";
    return DTMM_EINVAL;
  }
  // the scalars of Q2eps in the reference's operand order
  const double epse = ne * ne, epso = no * no;
  const double epsa_s = (epse - epso) / scale_factor;
  const double epsm = (epso * 2.0 + epse) / 3.0;
  const unsigned blocks = (unsigned)std::min<long long>((nvox + 127) / 128, 152LL * 16);
  k_q2data<<<blocks, 128, 0, (cudaStream_t)stream>>>(nvox, qtensor, (const unsigned char*)mask, epsa_s, epsm,
                                                     nhost * nhost, biaxial ? 1 : 0, epsv, epsa);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    dtmm::last_error_slot() = std::string("k_q2data: ") + cudaGetErrorString(e);
    return DTMM_ECUDA;
  }
  return DTMM_OK;
}
