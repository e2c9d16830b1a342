// Host-side effective medium of an anisotropic optical block (plain C++, no
// CUDA): shared by the engine and its host test.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <utility>

// Eigenvalues and eigenvectors of a symmetric 3x3 tensor by Eberly's
// non-iterative solver (D. Eberly, "A Robust Eigensolver for 3x3 Symmetric
// Matrices", Geometric Tools), in complex arithmetic as the reference runs it
// (dtmm/linalg.py:29-318): the tensor scaled by its largest entry, the
// eigenvalues q + 2 p cos(acos(det(B) / 2 p^3) / 3 + {2 pi / 3, 0}) in
// increasing order (the argument clamped to [-1, 1] for a real tensor), the
// eigenvector of the outer eigenvalue from the largest cross product of two
// rows of A - lambda I, the middle one inside its orthogonal complement, the
// third as a cross product (a right-handed frame); a tensor whose scaled
// off-diagonal sum of squares is at most 1e-12 is taken as diagonal.  vec
// holds the eigenvectors as rows.
namespace effmed {
using C = std::complex<double>;

inline void cross(const C a[3], const C b[3], C out[3]) {
  const C o0 = a[1] * b[2] - a[2] * b[1];
  const C o1 = a[2] * b[0] - a[0] * b[2];
  const C o2 = a[0] * b[1] - a[1] * b[0];
  out[0] = o0;
  out[1] = o1;
  out[2] = o2;
}
inline double abs2(const C v[3]) {  // v . conj(v)
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s += v[i].real() * v[i].real() + v[i].imag() * v[i].imag();
  return s;
}
inline C dot(const C a[3], const C b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// eigenvector of eigenvalue e: the largest of the rows' pairwise cross products
inline void eigvec0(const C a[3][3], C e, C vec[3]) {
  C r0[3] = {a[0][0] - e, a[0][1], a[0][2]};
  C r1[3] = {a[0][1], a[1][1] - e, a[1][2]};
  C r2[3] = {a[0][2], a[1][2], a[2][2] - e};
  C x01[3], x02[3], x12[3];
  cross(r0, r1, x01);
  cross(r0, r2, x02);
  cross(r1, r2, x12);
  const double d0 = abs2(x01), d1 = abs2(x02), d2 = abs2(x12);
  double dmax = d0;
  int imax = 0;
  if (d1 > dmax) {
    dmax = d1;
    imax = 1;
  }
  if (d2 > dmax) imax = 2;
  const C* r = imax == 0 ? x01 : (imax == 1 ? x02 : x12);
  const C inv = 1.0 / std::sqrt(dot(r, r));
  for (int i = 0; i < 3; ++i) vec[i] = r[i] * inv;
}

// eigenvector of eigenvalue e orthogonal to the unit eigenvector w
inline void eigvec1(const C a[3][3], const C w[3], C e, C vec[3]) {
  C u[3], v[3];
  if (std::abs(w[0]) > std::abs(w[1])) {
    u[0] = -w[2];
    u[1] = 0.0;
    u[2] = w[0];
  } else {
    u[0] = 0.0;
    u[1] = w[2];
    u[2] = -w[1];
  }
  const double sc = 1.0 / std::sqrt(abs2(u));
  for (int i = 0; i < 3; ++i) u[i] *= sc;
  cross(w, u, v);
  C au[3], av[3];
  for (int i = 0; i < 3; ++i) {
    au[i] = a[i][0] * u[0] + a[i][1] * u[1] + a[i][2] * u[2];
    av[i] = a[i][0] * v[0] + a[i][1] * v[1] + a[i][2] * v[2];
  }
  C m00 = dot(u, au) - e, m01 = dot(u, av), m11 = dot(v, av) - e;
  const double a00 = std::abs(m00), a01 = std::abs(m01), a11 = std::abs(m11);
  for (int i = 0; i < 3; ++i) vec[i] = u[i];
  if (a00 >= a11) {
    if (std::max(a00, a01) > 0.0) {
      if (a00 >= a01) {
        m01 /= m00;
        m00 = 1.0 / std::sqrt(1.0 + m01 * m01);
        m01 *= m00;
      } else {
        m00 /= m01;
        m01 = 1.0 / std::sqrt(1.0 + m00 * m00);
        m00 *= m01;
      }
      for (int i = 0; i < 3; ++i) vec[i] = m01 * u[i] - m00 * v[i];
    }
  } else {
    if (std::max(a11, a01) > 0.0) {
      if (a11 >= a01) {
        m01 /= m11;
        m11 = 1.0 / std::sqrt(1.0 + m01 * m01);
        m01 *= m11;
      } else {
        m11 /= m01;
        m01 = 1.0 / std::sqrt(1.0 + m11 * m11);
        m11 *= m01;
      }
      for (int i = 0; i < 3; ++i) vec[i] = m11 * u[i] - m01 * v[i];
    }
  }
}

inline void tensor_eig(const C t[6], bool is_real, C eig[3], C vec[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) vec[i][j] = i == j ? 1.0 : 0.0;
  const double scale = std::max(std::max(std::max(std::abs(t[0]), std::abs(t[1])), std::max(std::abs(t[2]),
                                std::abs(t[3]))), std::max(std::abs(t[4]), std::abs(t[5])));
  if (scale == 0.0) {
    eig[0] = eig[1] = eig[2] = 0.0;
    return;
  }
  const double sm = 1.0 / scale;
  C a[3][3];
  a[0][0] = t[0] * sm; a[1][1] = t[1] * sm; a[2][2] = t[2] * sm;
  a[0][1] = a[1][0] = t[3] * sm;
  a[0][2] = a[2][0] = t[4] * sm;
  a[1][2] = a[2][1] = t[5] * sm;
  const C q = (a[0][0] + a[1][1] + a[2][2]) / 3.0;
  const C b00 = a[0][0] - q, b11 = a[1][1] - q, b22 = a[2][2] - q;
  const C norm = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
  if (std::abs(norm) > 1e-12) {
    const C p = std::sqrt((b00 * b00 + b11 * b11 + b22 * b22 + 2.0 * norm) / 6.0);
    const C c00 = b11 * b22 - a[1][2] * a[1][2];
    const C c01 = a[0][1] * b22 - a[1][2] * a[0][2];
    const C c02 = a[0][1] * a[1][2] - b11 * a[0][2];
    C half_det = (b00 * c00 - a[0][1] * c01 + a[0][2] * c02) / (p * p * p * 2.0);
    if (is_real) half_det = std::min(std::max(half_det.real(), -1.0), 1.0);
    const C phi = std::acos(half_det) / 3.0;
    const double two_thirds_pi = 2.09439510239319549;
    C e0 = std::cos(phi + two_thirds_pi) * 2.0;
    C e2 = std::cos(phi) * 2.0;
    C e1 = -(e0 + e2);
    e0 = e0 * p + q;
    e1 = e1 * p + q;
    e2 = e2 * p + q;
    if (half_det.real() >= 0.0) {
      eigvec0(a, e2, vec[2]);
      eigvec1(a, vec[2], e1, vec[1]);
      cross(vec[1], vec[2], vec[0]);
    } else {
      eigvec0(a, e0, vec[0]);
      eigvec1(a, vec[0], e1, vec[1]);
      cross(vec[0], vec[1], vec[2]);
    }
    eig[0] = e0 * scale;
    eig[1] = e1 * scale;
    eig[2] = e2 * scale;
  } else {
    eig[0] = a[0][0] * scale;
    eig[1] = a[1][1] * scale;
    eig[2] = a[2][2] * scale;
  }
}
}  // namespace effmed

// Effective medium of uniaxial (sym 1) or biaxial (sym 2) symmetry from a
// block's mean lab-frame tensor t (00, 11, 22, 01, 02, 12 as re, im pairs;
// is_real: the reference's tensor has a real dtype) (effective_block,
// dtmm/data.py:1364-1419): the eigen-frame above; the cyclic permutation
// that moves the most distinct eigenvalue to the third place
// (dtmm/linalg.py:166-218); the Euler angles of the frame's real part
// (dtmm/rotation.py:154-171); for sym 1 the first two eigenvalues replaced by
// m - delta / 3 and the third by m + 2 delta / 3, m the mean eigenvalue and
// delta the third minus the mean of the first two (dtmm/data.py:1215-1233).
// out: sym, epsv (re, im) x 3, psi, theta, phi.
inline void eff_medium(const double* t, int sym, bool is_real, double* out) {
  using effmed::C;
  const C e[6] = {C(t[0], t[1]), C(t[2], t[3]), C(t[4], t[5]), C(t[6], t[7]), C(t[8], t[9]), C(t[10], t[11])};
  C w[3], vec[3][3];
  effmed::tensor_eig(e, is_real, w, vec);
  const double m2 = std::abs(w[1] - w[0]), m1 = std::abs(w[2] - w[0]), m0 = std::abs(w[2] - w[1]);
  int idx[3] = {0, 1, 2};
  if (m2 > m1 || m2 > m0) {
    if (m1 > m0) {
      idx[0] = 1; idx[1] = 2; idx[2] = 0;
    } else {
      idx[0] = 2; idx[1] = 0; idx[2] = 1;
    }
  }
  C ev[3];
  double R[3][3];  // columns: the sorted eigenvectors
  for (int k = 0; k < 3; ++k) {
    ev[k] = w[idx[k]];
    for (int i = 0; i < 3; ++i) R[i][k] = vec[idx[k]][i].real();
  }
  const double theta = std::acos(std::max(-1.0, std::min(1.0, R[2][2])));
  double psi, phi;
  if ((R[1][2] == 0.0 && R[0][2] == 0.0) || theta == 0.0) {
    psi = 0.0;
    phi = std::acos(std::max(-1.0, std::min(1.0, R[1][1])));
  } else {
    phi = std::atan2(R[1][2], R[0][2]);
    psi = std::atan2(R[2][1], -R[2][0]);
  }
  if (sym == 1) {
    const C m = (ev[0] + ev[1] + ev[2]) / 3.0;
    const C delta = ev[2] - (ev[0] + ev[1]) / 2.0;
    ev[0] = ev[1] = m - delta / 3.0;
    ev[2] = m + 2.0 * delta / 3.0;
  }
  out[0] = (double)sym;
  for (int k = 0; k < 3; ++k) {
    out[1 + 2 * k] = ev[k].real();
    out[2 + 2 * k] = ev[k].imag();
  }
  out[7] = psi;
  out[8] = theta;
  out[9] = phi;
}
