// Biaxial eigen-solve of one voxel in FP64 (dtmm/tmm.py:395-401): the
// rotated dielectric tensor, the Berreman matrix, its eigen-decomposition and
// the Poynting sort of the modes.
//
// The reference hands the Berreman matrix to LAPACK (numpy.linalg.eig).
// Here a 4 x 4 complex matrix is decomposed with the textbook dense method
// (Golub & Van Loan, Matrix Computations, 4th ed., 7.4-7.6): Householder
// reduction to upper Hessenberg form, single-shift complex QR sweeps with
// Wilkinson shifts and deflation of negligible subdiagonal entries, then the
// eigenvectors of the triangular Schur factor by back-substitution, mapped
// through the accumulated unitary transform.  Eigenvalues and eigenvectors
// agree with LAPACK's up to the order of the modes and the scale of each
// eigenvector; the transfer only uses F diag(P) F^-1 and the Poynting sign of
// each column, which depend on neither.
//
// Everything here is __host__ __device__, so the host test
// (tests/eig4_host.cu) runs the same code against numpy.
#pragma once

#include <cmath>

#include "dtmm_common.cuh"

namespace dtmm {
namespace e4 {

using C = cpx<double>;

__host__ __device__ inline double cabs1(C a) { return fabs(a.re) + fabs(a.im); }
__host__ __device__ inline double cabs(C a) { return hypot(a.re, a.im); }

// Smith's division; b == 0 gives inf / nan as IEEE division would
__host__ __device__ inline C cdivs(C a, C b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, den = b.re + b.im * r;
    return mk<double>((a.re + a.im * r) / den, (a.im - a.re * r) / den);
  }
  const double r = b.re / b.im, den = b.re * r + b.im;
  return mk<double>((a.re * r + a.im) / den, (a.im * r - a.re) / den);
}

// principal square root
__host__ __device__ inline C csqrts(C z) {
  if (z.re == 0.0 && z.im == 0.0) return mk<double>(0.0, z.im);
  const double m = hypot(z.re, z.im);
  const double t = sqrt(0.5 * (m + fabs(z.re)));
  if (z.re >= 0.0) return mk<double>(t, z.im / (2.0 * t));
  return mk<double>(fabs(z.im) / (2.0 * t), copysign(t, z.im));
}

// Similarity by the plane rotation of rows / columns k, k+1 that maps
// (x, y) to (r, 0): G = [[c, s], [-conj(s), c]], c real, applied as
// H <- G H G^H and Q <- Q G^H (every row and column of the 4 x 4 matrices;
// entries outside the active block are zeros and stay zeros).
__host__ __device__ inline void rotate(C H[4][4], C Q[4][4], int k, C x, C y) {
  const double ax = cabs(x), ay = cabs(y);
  if (ay == 0.0) return;
  double c;
  C s;
  if (ax == 0.0) {
    c = 0.0;
    s = mk<double>(y.re / ay, -y.im / ay);  // conj(y) / |y|
  } else {
    const double nrm = hypot(ax, ay);
    c = ax / nrm;
    const C ux = mk<double>(x.re / ax, x.im / ax);
    s = ux * conj(y) * (1.0 / nrm);
  }
  const C sc = conj(s);
  for (int j = 0; j < 4; ++j) {  // rows k, k+1
    const C a = H[k][j], b = H[k + 1][j];
    H[k][j] = a * c + s * b;
    H[k + 1][j] = b * c - sc * a;
  }
  for (int i = 0; i < 4; ++i) {  // columns k, k+1 (times G^H)
    const C a = H[i][k], b = H[i][k + 1];
    H[i][k] = a * c + b * sc;
    H[i][k + 1] = b * c - a * s;
    const C qa = Q[i][k], qb = Q[i][k + 1];
    Q[i][k] = qa * c + qb * sc;
    Q[i][k + 1] = qb * c - qa * s;
  }
}

// Eigenvalues lam and eigenvectors (columns of V) of A.  False when the QR
// iteration did not converge within its limit (lam and V are then undefined).
__host__ __device__ inline bool eig4(const C A[4][4], C lam[4], C V[4][4]) {
  C H[4][4], Q[4][4];
  double anorm = 0.0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      H[i][j] = A[i][j];
      Q[i][j] = mk<double>(i == j ? 1.0 : 0.0, 0.0);
      anorm = fmax(anorm, cabs1(A[i][j]));
    }
  if (anorm == 0.0) {
    for (int i = 0; i < 4; ++i) {
      lam[i] = mk<double>(0.0, 0.0);
      for (int j = 0; j < 4; ++j) V[i][j] = Q[i][j];
    }
    return true;
  }
  // Householder reduction to Hessenberg form: columns 0 and 1
  for (int k = 0; k < 2; ++k) {
    const int n = 3 - k;  // entries k+1 .. 3
    C v[3];
    double xn = 0.0;
    for (int i = 0; i < n; ++i) {
      v[i] = H[k + 1 + i][k];
      xn += norm2(v[i]);
    }
    xn = sqrt(xn);
    const double tail = xn * xn - norm2(v[0]);
    if (xn == 0.0 || tail <= 0.0) continue;  // already reduced
    const double a0 = cabs(v[0]);
    const C ph = a0 > 0.0 ? mk<double>(v[0].re / a0, v[0].im / a0) : mk<double>(1.0, 0.0);
    v[0] = v[0] + ph * xn;  // v = x + e^{i arg x0} |x| e1 (no cancellation)
    double vn = 0.0;
    for (int i = 0; i < n; ++i) vn += norm2(v[i]);
    if (vn == 0.0) continue;
    const double tau = 2.0 / vn;  // P = I - tau v v^H
    for (int j = 0; j < 4; ++j) {  // H <- P H (rows k+1..3)
      C s = mk<double>(0.0, 0.0);
      for (int i = 0; i < n; ++i) s = s + conj(v[i]) * H[k + 1 + i][j];
      s = s * tau;
      for (int i = 0; i < n; ++i) H[k + 1 + i][j] = H[k + 1 + i][j] - v[i] * s;
    }
    for (int i = 0; i < 4; ++i) {  // H <- H P, Q <- Q P (columns k+1..3)
      C s = mk<double>(0.0, 0.0), t = mk<double>(0.0, 0.0);
      for (int j = 0; j < n; ++j) {
        s = s + H[i][k + 1 + j] * v[j];
        t = t + Q[i][k + 1 + j] * v[j];
      }
      s = s * tau;
      t = t * tau;
      for (int j = 0; j < n; ++j) {
        H[i][k + 1 + j] = H[i][k + 1 + j] - s * conj(v[j]);
        Q[i][k + 1 + j] = Q[i][k + 1 + j] - t * conj(v[j]);
      }
    }
    for (int i = k + 2; i < 4; ++i) H[i][k] = mk<double>(0.0, 0.0);
  }
  // shifted QR sweeps on the active block [lo, hi]
  const double ulp = 2.220446049250313e-16;
  int hi = 3, its = 0, total = 0;
  while (hi > 0) {
    int lo = hi;
    while (lo > 0) {
      const double d = cabs1(H[lo - 1][lo - 1]) + cabs1(H[lo][lo]);
      if (cabs1(H[lo][lo - 1]) <= ulp * (d > 0.0 ? d : anorm)) {
        H[lo][lo - 1] = mk<double>(0.0, 0.0);
        break;
      }
      --lo;
    }
    if (lo == hi) {  // H[hi][hi] has converged
      --hi;
      its = 0;
      continue;
    }
    if (++total > 120) return false;
    ++its;
    C mu;
    if (its % 10 == 0) {  // exceptional shift against cycling
      mu = H[hi][hi] + mk<double>(0.75 * cabs1(H[hi][hi - 1]), 0.0);
    } else {  // Wilkinson: the eigenvalue of the trailing 2 x 2 closer to H[hi][hi]
      const C a = H[hi - 1][hi - 1], b = H[hi - 1][hi], c = H[hi][hi - 1], d = H[hi][hi];
      const C h = (a - d) * 0.5;
      const C disc = csqrts(h * h + b * c);
      const C m1 = d + h + disc, m2 = d + h - disc;  // (a + d) / 2 +- disc
      mu = cabs1(m1 - d) <= cabs1(m2 - d) ? m1 : m2;
    }
    C x = H[lo][lo] - mu, y = H[lo + 1][lo];
    for (int k = lo; k < hi; ++k) {
      rotate(H, Q, k, x, y);
      if (k > lo) H[k + 1][k - 1] = mk<double>(0.0, 0.0);  // the chased bulge
      if (k + 1 < hi) {
        x = H[k + 1][k];
        y = H[k + 2][k];
      }
    }
  }
  for (int i = 0; i < 4; ++i) lam[i] = H[i][i];
  // eigenvectors of the triangular factor: (T - lam_k) y = 0, y_k = 1
  const double small = ulp * anorm;
  for (int k = 0; k < 4; ++k) {
    C yv[4];
    for (int j = 0; j < 4; ++j) yv[j] = mk<double>(j == k ? 1.0 : 0.0, 0.0);
    for (int j = k - 1; j >= 0; --j) {
      C s = mk<double>(0.0, 0.0);
      for (int l = j + 1; l <= k; ++l) s = s + H[j][l] * yv[l];
      C den = H[j][j] - lam[k];
      if (cabs1(den) < small) den = mk<double>(small, 0.0);
      yv[j] = -cdivs(s, den);
    }
    for (int i = 0; i < 4; ++i) {
      C s = mk<double>(0.0, 0.0);
      for (int j = 0; j <= k; ++j) s = s + Q[i][j] * yv[j];
      V[i][k] = s;
    }
  }
  return true;
}

// z-Poynting of a field vector (Ex, Hy, Ey, Hx) (dtmm/tmm.py:293-298)
__host__ __device__ inline double poynting(C f0, C f1, C f2, C f3) {
  return (f0.re * f1.re + f0.im * f1.im) - (f2.re * f3.re + f2.im * f3.im);
}

}  // namespace e4

// Eigenvalues al and field matrix F (rows Ex, Hy, Ey, Hx; columns the modes)
// of a biaxial voxel in the plane of incidence (the frame rotated by the beam
// azimuth phi; the caller rotates F back, dtmm/linalg.py:674):
//   R = R(psi, theta, azimuth - phi)            (dtmm/rotation.py:125-150, :398)
//   eps = R diag(ev) R^T, 6 components          (dtmm/rotation.py:285-293)
//   Berreman matrix of (beta, eps)              (dtmm/tmm.py:100-121)
//   eigen-decomposition, then the modes with Poynting >= 0 into columns 0, 2
//   and the others into 1, 3 in the order found (dtmm/tmm.py:300-370); a
//   split other than two and two, or a failed decomposition, gives NaN
//   eigenvalues and a zero F, as the reference's failed sort does.
// cps/sps, ct/st, cf/sf: cos / sin of psi, theta and azimuth - phi.
__host__ __device__ inline void biaxial_fmat(double beta, const cpx<double> ev[3], double cps, double sps, double ct,
                                             double st, double cf, double sf, cpx<double> F[4][4],
                                             cpx<double> al[4]) {
  using e4::C;
  double R[3][3];
  const double sfsp = sf * sps, sfcp = sf * cps, cfsp = cf * sps, cfcp = cf * cps;
  R[0][0] = ct * cfcp - sfsp;
  R[0][1] = -ct * cfsp - sfcp;
  R[0][2] = cf * st;
  R[1][0] = ct * sfcp + cfsp;
  R[1][1] = cfcp - ct * sfsp;
  R[1][2] = st * sf;
  R[2][0] = -cps * st;
  R[2][1] = st * sps;
  R[2][2] = ct;
  C eps[6];
  for (int i = 0; i < 3; ++i) eps[i] = ev[0] * (R[i][0] * R[i][0]) + ev[1] * (R[i][1] * R[i][1]) + ev[2] * (R[i][2] * R[i][2]);
  eps[3] = ev[0] * (R[0][0] * R[1][0]) + ev[1] * (R[0][1] * R[1][1]) + ev[2] * (R[0][2] * R[1][2]);
  eps[4] = ev[0] * (R[0][0] * R[2][0]) + ev[1] * (R[0][1] * R[2][1]) + ev[2] * (R[0][2] * R[2][2]);
  eps[5] = ev[0] * (R[1][0] * R[2][0]) + ev[1] * (R[1][1] * R[2][1]) + ev[2] * (R[1][2] * R[2][2]);
  const C one = mk<double>(1.0, 0.0), z = mk<double>(0.0, 0.0);
  const C e2m = e4::cdivs(one, eps[2]);
  const C e4e2 = eps[4] * e2m, e5e2 = eps[5] * e2m;
  C L[4][4];
  L[0][0] = -(e4e2 * beta);
  L[0][1] = one - e2m * (beta * beta);
  L[0][2] = -(e5e2 * beta);
  L[0][3] = z;
  L[1][0] = eps[0] - eps[4] * e4e2;
  L[1][1] = L[0][0];
  L[1][2] = eps[3] - eps[5] * e4e2;
  L[1][3] = z;
  L[2][0] = z;
  L[2][1] = z;
  L[2][2] = z;
  L[2][3] = -one;
  L[3][0] = -L[1][2];
  L[3][1] = -L[0][2];
  L[3][2] = mk<double>(beta * beta, 0.0) + eps[5] * e5e2 - eps[1];
  L[3][3] = z;
  C lam[4], V[4][4];
  bool ok = e4::eig4(L, lam, V);
  int i = 0, j = 1;
  if (ok) {
    for (int k = 0; k < 4; ++k) {
      const bool fwd = e4::poynting(V[0][k], V[1][k], V[2][k], V[3][k]) >= 0.0;
      int& slot = fwd ? i : j;
      if (slot >= 4) {
        ok = false;
        break;
      }
      al[slot] = lam[k];
      for (int r = 0; r < 4; ++r) F[r][slot] = V[r][k];
      slot += 2;
    }
  }
  if (!ok) {
    const double nan_ = NAN;
    for (int k = 0; k < 4; ++k) {
      al[k] = mk<double>(nan_, nan_);
      for (int r = 0; r < 4; ++r) F[r][k] = z;
    }
  }
}

}  // namespace dtmm
