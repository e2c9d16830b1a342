// Host driver of the library's biaxial eigen-solve (dtmm_gb300/csrc/dtmm_eig4.cuh),
// compiled by nvcc for the CPU.  Reads little-endian float64 records from
// stdin and writes float64 records to stdout:
//
//   mode 0 (matrices):  n, then n x (4 x 4 complex, row-major)
//                       -> n x (ok, 4 eigenvalues, 4 x 4 eigenvectors as columns)
//   mode 1 (voxels):    n, then n x (beta, phi, 3 complex eps, psi, theta, azimuth)
//                       -> n x (4 alpha, 4 x 4 F), F rotated back by phi
//                          (dtmm/linalg.py:674) as the reference's alphaf returns it
//
// Complex numbers are (re, im) pairs; the mode is argv[1].
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dtmm_eig4.cuh"

using namespace dtmm;

static double get() {
  double v;
  if (std::fread(&v, sizeof(double), 1, stdin) != 1) std::exit(2);
  return v;
}
static void put(double v) { std::fwrite(&v, sizeof(double), 1, stdout); }
static void putc_(cpx<double> c) {
  put(c.re);
  put(c.im);
}

int main(int argc, char** argv) {
  const int mode = argc > 1 ? std::atoi(argv[1]) : 0;
  const long n = (long)get();
  for (long c = 0; c < n; ++c) {
    if (mode == 0) {
      cpx<double> A[4][4], lam[4], V[4][4];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          const double re = get(), im = get();
          A[i][j] = mk<double>(re, im);
        }
      const bool ok = e4::eig4(A, lam, V);
      put(ok ? 1.0 : 0.0);
      for (int i = 0; i < 4; ++i) putc_(lam[i]);
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) putc_(V[i][j]);
    } else {
      const double beta = get(), phi = get();
      cpx<double> ev[3];
      for (int i = 0; i < 3; ++i) {
        const double re = get(), im = get();
        ev[i] = mk<double>(re, im);
      }
      const double psi = get(), theta = get(), azim = get();
      cpx<double> F[4][4], al[4];
      biaxial_fmat(beta, ev, std::cos(psi), std::sin(psi), std::cos(theta), std::sin(theta), std::cos(azim - phi),
                   std::sin(azim - phi), F, al);
      const double c0 = std::cos(phi), s0 = std::sin(phi);
      for (int m = 0; m < 4; ++m) {  // rows (Ex, Hy, Ey, Hx) back by phi
        const cpx<double> f0 = F[0][m], f1 = F[1][m], f2 = F[2][m], f3 = F[3][m];
        F[0][m] = f0 * c0 - f2 * s0;
        F[1][m] = f1 * c0 + f3 * s0;
        F[2][m] = f0 * s0 + f2 * c0;
        F[3][m] = -(f1 * s0) + f3 * c0;
      }
      for (int i = 0; i < 4; ++i) putc_(al[i]);
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) putc_(F[i][j]);
    }
  }
  return 0;
}
