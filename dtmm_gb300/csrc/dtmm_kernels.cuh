// Kernels of the GB300 field-transfer engine (the hot path of dtmm's
// transfer_field) other than the register-transform row / column passes
// (dtmm_regkern.cuh).  All kernels are templated on the bulk real type R
// (float = complex64 bulk, double = complex128 bulk); eigen-solves, k-space
// operator tables and window statistics are always computed in FP64.  The
// data layout in HBM is described in dtmm_layer.cuh; k-space tables are
// [lam][H][W][rows][cols].
#pragma once

#include <type_traits>

#include "dtmm_common.cuh"
#include "dtmm_eig4.cuh"
#include "dtmm_layer.cuh"

namespace dtmm {

// ---------------------------------------------------------------------------
// FP64 Berreman eigen-data of an isotropic medium, in the phi = 0 frame, then
// rotated by phi (dtmm/tmm.py:124 and :372 with _dotr2m, dtmm/linalg.py:674).
// ---------------------------------------------------------------------------
__device__ inline void iso_alphaf(double beta, double phi, cpx<double> eps, cpx<double> alpha[4],
                                  cpx<double> F[4][4]) {
  cpx<double> a = csqrt_d(mk<double>(eps.re - beta * beta, eps.im));
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) F[i][j] = mk<double>(0.0, 0.0);
  if (a.re == 0.0 && a.im == 0.0) {
    for (int i = 0; i < 4; ++i) alpha[i] = mk<double>(0.0, 0.0);
    return;
  }
  cpx<double> gp = cdiv(eps, a);
  alpha[0] = a;
  alpha[1] = -a;
  alpha[2] = a;
  alpha[3] = -a;
  F[0][0] = mk<double>(0.5, 0.0);
  F[0][1] = mk<double>(0.5, 0.0);
  F[1][0] = gp * 0.5;
  F[1][1] = gp * -0.5;
  F[2][2] = mk<double>(0.5, 0.0);
  F[2][3] = mk<double>(0.5, 0.0);
  F[3][2] = a * -0.5;
  F[3][3] = a * 0.5;
  double s, c;
  sincos(phi, &s, &c);
  for (int j = 0; j < 4; ++j) {
    cpx<double> f0 = F[0][j], f1 = F[1][j], f2 = F[2][j], f3 = F[3][j];
    F[0][j] = f0 * c - f2 * s;
    F[1][j] = f1 * c + f3 * s;
    F[2][j] = f0 * s + f2 * c;
    F[3][j] = f3 * c - f1 * s;
  }
}

// 4x4 complex inverse by the adjugate (2x2 complementary minors); an exactly
// singular matrix maps to zero (dtmm/linalg.py:460-518).
__device__ inline void inv4(const cpx<double> a[4][4], cpx<double> o[4][4]) {
  cpx<double> s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
  cpx<double> s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
  cpx<double> s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
  cpx<double> s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
  cpx<double> s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
  cpx<double> s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
  cpx<double> c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
  cpx<double> c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
  cpx<double> c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
  cpx<double> c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
  cpx<double> c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
  cpx<double> c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
  cpx<double> det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
  cpx<double> r = (det.re == 0.0 && det.im == 0.0) ? mk<double>(0.0, 0.0) : cdiv(mk<double>(1.0, 0.0), det);
  o[0][0] = (a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3) * r;
  o[0][1] = (-a[0][1] * c5 + a[0][2] * c4 - a[0][3] * c3) * r;
  o[0][2] = (a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3) * r;
  o[0][3] = (-a[2][1] * s5 + a[2][2] * s4 - a[2][3] * s3) * r;
  o[1][0] = (-a[1][0] * c5 + a[1][2] * c2 - a[1][3] * c1) * r;
  o[1][1] = (a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1) * r;
  o[1][2] = (-a[3][0] * s5 + a[3][2] * s2 - a[3][3] * s1) * r;
  o[1][3] = (a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1) * r;
  o[2][0] = (a[1][0] * c4 - a[1][1] * c2 + a[1][3] * c0) * r;
  o[2][1] = (-a[0][0] * c4 + a[0][1] * c2 - a[0][3] * c0) * r;
  o[2][2] = (a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0) * r;
  o[2][3] = (-a[2][0] * s4 + a[2][1] * s2 - a[2][3] * s0) * r;
  o[3][0] = (-a[1][0] * c3 + a[1][1] * c1 - a[1][2] * c0) * r;
  o[3][1] = (a[0][0] * c3 - a[0][1] * c1 + a[0][2] * c0) * r;
  o[3][2] = (-a[3][0] * s3 + a[3][1] * s1 - a[3][2] * s0) * r;
  o[3][3] = (a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0) * r;
}

__device__ inline void inv2(const cpx<double> a[2][2], cpx<double> o[2][2]) {
  cpx<double> det = a[0][0] * a[1][1] - a[0][1] * a[1][0];
  cpx<double> r = (det.re == 0.0 && det.im == 0.0) ? mk<double>(0.0, 0.0) : cdiv(mk<double>(1.0, 0.0), det);
  o[0][0] = a[1][1] * r;
  o[0][1] = -a[0][1] * r;
  o[1][0] = -a[1][0] * r;
  o[1][1] = a[0][0] * r;
}

// ---------------------------------------------------------------------------
// Per-voxel layer operator (FP64 eigen-solve) for one (ray, window).
//
// The real-space step of the reference's split-step layer operator is
// E . diag(exp(i kd alpha)) . E^-1 acting on the "Epn" field (E-field rows of
// forward / backward modes), wrapped by the beam-phase correction C_w of the
// effective medium (dtmm/propagate_4x4.py:80-101, dtmm/matrix.py:133-174).
// For an isotropic effective medium C_w is a scalar per direction,
// exp(-/+ i k0 d/2 a_w) with a_w = sqrt(eps_eff - beta_w^2), so
// C_w M C_w = E . diag(exp(i k0 d (alpha_m -/+ a_w))) . E^-1 per block.
// Stored per voxel (14 complex records): forward block E (4), 1/det, phase
// arguments d*(alpha_0 - a_w), d*(alpha_2 - a_w); backward block E (4),
// 1/det, d*(alpha_1 + a_w), d*(alpha_3 + a_w).  E . P . E^-1 does not depend
// on the scale of E's columns, so the reference's column normalisation
// (dtmm/tmm.py:280-289) is skipped; a singular block (det == 0) zeroes the
// whole operator, as the reference's inverse does.
// ---------------------------------------------------------------------------
struct OpParams {
  const int* permW;       // digit reversal of the row length: records of pixel x go to slot permW[x] (null: x)
  const double* eps_dev;  // if set: (re, im) of the effective medium, overrides eps_eff
  const void* epsv;      // (L?,H?,W?,3) float64 or complex128
  const double* epsa;    // (L?,H?,W?,3) float64
  long long ev_s[3];     // element strides of epsv over (layer, y, x) (0 = broadcast)
  long long ea_s[3];
  int eps_complex;
  int layer;
  double d;              // sub-step thickness (pixels), direction not included
  const double* wbeta;   // [ray][nwin]
  const double* wphi;
  const double* wcos;    // cos, sin of wphi
  const double* wsin;
  const double* waw;     // real path: sqrt(eps_eff - wbeta^2)
  cpx<double> eps_eff;
  int nwin;
  int four;              // 1: 4x4 (both blocks), 0: 2x2 (forward block)
  int rays_per_thread;   // rays [blockIdx.y * rays_per_thread, ...) share the voxel's trigonometry
  int nray;
  // real path with one eps for every voxel: per (ray, window) eps11 - beta^2,
  // its square root and eps11 (eps11 - beta^2 + delta) (null otherwise)
  const double* wev02;
  const double* wevs;
  const double* wc2;
  // 1: no beam correction (a_w = 0): the plain E P E^-1 of a transfer without
  // diffraction matrices (2x2, reflection 1, diffraction 0)
  int uncorrected;
  double scale;          // folded into the records (the row pass's inverse-transform scale)
};

// Records per voxel and window, [ray][window][H][W][record] (REC_BLOCK per
// mode block): complex, or real when the host has proven the real path (real
// eps above beta^2 everywhere).

// Uniaxial / isotropic E rows and eigenvalues in real FP64 arithmetic, valid
// when every eigenvalue and the effective medium exceed beta^2 (then every
// radicand of the solve is positive; the host proves this before selecting
// the real path).  Same formulas as the complex path below.
struct VoxelInv {      // per-voxel invariants of the real-path solve
  double ev[3];        // eps eigenvalues (o, o, e)
  double ie;           // 1 / eps11
  double u, iu2;       // eps11 + delta cos^2(theta), 0.5 / u
  double st, ct;       // sin, cos of the director's polar angle
  double kv, kw;       // 2 delta sin(theta) cos(theta), delta sin^2(theta)
  bool iso;
};

__device__ inline void voxel_inv(const double* e, double theta, VoxelInv& vi) {
  vi.ev[0] = e[0];
  vi.ev[1] = e[1];
  vi.ev[2] = e[2];
  vi.iso = e[0] == e[1] && e[1] == e[2];
  sincos(theta, &vi.st, &vi.ct);
  const double delta = e[2] - e[0];
  vi.ie = 1.0 / e[0];
  vi.u = e[0] + delta * (vi.ct * vi.ct);
  vi.iu2 = 0.5 / vi.u;
  vi.kv = delta * (2.0 * vi.st * vi.ct);
  vi.kw = delta * (vi.st * vi.st);
}

// The biaxial solve with the angles of the voxel and the beam
__device__ __forceinline__ void biaxial_fmat_call(double beta, const cpx<double>* ev, double psi, double ct, double st,
                                               double cf, double sf, cpx<double> (*F)[4], cpx<double>* al) {
  double sps, cps;
  sincos(psi, &sps, &cps);
  biaxial_fmat(beta, ev, cps, sps, ct, st, cf, sf, F, al);
}

// Uniaxial / isotropic E rows (Ex, Ey of the four modes) and eigenvalues in
// real FP64 arithmetic (dtmm/tmm.py:157-278), valid when every eigenvalue
// and the effective medium exceed beta^2 (the host proves this before
// selecting the real path).  ev02 = eps11 - beta^2, evs = sqrt(ev02) and
// c2 = eps11 (ev02 + delta) come from the caller.  Without FOUR only the
// forward modes 0 and 2 are formed.
template <bool FOUR>
__device__ __forceinline__ bool voxel_E_real(double beta, const VoxelInv& vi, double ev02, double evs, double c2,
                                             double sf, double cf, double E[2][4], double al[4]) {
  const double st = vi.st, ct = vi.ct;
  if (vi.iso) {
    const double a = evs;  // sqrt(eps - beta^2)
    al[0] = a; al[1] = -a; al[2] = a; al[3] = -a;
    E[0][0] = 0.5; E[1][0] = 0.0;
    E[0][2] = 0.0; E[1][2] = 0.5;
    if (FOUR) {
      E[0][1] = 0.5; E[1][1] = 0.0;
      E[0][3] = 0.0; E[1][3] = 0.5;
    }
    return a == 0.0;
  }
  const double cfst = cf * st, sfst = st * sf;
  double evpp, evpm;
  if (beta == 0.0) {
    const double sq = sqrt(vi.u * c2) * (2.0 * vi.iu2);
    evpp = sq;
    evpm = -sq;
    E[0][0] = cf;        E[1][0] = sf;
    E[0][2] = -evs * sf; E[1][2] = evs * cf;
    if (FOUR) {
      E[0][1] = cf;        E[1][1] = sf;
      E[0][3] = -evs * sf; E[1][3] = evs * cf;
    }
  } else {
    const double gama = beta * cf;
    const double v = vi.kv * gama;
    const double w = vi.kw * (gama * gama) - c2;
    const double sq = sqrt(v * v - vi.u * w * 4.0) * vi.iu2;
    const double vh = v * vi.iu2;
    evpp = sq - vh;
    evpm = -vh - sq;
    const double ctbeta = ct * beta;
    const double ev02cf = ev02 * cfst;
    E[0][0] = (evpp * ctbeta - ev02cf) * vi.ie;  E[1][0] = -sfst;
    E[0][2] = evs * sfst;                        E[1][2] = ctbeta - evs * cfst;
    if (FOUR) {
      E[0][1] = (ev02cf - evpm * ctbeta) * vi.ie;  E[1][1] = sfst;
      E[0][3] = -evs * sfst;                       E[1][3] = evs * cfst + ctbeta;
    }
  }
  al[0] = evpp; al[1] = evpm; al[2] = evs; al[3] = -evs;
  return false;
}

// Lean solve for complex64 records (real eps above beta^2, uniaxial or
// isotropic voxels): the per-(ray, window) constants of the launch sit in
// shared memory (beam terms beta cos phi, beta sin phi; with one eps for
// every voxel eps11 - beta^2, its square root, eps11 (eps11 - beta^2 +
// delta) and the ordinary mode's phase record), and per voxel and window the
// eigenvalues of dtmm/tmm.py:157-278 take about 12 FP64 operations (16 with
// the backward modes):
//   gamma = beta cos(az - phi) = cos(az) beta cos(phi) + sin(az) beta sin(phi)
//   q = u c2 - eps11 kw gamma^2   (a quarter of the discriminant v^2 - 4 u w,
//                                  whose delta^2 terms cancel)
//   alpha+- = (-kvh gamma +- sqrt(q)) / u   (kvh = delta sin(t) cos(t); sqrt
//                                  from an FP32 seed and one Newton step)
// FP64 because the phase records (alpha - a_w) d cancel.  The E entries,
// which the records keep in FP32, are formed in FP32 from the FP32-rounded
// eigenvalue and voxel / beam terms (sin(t) folded into the cos / sin of
// (az - phi)), rotated back by phi, and their determinants formed and
// inverted in FP32: each entry within a few FP32 roundings of its FP64 value.
struct LeanWin {
  double beta, cp, sp, bcp, bsp;  // beam: beta, cos / sin phi, beta cos / sin phi
  double ev02, evs, c2;           // one eps for every voxel: eps11 - beta^2, its root, eps11 (ev02 + delta)
  double awd;                     // a_w d
  float cpf, spf, r6;             // cos / sin phi in FP32; (evs - a_w) d (one eps for every voxel)
  float betaf, ev02f, evsf;       // beta, and with one eps for every voxel ev02, evs, in FP32
};
constexpr int kLeanChunk = 32;  // windows per shared-memory chunk (<= the block size)

template <bool FOUR>
__device__ __forceinline__ void voxel_op_lean(const OpParams& p, const Grid& g, float* __restrict__ opv, int pix,
                                              int ray0, int ray1) {
  __shared__ LeanWin wc[kLeanChunk];
  constexpr int nrec = FOUR ? OP_REC : REC_BLOCK;
  const float scf = f32_rn(p.scale);
  const int HW = g.H * g.W;
  const bool active = pix < HW;
  const bool uni = p.wev02 != nullptr;
  // the voxel's invariants, shared by every ray and window
  double e0 = 0.0, delta = 0.0, ie = 0.0, iu = 0.0, ct = 0.0, ca = 0.0, sa = 0.0, sca = 0.0, ssa = 0.0;
  double kvh = 0.0, qb = 0.0, u = 0.0;
  float caf = 0.0f, saf = 0.0f, scaf = 0.0f, ssaf = 0.0f, ctf = 0.0f, ief = 0.0f;  // FP32 copies for E
  bool iso = false;
  size_t slot = 0;
  if (active) {
    const int y = pix / g.W, x = pix - y * g.W;
    const long long eo = p.layer * p.ev_s[0] + y * p.ev_s[1] + x * p.ev_s[2];
    const long long ao = p.layer * p.ea_s[0] + y * p.ea_s[1] + x * p.ea_s[2];
    const double* e = (const double*)p.epsv + eo;
    e0 = e[0];
    iso = e[0] == e[1] && e[1] == e[2];
    delta = e[2] - e[0];
    double st;
    sincos(p.epsa[ao + 1], &st, &ct);
    sincos(p.epsa[ao + 2], &sa, &ca);
    ie = rcp_newton(e0);
    u = fma(delta, ct * ct, e0);
    iu = rcp_newton(u);
    kvh = delta * (st * ct);
    qb = e0 * (delta * (st * st));
    sca = st * ca;
    ssa = st * sa;
    caf = f32_rn(ca);
    saf = f32_rn(sa);
    scaf = f32_rn(sca);
    ssaf = f32_rn(ssa);
    ctf = f32_rn(ct);
    ief = f32_rn(ie);
    slot = (size_t)y * g.W + (p.permW ? p.permW[x] : x);
  }
  const int rw0 = ray0 * p.nwin, rw1 = ray1 * p.nwin;
  for (int c0 = rw0; c0 < rw1; c0 += kLeanChunk) {
    const int n = min(kLeanChunk, rw1 - c0);
    __syncthreads();  // the previous chunk is read
    if ((int)threadIdx.x < n) {
      const int rw = c0 + threadIdx.x;
      LeanWin w;
      w.beta = p.wbeta[rw];
      w.cp = p.wcos[rw];
      w.sp = p.wsin[rw];
      w.bcp = w.beta * w.cp;
      w.bsp = w.beta * w.sp;
      const double aw = p.uncorrected ? 0.0 : p.waw[rw];
      w.awd = aw * p.d;
      w.cpf = f32_rn(w.cp);
      w.spf = f32_rn(w.sp);
      w.betaf = f32_rn(w.beta);
      if (uni) {
        w.ev02 = p.wev02[rw];
        w.evs = p.wevs[rw];
        w.c2 = p.wc2[rw];
        w.r6 = f32_rn((w.evs - aw) * p.d);
        w.ev02f = f32_rn(w.ev02);
        w.evsf = f32_rn(w.evs);
      } else {
        w.ev02 = w.evs = w.c2 = 0.0;
        w.r6 = w.ev02f = w.evsf = 0.0f;
      }
      wc[threadIdx.x] = w;
    }
    __syncthreads();
    if (!active) continue;
    for (int k = 0; k < n; ++k) {
      const LeanWin& w = wc[k];
      double ev02, evs, c2;
      float r6, ev02f, evsf;
      if (uni) {
        ev02 = w.ev02;
        evs = w.evs;
        c2 = w.c2;
        r6 = w.r6;
        ev02f = w.ev02f;
        evsf = w.evsf;
      } else {
        ev02 = e0 - w.beta * w.beta;
        evs = sqrt_pos_fast(ev02);
        c2 = e0 * (ev02 + delta);
        r6 = f32_rn(fma(evs, p.d, -w.awd));
        ev02f = f32_rn(ev02);
        evsf = f32_rn(evs);
      }
      // E rows (Ex, Ey) of the forward modes 0, 2 (backward 1, 3), in the beam
      // frame, in FP32; the eigenvalues in FP64
      float E00, E10, E02, E12, E01 = 0.0f, E11 = 0.0f, E03 = 0.0f, E13 = 0.0f;
      double al0, al1 = 0.0;
      bool zero = false;
      if (iso) {
        al0 = evs;
        al1 = -evs;
        E00 = 0.5f; E10 = 0.0f; E02 = 0.0f; E12 = 0.5f;
        if (FOUR) { E01 = 0.5f; E11 = 0.0f; E03 = 0.0f; E13 = 0.5f; }
        zero = evs == 0.0;
      } else if (w.beta == 0.0) {
        const float cf = fmaf(caf, w.cpf, saf * w.spf), sf = fmaf(saf, w.cpf, -caf * w.spf);
        const double sq = sqrt(u * c2) * iu;
        al0 = sq;
        al1 = -sq;
        E00 = cf; E10 = sf; E02 = -evsf * sf; E12 = evsf * cf;
        if (FOUR) { E01 = cf; E11 = sf; E03 = E02; E13 = E12; }
      } else {
        const double gama = fma(ca, w.bcp, sa * w.bsp);
        const double q = fma(-qb, gama * gama, u * c2);
        double r0, hy0, eq;
        sqrt_newton(q, r0, hy0, eq);
        const double kvg = kvh * gama;
        al0 = fma(hy0, eq, r0 - kvg) * iu;
        const float a0f = f32_rn(al0);
        const float cfst = fmaf(scaf, w.cpf, ssaf * w.spf), sfst = fmaf(ssaf, w.cpf, -scaf * w.spf);
        const float ctbeta = ctf * w.betaf;
        const float ev02cf = ev02f * cfst;
        E00 = fmaf(a0f, ctbeta, -ev02cf) * ief;  E10 = -sfst;
        E02 = evsf * sfst;                       E12 = fmaf(-evsf, cfst, ctbeta);
        if (FOUR) {
          al1 = -fma(hy0, eq, r0 + kvg) * iu;
          const float a1f = f32_rn(al1);
          E01 = fmaf(-a1f, ctbeta, ev02cf) * ief;  E11 = sfst;
          E03 = -E02;                              E13 = fmaf(evsf, cfst, ctbeta);
        }
      }
      const float df = fmaf(E00, E12, -(E02 * E10));
      const float db = FOUR ? fmaf(E01, E13, -(E03 * E11)) : 1.0f;
      if (df == 0.0f || db == 0.0f) zero = true;
      float rec[nrec];
      if (zero) {
#pragma unroll
        for (int i = 0; i < nrec; ++i) rec[i] = 0.0f;
      } else {
        // the E rows back to the lab frame (rotation by phi); the first
        // column times scale / det
        const float ex0 = E00, ey0 = E10, ex2 = E02, ey2 = E12;
        const float sf = (fabsf(df) > 1e-30f ? __frcp_rn(df) : f32_rn(1.0 / (double)df)) * scf;
        rec[0] = (ex0 * w.cpf - ey0 * w.spf) * sf;
        rec[1] = ex2 * w.cpf - ey2 * w.spf;
        rec[2] = (ex0 * w.spf + ey0 * w.cpf) * sf;
        rec[3] = ex2 * w.spf + ey2 * w.cpf;
        rec[4] = iso ? r6 : f32_rn(fma(al0, p.d, -w.awd));
        rec[5] = r6;
        if (FOUR) {
          const float ex1 = E01, ey1 = E11, ex3 = E03, ey3 = E13;
          const float sb = (fabsf(db) > 1e-30f ? __frcp_rn(db) : f32_rn(1.0 / (double)db)) * scf;
          rec[6] = (ex1 * w.cpf - ey1 * w.spf) * sb;
          rec[7] = ex3 * w.cpf - ey3 * w.spf;
          rec[8] = (ex1 * w.spf + ey1 * w.cpf) * sb;
          rec[9] = ex3 * w.spf + ey3 * w.cpf;
          rec[10] = iso ? -r6 : f32_rn(fma(al1, p.d, w.awd));
          rec[11] = -r6;
        }
      }
      store_recs<nrec, float>(opv + ((size_t)(c0 + k) * HW + slot) * nrec, rec);
    }
  }
}

// BIAX: the material holds biaxial voxels, which take the general
// eigen-solve (complex path only; without BIAX every voxel is isotropic or
// uniaxial and the kernel keeps the registers of those closed forms)
template <typename R, bool REAL, bool FOUR, bool BIAX>
__global__ void k_voxel_op(OpParams p, Grid g, void* __restrict__ opv) {
  const int HW = g.H * g.W;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const int ray0 = blockIdx.y * p.rays_per_thread;
  const int ray1 = min(ray0 + p.rays_per_thread, p.nray);
  if constexpr (REAL && sizeof(R) == 4) {  // every thread of the block: the solve shares window tables
    voxel_op_lean<FOUR>(p, g, (float*)opv, pix, ray0, ray1);
    return;
  }
  if (pix >= HW) return;
  const int y = pix / g.W, x = pix - y * g.W;
  const long long eo = p.layer * p.ev_s[0] + y * p.ev_s[1] + x * p.ev_s[2];
  const long long ao = p.layer * p.ea_s[0] + y * p.ea_s[1] + x * p.ea_s[2];
  const double theta = p.epsa[ao + 1], azim = p.epsa[ao + 2];
  if (p.eps_dev != nullptr) p.eps_eff = mk<double>(p.eps_dev[0], p.eps_dev[1]);
  constexpr int nrec = FOUR ? OP_REC : REC_BLOCK;
  const size_t slot = (size_t)y * g.W + (p.permW ? p.permW[x] : x);
  // the voxel's trigonometry and invariants, shared by every ray and window
  double sa, ca;
  sincos(azim, &sa, &ca);
  if constexpr (REAL) {
    VoxelInv vi;
    voxel_inv((const double*)p.epsv + eo, theta, vi);
    for (int rw = ray0 * p.nwin; rw < ray1 * p.nwin; ++rw) {
      const double beta = p.wbeta[rw];
      const double cp = p.wcos[rw], sp = p.wsin[rw];
      // cos / sin of (azimuth - phi) by the angle-difference identities
      const double cf = ca * cp + sa * sp, sf = sa * cp - ca * sp;
      const double aw = p.uncorrected ? 0.0 : p.waw[rw];
      double ev02, evs, c2;
      if (p.wev02 != nullptr) {
        ev02 = p.wev02[rw];
        evs = p.wevs[rw];
        c2 = p.wc2[rw];
      } else {
        ev02 = vi.ev[0] - beta * beta;
        evs = sqrt(ev02);
        c2 = vi.ev[0] * (ev02 + (vi.ev[2] - vi.ev[0]));
      }
      double E[2][4], al[4];
      bool zero = voxel_E_real<FOUR>(beta, vi, ev02, evs, c2, sf, cf, E, al);
      // back to the lab frame: rotate the E rows by the beam azimuth phi
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        if (!FOUR && (m & 1)) continue;
        const double ex = E[0][m], ey = E[1][m];
        E[0][m] = ex * cp - ey * sp;
        E[1][m] = ex * sp + ey * cp;
      }
      const double detf = E[0][0] * E[1][2] - E[0][2] * E[1][0];
      double detb = 1.0;
      if (FOUR) detb = E[0][1] * E[1][3] - E[0][3] * E[1][1];
      if (detf == 0.0 || detb == 0.0) zero = true;
      // records in the bulk precision, the first column times scale / det
      R rec[nrec];
      if (zero) {
#pragma unroll
        for (int i = 0; i < nrec; ++i) rec[i] = (R)0;
      } else {
        const double sfd = p.scale / detf;
        rec[0] = to_r<R>(E[0][0] * sfd); rec[1] = to_r<R>(E[0][2]); rec[2] = to_r<R>(E[1][0] * sfd); rec[3] = to_r<R>(E[1][2]);
        rec[4] = to_r<R>((al[0] - aw) * p.d);
        rec[5] = to_r<R>((al[2] - aw) * p.d);
        if (FOUR) {
          const double sbd = p.scale / detb;
          rec[6] = to_r<R>(E[0][1] * sbd); rec[7] = to_r<R>(E[0][3]); rec[8] = to_r<R>(E[1][1] * sbd); rec[9] = to_r<R>(E[1][3]);
          rec[10] = to_r<R>((al[1] + aw) * p.d);
          rec[11] = to_r<R>((al[3] + aw) * p.d);
        }
      }
      store_recs<nrec, R>((R*)opv + ((size_t)rw * HW + slot) * nrec, rec);
    }
    return;
  }
  double st, ct;
  sincos(theta, &st, &ct);
  for (int rw = ray0 * p.nwin; rw < ray1 * p.nwin; ++rw) {
    const double beta = p.wbeta[rw];
    const double cp = p.wcos[rw], sp = p.wsin[rw];
    const double cfw = ca * cp + sa * sp, sfw = sa * cp - ca * sp;
  cpx<double> ev[3];
  if (p.eps_complex) {
    const cpx<double>* e = (const cpx<double>*)p.epsv + eo;
    ev[0] = e[0];
    ev[1] = e[1];
    ev[2] = e[2];
  } else {
    const double* e = (const double*)p.epsv + eo;
    ev[0] = mk<double>(e[0], 0.0);
    ev[1] = mk<double>(e[1], 0.0);
    ev[2] = mk<double>(e[2], 0.0);
  }
  cpx<double> aw = p.uncorrected ? mk<double>(0.0, 0.0) : csqrt_d(mk<double>(p.eps_eff.re - beta * beta, p.eps_eff.im));
  cpx<double> E[2][4];  // rows Ex, Ey of the four mode columns
  cpx<double> al[4];
  bool zero = false;
  const cpx<double> z0 = mk<double>(0.0, 0.0);
  if (ev[0].re == ev[1].re && ev[0].im == ev[1].im && ev[1].re == ev[2].re && ev[1].im == ev[2].im) {
    cpx<double> a = csqrt_d(mk<double>(ev[0].re - beta * beta, ev[0].im));
    if (a.re == 0.0 && a.im == 0.0) zero = true;
    al[0] = a;
    al[1] = -a;
    al[2] = a;
    al[3] = -a;
    const cpx<double> h = mk<double>(0.5, 0.0);
    E[0][0] = h; E[1][0] = z0;
    E[0][1] = h; E[1][1] = z0;
    E[0][2] = z0; E[1][2] = h;
    E[0][3] = z0; E[1][3] = h;
  } else if (BIAX && (ev[0].re != ev[1].re || ev[0].im != ev[1].im)) {
    // biaxial: general eigen-solve and Poynting sort (dtmm/tmm.py:395-401);
    // a failed sort gives a zero F and so a zero operator
    cpx<double> F[4][4];
    biaxial_fmat_call(beta, ev, p.epsa[ao], ct, st, cfw, sfw, F, al);
    for (int m = 0; m < 4; ++m) {
      E[0][m] = F[0][m];
      E[1][m] = F[2][m];
    }
  } else {
    // uniaxial, optic axis rotated by (theta, azimuth - phi) (dtmm/tmm.py:157-278,
    // rotation dtmm/rotation.py:176-194 via :390)
    const double sf = sfw, cf = cfw;
    const double cfst = cf * st, sfst = st * sf;
    const cpx<double> eps11 = ev[0];
    const cpx<double> delta = ev[2] - eps11;
    cpx<double> ev02, evs, evpp, evpm;
    if (beta == 0.0) {
      ev02 = eps11;
      evs = csqrt_d(ev02);
      cpx<double> u = eps11 + delta * (ct * ct);
      cpx<double> w = eps11 * (ev02 + delta);
      cpx<double> sq = cdiv(csqrt_d(u * w), u);
      evpp = sq;
      evpm = -sq;
      E[0][0] = mk<double>(cf, 0.0); E[1][0] = mk<double>(sf, 0.0);
      E[0][1] = mk<double>(cf, 0.0); E[1][1] = mk<double>(sf, 0.0);
      E[0][2] = evs * (-sf);         E[1][2] = evs * cf;
      E[0][3] = evs * (-sf);         E[1][3] = evs * cf;
    } else {
      ev02 = mk<double>(eps11.re - beta * beta, eps11.im);
      evs = csqrt_d(ev02);
      cpx<double> u = eps11 + delta * (ct * ct);
      const double gama = beta * cf;
      cpx<double> v = delta * (gama * 2.0 * st * ct);
      cpx<double> w = delta * (gama * gama * st * st) - eps11 * (ev02 + delta);
      cpx<double> u2 = u * 2.0;
      cpx<double> sq = cdiv(csqrt_d(v * v - u * w * 4.0), u2);
      cpx<double> vh = cdiv(v, u2);
      evpp = sq - vh;
      evpm = -vh - sq;
      const double ctbeta = ct * beta;
      cpx<double> ie = cdiv(mk<double>(1.0, 0.0), eps11);
      cpx<double> ev02cf = ev02 * cfst;
      E[0][0] = (evpp * ctbeta - ev02cf) * ie;  E[1][0] = mk<double>(-sfst, 0.0);
      E[0][1] = (ev02cf - evpm * ctbeta) * ie;  E[1][1] = mk<double>(sfst, 0.0);
      E[0][2] = evs * sfst;                     E[1][2] = mk<double>(ctbeta, 0.0) - evs * cfst;
      E[0][3] = evs * (-sfst);                  E[1][3] = evs * cfst + mk<double>(ctbeta, 0.0);
    }
    al[0] = evpp;
    al[1] = evpm;
    al[2] = evs;
    al[3] = -evs;
  }
  // rotate the E rows back by the beam azimuth phi
  for (int m = 0; m < 4; ++m) {
    cpx<double> ex = E[0][m], ey = E[1][m];
    E[0][m] = ex * cp - ey * sp;
    E[1][m] = ex * sp + ey * cp;
  }
  // forward block: modes 0, 2 ; backward block: modes 1, 3
  cpx<double> detf = E[0][0] * E[1][2] - E[0][2] * E[1][0];
  cpx<double> detb = E[0][1] * E[1][3] - E[0][3] * E[1][1];
  const bool zf = (detf.re == 0.0 && detf.im == 0.0);
  const bool zb = (detb.re == 0.0 && detb.im == 0.0);
  if (zf || (FOUR && zb)) zero = true;
  cpx<R> rec[nrec];
  if (zero) {
    for (int i = 0; i < nrec; ++i) rec[i] = cvt<R>(z0);
  } else {
    // first column times scale / det
    const cpx<double> sfc = cdiv(mk<double>(p.scale, 0.0), detf);
    rec[0] = cvt<R>(E[0][0] * sfc); rec[1] = cvt<R>(E[0][2]); rec[2] = cvt<R>(E[1][0] * sfc); rec[3] = cvt<R>(E[1][2]);
    rec[4] = cvt<R>((al[0] - aw) * p.d);
    rec[5] = cvt<R>((al[2] - aw) * p.d);
    if (FOUR) {
      const cpx<double> sbc = cdiv(mk<double>(p.scale, 0.0), detb);
      rec[6] = cvt<R>(E[0][1] * sbc); rec[7] = cvt<R>(E[0][3]); rec[8] = cvt<R>(E[1][1] * sbc); rec[9] = cvt<R>(E[1][3]);
      rec[10] = cvt<R>((al[1] + aw) * p.d);
      rec[11] = cvt<R>((al[3] + aw) * p.d);
    }
  }
  store_recs<nrec, cpx<R>>((cpx<R>*)opv + ((size_t)rw * HW + slot) * nrec, rec);
  }
}

// ---------------------------------------------------------------------------
// 4x4 transfer without diffraction, reflection mode 2 (dtmm/propagate_4x4.py:18-52
// with no diffraction matrices; dtmm/transfer.py:618-884 without the k-space
// sweep): per pixel, field <- F . diag(exp(i k0 d alpha)) . F^-1 . field for
// every layer and sub-step, with the voxel's Berreman field matrix F and
// eigenvalues alpha for the ray's (beta, phi) (dtmm/tmm.py:124, :157-289,
// rotated back by phi as dtmm/linalg.py:674).  F P F^-1 does not depend on
// the scale of F's columns, so they are not normalised; a singular F gives a
// zero operator, as the reference's inverse does (dtmm/linalg.py:460-518).
// One thread per (pixel, ray) and layer: the FP64 solve once, then the
// operator on every polarisation and wavelength of the ray.
// ---------------------------------------------------------------------------
struct Local4Params {
  const void* epsv;   // (L?,H?,W?,3) float64 or complex128
  const double* epsa; // (L?,H?,W?,3) float64
  long long ev_s[3];
  long long ea_s[3];
  int eps_complex;
  int layer;
  double d;           // sub-step thickness (pixels, signed by direction)
  int nst;            // sub-steps
  const double* ks;   // [lam]
  const double* beta; // [ray * bstride]
  const double* phi;  // [ray * bstride]
  int bstride;        // 1 for the rays' beams, the windows per ray for one window's beams
  // operator: 0 F . P . F^-1; 1 E . P . F^-1 and 2 F . P . E^-1 with E the
  // block matrix of the forward (rows/columns 0, 2) and backward (1, 3)
  // E parts (dtmm/tmm.py:974-996), the half steps of reflection mode 2;
  // 3 E . P . E^-1, the per-voxel step of reflection mode 1
  // (dtmm/propagate_4x4.py:80-101)
  int op;
};

// field matrix and eigenvalues of one voxel (isotropic, uniaxial or biaxial)
__device__ void local_fmat(double beta, double phi, const cpx<double> ev[3], double psi, double theta, double azim,
                           cpx<double> F[4][4], cpx<double> al[4]) {
  const cpx<double> z0 = mk<double>(0.0, 0.0);
  for (int i = 0; i < 4; ++i) {
    al[i] = z0;
    for (int j = 0; j < 4; ++j) F[i][j] = z0;
  }
  const bool e01 = ev[0].re == ev[1].re && ev[0].im == ev[1].im;
  const bool e12 = ev[1].re == ev[2].re && ev[1].im == ev[2].im;
  if (e01 && e12) {
    iso_alphaf(beta, phi, ev[0], al, F);  // already rotated by phi
    return;
  }
  if (e01) {
    double st, ct, sf, cf;
    sincos(theta, &st, &ct);
    sincos(azim - phi, &sf, &cf);
    const cpx<double> eps11 = ev[0], delta = ev[2] - ev[0];
    const cpx<double> u = eps11 + delta * (ct * ct);
    cpx<double> evs, evpp, evpm;
    if (beta == 0.0) {
      evs = csqrt_d(eps11);
      const cpx<double> w = eps11 * (eps11 + delta);
      const cpx<double> sq = cdiv(csqrt_d(u * w), u);
      evpp = sq;
      evpm = -sq;
      F[0][2] = evs * (-sf); F[1][2] = eps11 * (-sf); F[2][2] = evs * cf;    F[3][2] = eps11 * (-cf);
      F[0][3] = evs * (-sf); F[1][3] = eps11 * sf;    F[2][3] = evs * cf;    F[3][3] = eps11 * cf;
      F[0][0] = mk<double>(cf, 0.0); F[1][0] = evpp * cf; F[2][0] = mk<double>(sf, 0.0); F[3][0] = evpp * (-sf);
      F[0][1] = mk<double>(cf, 0.0); F[1][1] = evpm * cf; F[2][1] = mk<double>(sf, 0.0); F[3][1] = evpm * (-sf);
    } else {
      const cpx<double> ev02 = mk<double>(eps11.re - beta * beta, eps11.im);
      evs = csqrt_d(ev02);
      const double gama = beta * cf;
      const cpx<double> v = delta * (gama * 2.0 * st * ct);
      const cpx<double> w = delta * (gama * gama * st * st) - eps11 * (ev02 + delta);
      const cpx<double> u2 = u * 2.0;
      const cpx<double> sq = cdiv(csqrt_d(v * v - u * w * 4.0), u2);
      const cpx<double> vh = cdiv(v, u2);
      evpp = sq - vh;
      evpm = -vh - sq;
      const double sfst = st * sf, cfst = cf * st, ctbeta = ct * beta;
      const cpx<double> ie = cdiv(mk<double>(1.0, 0.0), eps11);
      const cpx<double> ev02cfst = ev02 * cfst;
      const cpx<double> evssfst = evs * sfst, evscfst = evs * cfst, evsctbeta = evs * ctbeta;
      const cpx<double> eps11sfst = eps11 * sfst;
      F[0][2] = evssfst;  F[1][2] = eps11sfst; F[2][2] = mk<double>(ctbeta, 0.0) - evscfst; F[3][2] = ev02cfst - evsctbeta;
      F[0][3] = -evssfst; F[1][3] = eps11sfst; F[2][3] = evscfst + mk<double>(ctbeta, 0.0); F[3][3] = ev02cfst + evsctbeta;
      F[0][0] = (evpp * ctbeta - ev02cfst) * ie;  F[1][0] = mk<double>(ctbeta, 0.0) - evpp * cfst;
      F[2][0] = mk<double>(-sfst, 0.0);           F[3][0] = evpp * sfst;
      F[0][1] = (ev02cfst - evpm * ctbeta) * ie;  F[1][1] = evpm * cfst - mk<double>(ctbeta, 0.0);
      F[2][1] = mk<double>(sfst, 0.0);            F[3][1] = evpm * (-sfst);
    }
    al[0] = evpp; al[1] = evpm; al[2] = evs; al[3] = -evs;
  } else {
    double st, ct, sf, cf;
    sincos(theta, &st, &ct);
    sincos(azim - phi, &sf, &cf);
    biaxial_fmat_call(beta, ev, psi, ct, st, cf, sf, F, al);
  }
  // rotate the field rows (Ex, Hy, Ey, Hx) back by phi
  double s, c;
  sincos(phi, &s, &c);
  for (int m = 0; m < 4; ++m) {
    const cpx<double> f0 = F[0][m], f1 = F[1][m], f2 = F[2][m], f3 = F[3][m];
    F[0][m] = f0 * c - f2 * s;
    F[1][m] = f1 * c + f3 * s;
    F[2][m] = f0 * s + f2 * c;
    F[3][m] = -(f1 * s) + f3 * c;
  }
}

// exp(i kd alpha) of a complex eigenvalue in the bulk precision
template <typename R>
__device__ __forceinline__ cpx<R> local_phase(double kd, cpx<double> a) {
  if constexpr (sizeof(R) == 4) {
    const float e = __expf(-(float)(kd * a.im));
    return phase_of<float>(f32_rn(kd * a.re), 1.0f) * e;
  } else {
    double s, c;
    sincos(kd * a.re, &s, &c);
    const double e = exp(-kd * a.im);
    return mk<double>(e * c, e * s);
  }
}

template <typename R>
__global__ void __launch_bounds__(128) k_local4(Local4Params p, Grid g, const cpx<R>* in, cpx<R>* out,
                                                cpx<R>* bulk_slab) {
  const int HW = g.H * g.W;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const int ray = blockIdx.y;
  if (pix >= HW) return;
  const int y = pix / g.W, x = pix - y * g.W;
  const long long eo = p.layer * p.ev_s[0] + y * p.ev_s[1] + x * p.ev_s[2];
  const long long ao = p.layer * p.ea_s[0] + y * p.ea_s[1] + x * p.ea_s[2];
  cpx<double> ev[3];
  if (p.eps_complex) {
    const cpx<double>* e = (const cpx<double>*)p.epsv + eo;
    ev[0] = e[0]; ev[1] = e[1]; ev[2] = e[2];
  } else {
    const double* e = (const double*)p.epsv + eo;
    ev[0] = mk<double>(e[0], 0.0); ev[1] = mk<double>(e[1], 0.0); ev[2] = mk<double>(e[2], 0.0);
  }
  cpx<double> F[4][4], al[4], Fi[4][4];
  local_fmat(p.beta[ray * p.bstride], p.phi[ray * p.bstride], ev, p.epsa[ao], p.epsa[ao + 1], p.epsa[ao + 2], F, al);
  inv4(F, Fi);
  if (p.op != 0) {
    cpx<double> E[4][4];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) E[i][j] = mk<double>(0.0, 0.0);
    E[0][0] = F[0][0]; E[0][2] = F[0][2]; E[2][0] = F[2][0]; E[2][2] = F[2][2];
    E[1][1] = F[0][1]; E[1][3] = F[0][3]; E[3][1] = F[2][1]; E[3][3] = F[2][3];
    if (p.op != 1) inv4(E, Fi);
    if (p.op != 2) {
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) F[i][j] = E[i][j];
    }
  }
  cpx<R> f[4][4], fi[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      f[i][j] = cvt<R>(F[i][j]);
      fi[i][j] = cvt<R>(Fi[i][j]);
    }
  const int per = g.npol * g.nlam;
  for (int q = 0; q < per; ++q) {
    const int lam = q % g.nlam;
    const int img = ray * per + q;
    const double kd = p.ks[lam] * p.d;
    cpx<R> ph[4];
    for (int m = 0; m < 4; ++m) ph[m] = local_phase<R>(kd, al[m]);
    const cpx<R>* src = in + (size_t)img * 4 * HW + pix;
    cpx<R> v[4];
    for (int c = 0; c < 4; ++c) v[c] = src[(size_t)c * HW];
    for (int st = 0; st < p.nst; ++st) {
      cpx<R> u[4];
      for (int m = 0; m < 4; ++m) {
        cpx<R> acc = mk<R>((R)0, (R)0);
        for (int c = 0; c < 4; ++c) acc = cfma(fi[m][c], v[c], acc);
        u[m] = acc * ph[m];
      }
      for (int c = 0; c < 4; ++c) {
        cpx<R> acc = mk<R>((R)0, (R)0);
        for (int m = 0; m < 4; ++m) acc = cfma(f[c][m], u[m], acc);
        v[c] = acc;
      }
    }
    cpx<R>* dst = out + (size_t)img * 4 * HW + pix;
    for (int c = 0; c < 4; ++c) dst[(size_t)c * HW] = v[c];
    if (bulk_slab) {
      cpx<R>* b = bulk_slab + (size_t)img * 4 * HW + pix;
      for (int c = 0; c < 4; ++c) b[(size_t)c * HW] = v[c];
    }
  }
}

// ---------------------------------------------------------------------------
// 2x2 method in real space (reflection mode 2, and diffraction 0 without
// reflections): one step of the reference's _transfer_ray_2x2_2
// (dtmm/propagate_2x2.py:91-190) per (pixel, beam).  The FP64 field matrices
// of the voxels on both sides of the interface (dtmm/tmm.py:124-403, rotated
// back by phi), then, on every image of the beam's ray (polarisations x
// wavelengths), one E-field operator of the mode's columns:
//   L2_HALF  f <- E P E^-1 f, `reps` times (E, P of the output voxel)
//   L2_ETI   f <- E P Eti f, Eti = St^-1 A^-1 (interface without tracked
//            reflections, dtmm/tmm.py:999-1022)
//   L2_TR    with the interface t (dtmm/tmm.py:925-949) and the tracked wave
//            R: R' = f - t f, g = t f + R; with `bulk` (backward modes, the
//            input medium): bulk += [g ; E2H g]; then f <- E P E^-1 g (E E^-1 g
//            when the output layer has no thickness)
//   L2_BULK  bulk += [f ; E2H f]   (E2H of the output voxel, dtmm/tmm.py:1051)
// Fields: f and R [image][2][H][W], bulk [image][4][H][W].  A singular
// matrix inverts to zero, as the reference's inverse does.
// ---------------------------------------------------------------------------
enum { L2_HALF = 0, L2_ETI = 1, L2_TR = 2, L2_BULK = 3 };

struct Local2Params {
  const void* epsv;   // (L?,H?,W?,3) float64 or complex128
  const double* epsa; // (L?,H?,W?,3) float64
  long long ev_s[3];
  long long ea_s[3];
  int eps_complex;
  int lin, lout;      // layers on both sides: >= 0 a layer of the block, -1 the input medium, -2 the output medium
  double nin2, nout2; // eps of the isotropic boundary media
  double d;           // phase thickness (pixels, signed by the direction)
  int dzero;          // the output layer has no thickness (E E^-1 instead of E P E^-1)
  int mode;           // +1 forward, -1 backward modes
  int reps;           // L2_HALF: applications
  int op;
  const double* ks;   // [lam]
  const double* beta; // [ray * bstride]
  const double* phi;
  int bstride;
};

__device__ __forceinline__ void local2_voxel(const Local2Params& p, int layer, int y, int x, double beta, double phi,
                                             cpx<double> F[4][4], cpx<double> al[4]) {
  cpx<double> ev[3];
  double psi = 0.0, theta = 0.0, azim = 0.0;
  if (layer < 0) {
    const double e = layer == -1 ? p.nin2 : p.nout2;
    ev[0] = ev[1] = ev[2] = mk<double>(e, 0.0);
  } else {
    const long long eo = layer * p.ev_s[0] + y * p.ev_s[1] + x * p.ev_s[2];
    const long long ao = layer * p.ea_s[0] + y * p.ea_s[1] + x * p.ea_s[2];
    if (p.eps_complex) {
      const cpx<double>* e = (const cpx<double>*)p.epsv + eo;
      ev[0] = e[0]; ev[1] = e[1]; ev[2] = e[2];
    } else {
      const double* e = (const double*)p.epsv + eo;
      ev[0] = mk<double>(e[0], 0.0); ev[1] = mk<double>(e[1], 0.0); ev[2] = mk<double>(e[2], 0.0);
    }
    psi = p.epsa[ao];
    theta = p.epsa[ao + 1];
    azim = p.epsa[ao + 2];
  }
  local_fmat(beta, phi, ev, psi, theta, azim, F, al);
}

__device__ __forceinline__ void mul2(const cpx<double> a[2][2], const cpx<double> b[2][2], cpx<double> o[2][2]) {
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) o[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j];
}

template <typename R>
__device__ __forceinline__ void apply2(const cpx<R> m[2][2], cpx<R> v[2]) {
  const cpx<R> a = cfma(m[0][1], v[1], m[0][0] * v[0]);
  const cpx<R> b = cfma(m[1][1], v[1], m[1][0] * v[0]);
  v[0] = a;
  v[1] = b;
}

template <typename R>
__global__ void __launch_bounds__(128) k_local2(Local2Params p, Grid g, cpx<R>* f, cpx<R>* refl, cpx<R>* bulk) {
  const int HW = g.H * g.W;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const int ray = blockIdx.y;
  if (pix >= HW) return;
  const int y = pix / g.W, x = pix - y * g.W;
  const double beta = p.beta[ray * p.bstride], phi = p.phi[ray * p.bstride];
  const int m = p.mode < 0 ? 1 : 0;
  cpx<double> Fb[4][4], alb[4];
  local2_voxel(p, p.lout, y, x, beta, phi, Fb, alb);
  cpx<double> E[2][2], Ei[2][2], A[2][2], L[2][2], T[2][2], H[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) E[i][j] = Fb[2 * i][2 * j + m];
  inv2(E, Ei);
  const cpx<double> z = mk<double>(0.0, 0.0), one = mk<double>(1.0, 0.0);
  // L: the right factor of E P L (E^-1, or Eti through the interface); T: t
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      L[i][j] = Ei[i][j];
      T[i][j] = i == j ? one : z;
      H[i][j] = z;
    }
  if (p.op == L2_ETI || p.op == L2_TR) {
    cpx<double> Fa[4][4], ala[4], Fai[4][4];
    local2_voxel(p, p.lin, y, x, beta, phi, Fa, ala);
    inv4(Fa, Fai);
    cpx<double> St[2][2], Sti[2][2], Ai[2][2], ei[2][2];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        cpx<double> s = z;
        for (int q = 0; q < 4; ++q) s = s + Fai[2 * i + m][q] * Fb[q][2 * j + m];
        St[i][j] = s;
        A[i][j] = Fa[2 * i][2 * j + m];
      }
    inv2(St, Sti);
    inv2(A, Ai);
    mul2(Sti, Ai, ei);
    if (p.op == L2_ETI) {
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) L[i][j] = ei[i][j];
    } else {
      mul2(E, ei, T);  // t = Et . ei
    }
  }
  if (p.op == L2_BULK || (p.op == L2_TR && bulk != nullptr)) {
    cpx<double> B[2][2], Ai2[2][2];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) B[i][j] = Fb[2 * i + 1][2 * j + m];
    inv2(E, Ai2);
    mul2(B, Ai2, H);
  }
  cpx<R> e[2][2], l[2][2], t[2][2], h[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      e[i][j] = cvt<R>(E[i][j]);
      l[i][j] = cvt<R>(L[i][j]);
      t[i][j] = cvt<R>(T[i][j]);
      h[i][j] = cvt<R>(H[i][j]);
    }
  // E L of a layer without thickness (no phase), in FP64 as the reference forms it
  cpx<R> eei[2][2];
  if (p.dzero) {
    cpx<double> M[2][2];
    mul2(E, L, M);
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) eei[i][j] = cvt<R>(M[i][j]);
  }
  const int per = g.npol * g.nlam;
  for (int q = 0; q < per; ++q) {
    const int lam = q % g.nlam;
    const int img = ray * per + q;
    cpx<R>* fs = f + (size_t)img * 2 * HW + pix;
    cpx<R> v[2] = {fs[0], fs[HW]};
    if (p.op == L2_BULK) {
      cpx<R>* b = bulk + (size_t)img * 4 * HW + pix;
      cpx<R> hv[2] = {v[0], v[1]};
      apply2(h, hv);
      b[0] = b[0] + v[0];
      b[(size_t)2 * HW] = b[(size_t)2 * HW] + v[1];
      b[(size_t)HW] = b[(size_t)HW] + hv[0];
      b[(size_t)3 * HW] = b[(size_t)3 * HW] + hv[1];
      continue;
    }
    if (p.op == L2_TR) {
      cpx<R>* rs = refl + (size_t)img * 2 * HW + pix;
      cpx<R> tv[2] = {v[0], v[1]};
      apply2(t, tv);
      const cpx<R> r0 = rs[0], r1 = rs[HW];
      rs[0] = v[0] - tv[0];
      rs[HW] = v[1] - tv[1];
      v[0] = tv[0] + r0;
      v[1] = tv[1] + r1;
      if (bulk != nullptr) {
        cpx<R>* b = bulk + (size_t)img * 4 * HW + pix;
        cpx<R> hv[2] = {v[0], v[1]};
        apply2(h, hv);
        b[0] = b[0] + v[0];
        b[(size_t)2 * HW] = b[(size_t)2 * HW] + v[1];
        b[(size_t)HW] = b[(size_t)HW] + hv[0];
        b[(size_t)3 * HW] = b[(size_t)3 * HW] + hv[1];
      }
    }
    if (p.dzero) {
      apply2(eei, v);
    } else {
      const double kd = p.ks[lam] * p.d;
      const cpx<R> ph0 = local_phase<R>(kd, alb[m]), ph1 = local_phase<R>(kd, alb[m + 2]);
      const int reps = p.op == L2_HALF ? p.reps : 1;
      for (int r = 0; r < reps; ++r) {
        cpx<R> u[2] = {v[0], v[1]};
        apply2(l, u);
        u[0] = u[0] * ph0;
        u[1] = u[1] * ph1;
        apply2(e, u);
        v[0] = u[0];
        v[1] = u[1];
      }
    }
    fs[0] = v[0];
    fs[HW] = v[1];
  }
}

// The forward part of a field for its ray's beam direction in the isotropic
// medium eps, in real space: F diag(1, 0, 1, 0) F^-1 per pixel
// (transmitted_field_direct, dtmm/transfer.py:94-101); in place on [image][4][H][W].
template <typename R>
__global__ void k_project_beam(cpx<R>* f, const double* beta, const double* phi, double eps, Grid g) {
  const int HW = g.H * g.W;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const int ray = blockIdx.y;
  if (pix >= HW) return;
  cpx<double> al[4], F[4][4], Fi[4][4];
  iso_alphaf(beta[ray], phi[ray], mk<double>(eps, 0.0), al, F);
  inv4(F, Fi);
  cpx<R> P[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) P[i][j] = cvt<R>(F[i][0] * Fi[0][j] + F[i][2] * Fi[2][j]);
  const int per = g.npol * g.nlam;
  for (int q = 0; q < per; ++q) {
    cpx<R>* v = f + (size_t)(ray * per + q) * 4 * HW + pix;
    cpx<R> a[4], o[4];
    for (int c = 0; c < 4; ++c) a[c] = v[(size_t)c * HW];
    for (int i = 0; i < 4; ++i) {
      cpx<R> acc = mk<R>((R)0, (R)0);
      for (int j = 0; j < 4; ++j) acc = cfma(P[i][j], a[j], acc);
      o[i] = acc;
    }
    for (int c = 0; c < 4; ++c) v[(size_t)c * HW] = o[c];
  }
}

// E part (components Ex, Ey) of [image][4][H][W] fields into [image][2][H][W]
template <typename R>
__global__ void k_epart(const cpx<R>* __restrict__ f4, cpx<R>* __restrict__ f2, Grid g) {
  const size_t HW = (size_t)g.H * g.W;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)g.NI * 2 * HW) return;
  const size_t img = t / (2 * HW), r = t - img * 2 * HW;
  const size_t c = r / HW, k = r - c * HW;
  f2[t] = f4[(img * 4 + 2 * c) * HW + k];
}

// ref[image] = (E0, H0, E1, H1): the 4-component field of E parts e and H parts h
// ([image][2][H][W] each)
template <typename R>
__global__ void k_join_eh(cpx<R>* __restrict__ ref, const cpx<R>* __restrict__ e, const cpx<R>* __restrict__ h, Grid g) {
  const size_t HW = (size_t)g.H * g.W;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)g.NI * 2 * HW) return;
  const size_t img = t / (2 * HW), r = t - img * 2 * HW;
  const size_t c = r / HW, k = r - c * HW;
  ref[(img * 4 + 2 * c) * HW + k] = e[t];
  ref[(img * 4 + 2 * c + 1) * HW + k] = h[t];
}

// The field matrix of the isotropic medium eps at normal incidence with its
// columns scaled to unit z-Poynting (f_iso with normalize_f, dtmm/tmm.py:1074,
// :701-724) and its inverse: out[0..15] F, out[16..31] F^-1 (one thread)
__global__ void k_iso_fnorm(double eps, cpx<double>* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  cpx<double> al[4], F[4][4], Fi[4][4];
  iso_alphaf(0.0, 0.0, mk<double>(eps, 0.0), al, F);
  for (int i = 0; i < 4; ++i) {
    const double t1 = F[0][i].re * F[1][i].re + F[0][i].im * F[1][i].im;
    const double t2 = F[2][i].re * F[3][i].re + F[2][i].im * F[3][i].im;
    const double n = sqrt(fabs(t1 - t2));
    const double sc = n == 0.0 ? 0.0 : 1.0 / n;
    for (int r = 0; r < 4; ++r) F[r][i] = F[r][i] * sc;
  }
  inv4(F, Fi);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      out[r * 4 + c] = F[r][c];
      out[16 + r * 4 + c] = Fi[r][c];
    }
}

// The reference's "local" normalisation of a projected real-space field f
// with the reference field ref, per pixel in FP64 (dtmm/transfer.py:103-136):
// a = Fn^-1 f the eigen-amplitudes in the output medium at normal incidence,
// J the polarizer of the normalised forward Jones vector (a0, a2), P1 = Fn
// [J, conj J interleaved] Fn^-1; f <- f |clip(I(P1 ref) / I(f))| + (ref - P1 ref)
template <typename R>
__global__ void k_local_norm(cpx<R>* __restrict__ f, const cpx<R>* __restrict__ ref, const cpx<double>* __restrict__ fn,
                             Grid g) {
  const size_t HW = (size_t)g.H * g.W;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)g.NI * HW) return;
  const size_t img = t / HW, k = t - img * HW;
  cpx<double> v[4], r[4], a[4];
  for (int c = 0; c < 4; ++c) {
    v[c] = cvt_d(f[(img * 4 + c) * HW + k]);
    r[c] = cvt_d(ref[(img * 4 + c) * HW + k]);
  }
  const cpx<double>* Fn = fn;
  const cpx<double>* Fi = fn + 16;
  for (int i = 0; i < 4; ++i) {
    cpx<double> s = mk<double>(0.0, 0.0);
    for (int c = 0; c < 4; ++c) s = s + Fi[i * 4 + c] * v[c];
    a[i] = s;
  }
  const double nrm = sqrt(a[0].re * a[0].re + a[0].im * a[0].im + a[2].re * a[2].re + a[2].im * a[2].im);
  const cpx<double> jc = mk<double>(a[0].re / nrm, a[0].im / nrm), js = mk<double>(a[2].re / nrm, a[2].im / nrm);
  const cpx<double> J[2][2] = {{jc * conj(jc), jc * conj(js)}, {js * conj(jc), js * conj(js)}};
  // P1 ref = Fn (M (Fn^-1 ref)), M = J on the forward modes, conj J on the backward ones
  cpx<double> b[4], m[4], p[4];
  for (int i = 0; i < 4; ++i) {
    cpx<double> s = mk<double>(0.0, 0.0);
    for (int c = 0; c < 4; ++c) s = s + Fi[i * 4 + c] * r[c];
    b[i] = s;
  }
  m[0] = J[0][0] * b[0] + J[0][1] * b[2];
  m[2] = J[1][0] * b[0] + J[1][1] * b[2];
  m[1] = conj(J[0][0]) * b[1] + conj(J[0][1]) * b[3];
  m[3] = conj(J[1][0]) * b[1] + conj(J[1][1]) * b[3];
  for (int i = 0; i < 4; ++i) {
    cpx<double> s = mk<double>(0.0, 0.0);
    for (int c = 0; c < 4; ++c) s = s + Fn[i * 4 + c] * m[c];
    p[i] = s;
  }
  double i1 = (p[0].re * p[1].re + p[0].im * p[1].im) - (p[2].re * p[3].re + p[2].im * p[3].im);
  double i2 = (v[0].re * v[1].re + v[0].im * v[1].im) - (v[2].re * v[3].re + v[2].im * v[3].im);
  if (i2 == 0.0) {
    i2 = 1.0;
    i1 = 0.0;
  }
  double fact = i1 / i2;
  if (fact <= -1.0) fact = -1.0;
  if (fact >= 1.0) fact = 1.0;
  fact = fabs(fact);
  for (int c = 0; c < 4; ++c) f[(img * 4 + c) * HW + k] = cvt<R>(v[c] * fact + (r[c] - p[c]));
}

// ---------------------------------------------------------------------------
// 4x4 transfer with diffraction = inf (dtmm/propagate_4x4.py:515-560): per
// wavelength, the FFT amplitude of every eigenwave with beta < betamax is
// carried as a plane wave through every voxel's F . P . F^-1 for that
// wave's own (beta, phi), and the waves are summed in real space, in order
// of increasing beta (ties in FFT-grid order) as the reference sums them.
//   k_full_betaphi  beta, phi of every FFT-grid point (dtmm/wave.py:54)
//   k_full_rank     the sorted in-band mode list of each wavelength
//   k_full_rowdft   amplitudes, step 1: DFT of every row at the in-band
//                   columns (|f_x| <= the largest band limit)
//   k_full_coldft   step 2: the column DFT at each mode's row frequency
//   k_full_apply    the plane waves through the voxels, summed per pixel
// Everything but the stored field is FP64 in both precisions; the sums over
// pixels run in a fixed order (no atomics), so results are deterministic.
// ---------------------------------------------------------------------------
struct FullParams {
  const double* ks;    // [lam]
  double betamax;
  double* beta;        // [lam][H W]
  double* phi;         // [lam][H W]
  int* modes;          // [lam][H W] FFT-grid index of the m-th mode
  int* count;          // [lam] in-band modes
  int limx;            // in-band column half width; S = 2 limx + 1 slots, or all W columns
  int S;
  int C;               // field components per image (4: 4x4, 2: the 2x2 E field)
};

__host__ __device__ __forceinline__ int full_slot_ix(const FullParams& p, int s, int W) {
  return p.S == W ? s : (s - p.limx + W) % W;
}

__global__ void k_full_betaphi(FullParams p, Grid g) {
  const int HW = g.H * g.W;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int lam = blockIdx.y;
  if (k >= HW) return;
  const int iy = k / g.W, ix = k - iy * g.W;
  // numpy.fft.fftfreq: the signed index times 1 / n; the same expression as
  // the band limit of the W axis at yy = 0, so every in-band mode's column
  // lies within the band limit
  const double xx = (double)fsigned(ix, g.W) * (1.0 / g.W), yy = (double)fsigned(iy, g.H) * (1.0 / g.H);
  p.beta[(size_t)lam * HW + k] = (2.0 * M_PI / fabs(p.ks[lam])) * sqrt(xx * xx + yy * yy);
  p.phi[(size_t)lam * HW + k] = atan2(yy, xx);
}

__global__ void k_full_rank(FullParams p, Grid g) {
  const int HW = g.H * g.W;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int lam = blockIdx.y;
  if (k >= HW) return;
  const double* b = p.beta + (size_t)lam * HW;
  const double bk = b[k];
  if (!(bk < p.betamax)) return;
  int rank = 0;
  for (int j = 0; j < HW; ++j) {
    const double bj = b[j];
    rank += (bj < p.betamax) && (bj < bk || (bj == bk && j < k));
  }
  p.modes[(size_t)lam * HW + rank] = k;
  atomicAdd(p.count + lam, 1);
}

template <typename R>
__global__ void k_full_rowdft(FullParams p, Grid g, const cpx<R>* __restrict__ field, cpx<double>* __restrict__ A) {
  const int y = blockIdx.x, line = blockIdx.y;  // line = img * 4 + c
  const int W = g.W;
  const cpx<R>* row = field + ((size_t)line * g.H + y) * W;
  for (int s = threadIdx.x; s < p.S; s += blockDim.x) {
    const int ix = full_slot_ix(p, s, W);
    cpx<double> acc = mk<double>(0.0, 0.0);
    for (int x = 0; x < W; ++x) {
      double sn, cs;
      sincospi(-2.0 * (double)(((long long)ix * x) % W) / W, &sn, &cs);
      const cpx<R> v = row[x];
      acc = acc + mk<double>((double)v.re, (double)v.im) * mk<double>(cs, sn);
    }
    A[((size_t)line * g.H + y) * p.S + s] = acc;
  }
}

__global__ void k_full_coldft(FullParams p, Grid g, const cpx<double>* __restrict__ A, cpx<double>* __restrict__ amp) {
  const int HW = g.H * g.W;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int line = blockIdx.y, img = line / p.C;
  const int lam = img_lam(g, img);
  if (m >= p.count[lam]) return;
  const int k = p.modes[(size_t)lam * HW + m];
  const int iy = k / g.W, ix = k - iy * g.W;
  const int s = p.S == g.W ? ix : fsigned(ix, g.W) + p.limx;
  if (s < 0 || s >= p.S) {  // not reached: in-band modes lie within the band limit
    amp[(size_t)line * HW + m] = mk<double>(0.0, 0.0);
    return;
  }
  const cpx<double>* col = A + (size_t)line * g.H * p.S + s;
  cpx<double> acc = mk<double>(0.0, 0.0);
  for (int y = 0; y < g.H; ++y) {
    double sn, cs;
    sincospi(-2.0 * (double)(((long long)iy * y) % g.H) / g.H, &sn, &cs);
    acc = acc + col[(size_t)y * p.S] * mk<double>(cs, sn);
  }
  amp[(size_t)line * HW + m] = acc;
}

constexpr int kFullImg = 4;  // images of one wavelength accumulated per sweep over the modes

template <typename R>
__global__ void __launch_bounds__(128) k_full_apply(FullParams p, Local4Params q, Grid g,
                                                    const cpx<double>* __restrict__ amp, cpx<R>* __restrict__ out) {
  const int HW = g.H * g.W;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const int lam = blockIdx.y;
  if (pix >= HW) return;
  const int y = pix / g.W, x = pix - y * g.W;
  const long long eo = q.layer * q.ev_s[0] + y * q.ev_s[1] + x * q.ev_s[2];
  const long long ao = q.layer * q.ea_s[0] + y * q.ea_s[1] + x * q.ea_s[2];
  cpx<double> ev[3];
  if (q.eps_complex) {
    const cpx<double>* e = (const cpx<double>*)q.epsv + eo;
    ev[0] = e[0]; ev[1] = e[1]; ev[2] = e[2];
  } else {
    const double* e = (const double*)q.epsv + eo;
    ev[0] = mk<double>(e[0], 0.0); ev[1] = mk<double>(e[1], 0.0); ev[2] = mk<double>(e[2], 0.0);
  }
  const double psi = q.epsa[ao], theta = q.epsa[ao + 1], azim = q.epsa[ao + 2];
  const int nm = p.count[lam];
  const double kd = p.ks[lam] * q.d;
  const double inv_n = 1.0 / ((double)g.H * g.W);
  const int per = g.nray * g.npol;  // images of this wavelength
  for (int q0 = 0; q0 < per; q0 += kFullImg) {
    const int nq = min(kFullImg, per - q0);
    cpx<double> acc[kFullImg][4];
    for (int i = 0; i < kFullImg; ++i)
      for (int c = 0; c < 4; ++c) acc[i][c] = mk<double>(0.0, 0.0);
    for (int m = 0; m < nm; ++m) {
      const int k = p.modes[(size_t)lam * HW + m];
      const int iy = k / g.W, ix = k - iy * g.W;
      cpx<double> F[4][4], Fi[4][4], al[4];
      local_fmat(p.beta[(size_t)lam * HW + k], p.phi[(size_t)lam * HW + k], ev, psi, theta, azim, F, al);
      inv4(F, Fi);
      cpx<double> ph[4];
      for (int i = 0; i < 4; ++i) ph[i] = cexp_i(al[i] * kd);
      double sn, cs;
      const double r = (double)(((long long)iy * y) % g.H) / g.H + (double)(((long long)ix * x) % g.W) / g.W;
      sincospi(2.0 * r, &sn, &cs);
      const cpx<double> wave = mk<double>(cs * inv_n, sn * inv_n);
      for (int i = 0; i < kFullImg; ++i) {
        if (i >= nq) break;
        const int img = (q0 + i) * g.nlam + lam;
        cpx<double> w[4], u[4];
        for (int c = 0; c < 4; ++c) w[c] = amp[((size_t)img * 4 + c) * HW + m] * wave;
        for (int a = 0; a < 4; ++a) {
          cpx<double> t = mk<double>(0.0, 0.0);
          for (int c = 0; c < 4; ++c) t = t + Fi[a][c] * w[c];
          u[a] = t * ph[a];
        }
        for (int c = 0; c < 4; ++c) {
          cpx<double> t = mk<double>(0.0, 0.0);
          for (int a = 0; a < 4; ++a) t = t + F[c][a] * u[a];
          acc[i][c] = acc[i][c] + t;
        }
      }
    }
    for (int i = 0; i < nq; ++i) {
      const int img = (q0 + i) * g.nlam + lam;
      for (int c = 0; c < 4; ++c) out[((size_t)img * 4 + c) * HW + pix] = cvt<R>(acc[i][c]);
    }
  }
}

// 2x2 with diffraction = inf (dtmm/propagate_2x2.py:379-464): per pixel and
// wavelength, every in-band eigenwave (amplitudes amp, in order of
// increasing beta) through the output voxel's E P E^-1 for its own (beta,
// phi) of the mode's columns; when the step passes the interface (q.op = 1)
// E P Eti with the input voxel, or with a tracked wave (tamp) E P (ei w +
// E^-1 t), whose reflected part Ein . eri . w is summed into refl; the
// summed waves replace the field, and with `bulk` they and their H parts
// (E2H of the output voxel) are added to it.  FP64 throughout but the stored
// fields; q.d is the signed thickness of the one step the reference takes.
template <typename R>
__global__ void __launch_bounds__(128) k_full2_apply(FullParams p, Local2Params q, Grid g,
                                                     const cpx<double>* __restrict__ amp,
                                                     const cpx<double>* __restrict__ tamp, cpx<R>* __restrict__ out,
                                                     cpx<R>* __restrict__ refl, cpx<R>* __restrict__ bulk) {
  const int HW = g.H * g.W;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const int lam = blockIdx.y;
  if (pix >= HW) return;
  const int y = pix / g.W, x = pix - y * g.W;
  const int m = q.mode < 0 ? 1 : 0, o = 1 - m;
  const bool iface = q.op != 0, tracked = iface && tamp != nullptr;
  const int nm = p.count[lam];
  const double kd = p.ks[lam] * q.d;
  const double inv_n = 1.0 / ((double)g.H * g.W);
  const int per = g.nray * g.npol;  // images of this wavelength
  const cpx<double> z = mk<double>(0.0, 0.0);
  for (int q0 = 0; q0 < per; q0 += kFullImg) {
    const int nq = min(kFullImg, per - q0);
    cpx<double> acc[kFullImg][2], racc[kFullImg][2], bacc[kFullImg][4];
    for (int i = 0; i < kFullImg; ++i) {
      acc[i][0] = acc[i][1] = racc[i][0] = racc[i][1] = z;
      for (int c = 0; c < 4; ++c) bacc[i][c] = z;
    }
    for (int mm = 0; mm < nm; ++mm) {
      const int k = p.modes[(size_t)lam * HW + mm];
      const int iy = k / g.W, ix = k - iy * g.W;
      const double beta = p.beta[(size_t)lam * HW + k], phi = p.phi[(size_t)lam * HW + k];
      cpx<double> Fb[4][4], alb[4];
      local2_voxel(q, q.lout, y, x, beta, phi, Fb, alb);
      cpx<double> E[2][2], Ei[2][2], Lw[2][2], RM[2][2], H[2][2];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
          E[i][j] = Fb[2 * i][2 * j + m];
          RM[i][j] = H[i][j] = z;
        }
      inv2(E, Ei);
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) Lw[i][j] = Ei[i][j];
      if (iface) {
        cpx<double> Fa[4][4], ala[4], Fai[4][4], St[2][2], Sr[2][2], A[2][2], Sti[2][2], Ai[2][2], ei[2][2];
        local2_voxel(q, q.lin, y, x, beta, phi, Fa, ala);
        inv4(Fa, Fai);
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) {
            cpx<double> st = z, sr = z;
            for (int c = 0; c < 4; ++c) {
              st = st + Fai[2 * i + m][c] * Fb[c][2 * j + m];
              sr = sr + Fai[2 * i + o][c] * Fb[c][2 * j + m];
            }
            St[i][j] = st;
            Sr[i][j] = sr;
            A[i][j] = Fa[2 * i][2 * j + m];
          }
        inv2(St, Sti);
        inv2(A, Ai);
        mul2(Sti, Ai, ei);
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) Lw[i][j] = ei[i][j];
        if (tracked) {
          cpx<double> eri[2][2], Ein[2][2];
          mul2(Sr, ei, eri);
          for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) Ein[i][j] = Fa[2 * i][2 * j + o];
          mul2(Ein, eri, RM);
        }
      }
      if (bulk != nullptr) {
        cpx<double> B[2][2];
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) B[i][j] = Fb[2 * i + 1][2 * j + m];
        mul2(B, Ei, H);
      }
      const cpx<double> ph[2] = {cexp_i(alb[m] * kd), cexp_i(alb[m + 2] * kd)};
      double sn, cs;
      const double r = (double)(((long long)iy * y) % g.H) / g.H + (double)(((long long)ix * x) % g.W) / g.W;
      sincospi(2.0 * r, &sn, &cs);
      const cpx<double> wave = mk<double>(cs * inv_n, sn * inv_n);
      for (int i = 0; i < kFullImg; ++i) {
        if (i >= nq) break;
        const int img = (q0 + i) * g.nlam + lam;
        cpx<double> w[2], v[2];
        for (int c = 0; c < 2; ++c) w[c] = amp[((size_t)img * 2 + c) * HW + mm] * wave;
        for (int a = 0; a < 2; ++a) v[a] = Lw[a][0] * w[0] + Lw[a][1] * w[1];
        if (tracked) {
          cpx<double> t[2];
          for (int c = 0; c < 2; ++c) t[c] = tamp[((size_t)img * 2 + c) * HW + mm] * wave;
          for (int a = 0; a < 2; ++a) {
            racc[i][a] = racc[i][a] + RM[a][0] * w[0] + RM[a][1] * w[1];
            v[a] = v[a] + Ei[a][0] * t[0] + Ei[a][1] * t[1];
          }
        }
        v[0] = v[0] * ph[0];
        v[1] = v[1] * ph[1];
        const cpx<double> e0 = E[0][0] * v[0] + E[0][1] * v[1], e1 = E[1][0] * v[0] + E[1][1] * v[1];
        acc[i][0] = acc[i][0] + e0;
        acc[i][1] = acc[i][1] + e1;
        if (bulk != nullptr) {
          bacc[i][0] = bacc[i][0] + e0;
          bacc[i][2] = bacc[i][2] + e1;
          bacc[i][1] = bacc[i][1] + H[0][0] * e0 + H[0][1] * e1;
          bacc[i][3] = bacc[i][3] + H[1][0] * e0 + H[1][1] * e1;
        }
      }
    }
    for (int i = 0; i < nq; ++i) {
      const int img = (q0 + i) * g.nlam + lam;
      for (int c = 0; c < 2; ++c) {
        out[((size_t)img * 2 + c) * HW + pix] = cvt<R>(acc[i][c]);
        if (tracked) refl[((size_t)img * 2 + c) * HW + pix] = cvt<R>(racc[i][c]);
      }
      if (bulk != nullptr)
        for (int c = 0; c < 4; ++c) {
          cpx<R>& b = bulk[((size_t)img * 4 + c) * HW + pix];
          b = cvt<R>(cvt_d(b) + bacc[i][c]);
        }
    }
  }
}

// ---------------------------------------------------------------------------
// Window statistics and 1D window weight tables (diffraction > 1).
//
// Window (i, j) of the n x n grid is the tent cx_i(beta_x) * cy_j(beta_y),
// open-ended at the grid edges, zero for beta >= betamax, with centres on
// linspace(-betamax, betamax, n) shifted by the folded beam offset
// (dtmm/mode.py:11-70).  Its mean beta, phi is the window^2-weighted mean of
// (beta_x, beta_y) over every wavelength and k (dtmm/mode.py:104-130).
// ---------------------------------------------------------------------------
struct WinParams {
  int n;               // diffraction (windows per axis)
  double betamax;
  double step;         // centre spacing
  const double* xoff;  // [ray] folded offsets
  const double* yoff;
  const double* ks;    // [lam]
};

__device__ __forceinline__ double tent(double db, int typ) {
  double c = 1.0 - fabs(db);
  if (c < 0.0) return 0.0;
  if (typ < 0 && db < 0) return 1.0;
  if (typ > 0 && db > 0) return 1.0;
  return c;
}

__device__ __forceinline__ double win_center(const WinParams& w, int i) {
  // numpy.linspace(-betamax, betamax, n)[i]
  if (i == w.n - 1) return w.betamax;
  double step = (2.0 * w.betamax) / (w.n - 1);
  return -w.betamax + i * step;
}

// partial sums of w^2 bx, w^2 by, w^2 and the non-zero flag over (lam, ky, kx):
// grid (chunks, window row j, ray); each element's beta and row weight once,
// then every window (i, j) of the row; part[((ray * nwin + win) * chunks +
// chunk) * 4 + q].  The final means add the chunks in a fixed order, so
// results are bitwise reproducible.
constexpr int kWinRowMax = 8;  // windows of a row accumulated in registers per sweep

__global__ void k_window_stats(WinParams w, Grid g, double* part) {
  const int ray = blockIdx.z, j = blockIdx.y;
  const int yt = (j == 0) ? -1 : ((j == w.n - 1) ? 1 : 0);
  const double cy0 = win_center(w, j) + w.yoff[ray];
  const int total = g.nlam * g.H * g.W;
  __shared__ double red[4][256];
  for (int i0 = 0; i0 < w.n; i0 += kWinRowMax) {
    const int ni = min(kWinRowMax, w.n - i0);
    double acc[kWinRowMax][4];
    for (int a = 0; a < kWinRowMax; ++a) acc[a][0] = acc[a][1] = acc[a][2] = acc[a][3] = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
      const int lam = t / (g.H * g.W);
      const int k = t - lam * g.H * g.W;
      const int ky = k / g.W, kx = k - ky * g.W;
      const double l = 2.0 * M_PI / w.ks[lam];
      const double bx = l * ((double)fsigned(kx, g.W) * (1.0 / g.W));
      const double by = l * ((double)fsigned(ky, g.H) * (1.0 / g.H));
      const double b = sqrt(bx * bx + by * by);
      if (!(b < w.betamax)) continue;
      const double ty = tent((by - cy0) / w.step, yt);
      if (ty == 0.0) continue;
#pragma unroll
      for (int a = 0; a < kWinRowMax; ++a) {
        if (a >= ni) break;
        const int i = i0 + a;
        const int xt = (i == 0) ? -1 : ((i == w.n - 1) ? 1 : 0);
        const double c = tent((bx - (win_center(w, i) + w.xoff[ray])) / w.step, xt) * ty;
        if (c > 0.0) {
          const double c2 = c * c;
          acc[a][0] += bx * c2;
          acc[a][1] += by * c2;
          acc[a][2] += c2;
          acc[a][3] = 1.0;
        }
      }
    }
    for (int a = 0; a < ni; ++a) {
      __syncthreads();  // the previous window's reads of red are done
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = acc[a][q];
      __syncthreads();
      for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st)
          for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + st];
        __syncthreads();
      }
      const int win = (i0 + a) * w.n + j;
      if (threadIdx.x < 4)
        part[(((size_t)ray * w.n * w.n + win) * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = red[threadIdx.x][0];
    }
  }
}

__global__ void k_window_final(const double* part, int chunks, double* wbeta, double* wphi, int* wzero, double* wcos,
                               double* wsin, int n) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  double acc[4] = {0, 0, 0, 0};
  for (int c = 0; c < chunks; ++c)
    for (int q = 0; q < 4; ++q) acc[q] += part[((size_t)idx * chunks + c) * 4 + q];
  double mx = acc[0], my = acc[1], mn = acc[2];
  if (mn > 0) {
    mx /= mn;
    my /= mn;
  }
  wbeta[idx] = sqrt(mx * mx + my * my);
  wphi[idx] = atan2(my, mx);
  sincos(wphi[idx], wsin + idx, wcos + idx);
  wzero[idx] = acc[3] > 0 ? 0 : 1;
}

// cx[ray][i][lam][kx] and cy[ray][j][lam][ky]; the beta >= betamax cut is
// carried by the diffraction operators, which vanish there.
template <typename R>
__global__ void k_window_tables(WinParams w, Grid g, R* cx, R* cy) {
  const int ray = blockIdx.z;
  const int lam = blockIdx.y;
  const int nmax = g.H > g.W ? g.H : g.W;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < w.n * nmax; t += gridDim.x * blockDim.x) {
    const int i = t / nmax, k = t - i * nmax;
    const int typ = (i == 0) ? -1 : ((i == w.n - 1) ? 1 : 0);
    const double l = 2.0 * M_PI / w.ks[lam];
    if (k < g.W) {
      const double bx = l * ((double)fsigned(k, g.W) * (1.0 / g.W));
      cx[(((size_t)ray * w.n + i) * g.nlam + lam) * g.W + k] = (R)tent((bx - (win_center(w, i) + w.xoff[ray])) / w.step, typ);
    }
    if (k < g.H) {
      const double by = l * ((double)fsigned(k, g.H) * (1.0 / g.H));
      cy[(((size_t)ray * w.n + i) * g.nlam + lam) * g.H + k] = (R)tent((by - (win_center(w, i) + w.yoff[ray])) / w.step, typ);
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 k-space operator tables of the isotropic effective medium, one matrix
// per (lam, ky, kx).  beta >= betamax zeroes the eigen-data (and hence the
// operator), as the reference's diffraction matrices do
// (dtmm/diffract.py:22-70).
// ---------------------------------------------------------------------------
enum KTab {
  KT_D1 = 0,     // 4x4 field -> Epn over d: E . P(d) . F^-1          (dtmm/matrix.py:110)
  KT_D2 = 1,     // 4x4 Epn -> field over d: F . P(d) . E^-1          (dtmm/matrix.py:121)
  KT_PROJ = 2,   // 4x4 forward projection F . diag(1,0,1,0) . F^-1   (dtmm/diffract.py:242)
  KT_DIAG = 3,   // (e+, e-) = exp(+/- i k0 d a_k), stored [lam][kx][ky] (D1 . D2 of two half steps)
  KT_2IN = 4,    // 2x4 [E(d) . t_in] . P_in[rows Ex, Ey]   (2x2 method entry)
  KT_2OUT = 5,   // 4x2 [sum_w win_w ; sum_w win_w E2H_w] . t_out . E(d)   (2x2 method exit)
  KT_WINMAT = 6, // 4x4 window w (proj_mode) of the n x n grid times I     (dtmm/mode.py:11-50)
  KT_CFD = 7,    // 4x4 C . D(d) . C, D = F . P(d) . F^-1 per k, C the correction of window /
                 // beam proj_mode over -d/2 (corrected_field_diffraction_matrix, dtmm/matrix.py:86-93)
  KT_CEPN = 8,   // 4x4 with the 2x2 C . D(d) . C of the forward modes on rows / columns 0, 2 and
                 // of the backward modes on 1, 3, D = j . P(d) . j^-1 of the E parts, C over -d/2
                 // (corrected_Epn_diffraction_matrix, dtmm/matrix.py:38-68)
  KT_CD = 9,     // 4x4 C . D(d), C the correction over -d        (second_field_diffraction_matrix,
  KT_DC = 10,    // 4x4 D(d) . C                                  first_field_..., dtmm/matrix.py:95-107)
  // 2x2 method, E fields of the forward (mode +1) or backward (mode -1) modes;
  // T, Rm the interface transmission / reflection from medium ta into tb
  // (dtmm/diffract.py:215 E_tr_matrix), E(d) the effective medium over d
  // (dtmm/diffract.py:173), wsum the sum of the ray's window weights at k
  KT_2RIN = 11,  // 2x4 wsum . Rm . P_in[rows Ex, Ey]        (entry reflection of the input field)
  KT_2E = 12,    // 2x2 E(d)
  KT_2TE = 13,   // 2x2 T . E(d)
  KT_2R = 14,    // 2x2 wsum . Rm . E(d)
  KT_2X = 15,    // 4x2 [sum_w win_w ; sum_w win_w E2H_w] (E2H in medium tb), masked
  KT_2CE = 16,   // 2x2 C . E(d) . C of window proj_mode (corrected_E_diffraction_matrix, dtmm/matrix.py:38-43)
  KT_2WIN = 17,  // 2x2 window proj_mode of the n x n grid times I
  // boundaries between blocks of different effective media (eps here, eps2 before)
  KT_D12 = 18,   // 4x4 D1(eps, d) . D2(eps2, d2): the merged half steps E P F^-1 . F P E^-1
  KT_2BX = 19,   // 2x2 E(eps, d) . T(eps2 -> eps) . E(eps2, d2), forward modes
  KT_2H = 20,    // 2x2 H from E of the forward modes in the isotropic medium eps (E2H, dtmm/transfer.py:255-267)
  // reflection mode 1 around an anisotropic effective medium, per window of the ray
  KT_C1 = 21,    // 4x4 C . E P(d) F^-1, C = E_w P_w(-d) E_w^-1 of the window's beam (first_corrected_Epn_
                 //   diffraction_matrix, dtmm/matrix.py:127-157)
  KT_C2 = 22,    // 4x4 F P(d) E^-1 . C                 (second_corrected_Epn_diffraction_matrix, :159-174)
  // the 2x2 method's k-space step around an anisotropic effective medium, per window of the ray
  KT_2C1 = 23,   // 2x2 C . E(d), C = j_w P_w(-d) j_w^-1 of the window's beam (first_E_diffraction_matrix,
                 //   dtmm/matrix.py:53-58)
  KT_2C2 = 24,   // 2x2 E(d) . C                       (second_E_diffraction_matrix, :46-51)
};

// the module default of betamax, which the reference's windowed reflection
// mode 4 passes to its diffraction matrices instead of the caller's
// (dtmm/conf.py:148, dtmm/propagate_4x4.py:262-264)
constexpr double kDefaultBetamax = 0.8;

struct KTabParams {
  int what;
  int proj_mode;       // KT_PROJ: +1 forward, -1 backward modes
  const double* eps_dev; // if set: (re, im) of the effective medium, overrides eps
  const double* effx;    // if set: the anisotropic effective medium (symmetry, epsv re/im x 3, psi, theta, phi)
  const double* eps_dev2;  // KT_D12 / KT_2BX: (re, im) of the effective medium before the boundary
  cpx<double> eps2;
  double d2;               // KT_D12 / KT_2BX: thickness of the half step before the boundary
  double d;            // phase thickness (pixels, signed)
  cpx<double> eps;     // effective medium (or the projection medium)
  cpx<double> eps_in;  // 2x2: medium below the stack (entry interface n_in -> effective)
  cpx<double> eps_out; // 2x2: medium above the stack (exit interface, and the E2H medium)
  cpx<double> eps_p;   // 2x2 entry: projection medium of the input field
  int with_t;          // 2x2: apply the interface transmission
  int proj_in;         // 2x2 entry: 1 the input's forward part per k, 0 the input as it is (already projected)
  int mode;            // 2x2: +1 forward, -1 backward modes
  int ta, tb;          // 2x2: interface media (from, into): 0 the effective medium, 1 eps_in, 2 eps_out;
                       // tb is also the E2H medium of KT_2OUT / KT_2X
  double betamax;
  const double* ks;
  // KT_2OUT windows
  int nwin_axis;       // n (1 = no windows)
  const double* wbeta;
  const double* wphi;
  const int* wzero;
  WinParams win;
  int ray;
};

__device__ inline void betaphi_k(const Grid& g, double ks, int ky, int kx, double& beta, double& phi) {
  const double xx = (double)fsigned(kx, g.W) * (1.0 / g.W);
  const double yy = (double)fsigned(ky, g.H) * (1.0 / g.H);
  beta = (2.0 * M_PI / fabs(ks)) * sqrt(xx * xx + yy * yy);
  phi = atan2(yy, xx);
}

// Inverse of the isotropic field matrix in closed form: F = M . blockdiag(A, B)
// with M the rotation of the (Ex, Ey) and (Hy, Hx) row pairs by phi,
// A = [[1/2, 1/2], [gp/2, -gp/2]], B = [[1/2, 1/2], [-a/2, a/2]]; hence
// F^-1 = blockdiag(A^-1, B^-1) . M^T with A^-1 = [[1, 1/gp], [1, -1/gp]],
// B^-1 = [[1, -1/a], [1, 1/a]] (zero when a = 0, as the reference's inverse
// of the zero matrix).
__device__ inline void iso_inv(double phi, cpx<double> eps, cpx<double> a, cpx<double> Fi[4][4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) Fi[i][j] = mk<double>(0.0, 0.0);
  if (a.re == 0.0 && a.im == 0.0) return;
  const cpx<double> igp = cdiv(a, eps);               // 1 / gp = a / eps
  const cpx<double> ia = cdiv(mk<double>(1.0, 0.0), a);
  double s, c;
  sincos(phi, &s, &c);
  // M^T maps (Ex, Hy, Ey, Hx) to the unrotated frame:
  //   Ex0 = c Ex + s Ey, Ey0 = -s Ex + c Ey, Hy0 = c Hy - s Hx, Hx0 = s Hy + c Hx
  // modes 0, 1 use (Ex0, Hy0); modes 2, 3 use (Ey0, Hx0)
  const cpx<double> one = mk<double>(1.0, 0.0);
  Fi[0][0] = one * c; Fi[0][2] = one * s; Fi[0][1] = igp * c; Fi[0][3] = igp * (-s);
  Fi[1][0] = one * c; Fi[1][2] = one * s; Fi[1][1] = igp * (-c); Fi[1][3] = igp * s;
  Fi[2][0] = one * (-s); Fi[2][2] = one * c; Fi[2][1] = ia * (-s); Fi[2][3] = ia * (-c);
  Fi[3][0] = one * (-s); Fi[3][2] = one * c; Fi[3][1] = ia * s; Fi[3][3] = ia * c;
}

// iso eigen-data at grid point k with the betamax cut
__device__ inline void iso_k(double beta, double phi, cpx<double> eps, double betamax, cpx<double> al[4],
                             cpx<double> F[4][4], cpx<double> Fi[4][4]) {
  iso_alphaf(beta, phi, eps, al, F);
  iso_inv(phi, eps, al[0], Fi);
  if (beta >= betamax) {
    for (int i = 0; i < 4; ++i) {
      al[i] = mk<double>(0.0, 0.0);
      for (int j = 0; j < 4; ++j) F[i][j] = Fi[i][j] = mk<double>(0.0, 0.0);
    }
  }
}

// eigen-data of the table's effective medium at (beta, phi), uncut: the
// isotropic closed form, or with an anisotropic effective medium (effx) its
// uniaxial / biaxial field matrix from the eigenvalues and Euler angles
__device__ inline void eff_alphaf(const KTabParams& p, double beta, double phi, cpx<double> al[4],
                                  cpx<double> F[4][4]) {
  if (p.effx == nullptr) {
    iso_alphaf(beta, phi, p.eps, al, F);
    return;
  }
  const cpx<double> ev[3] = {mk<double>(p.effx[1], p.effx[2]), mk<double>(p.effx[3], p.effx[4]),
                             mk<double>(p.effx[5], p.effx[6])};
  local_fmat(beta, phi, ev, p.effx[7], p.effx[8], p.effx[9], F, al);
}

// the same with the inverse and the betamax cut of the diffraction eigen-data
// (dtmm/diffract.py:22-77: every entry zero for beta >= betamax)
__device__ inline void eff_k(const KTabParams& p, double beta, double phi, double betamax, cpx<double> al[4],
                             cpx<double> F[4][4], cpx<double> Fi[4][4]) {
  if (p.effx == nullptr) {
    iso_k(beta, phi, p.eps, betamax, al, F, Fi);
    return;
  }
  if (beta >= betamax) {
    for (int i = 0; i < 4; ++i) {
      al[i] = mk<double>(0.0, 0.0);
      for (int j = 0; j < 4; ++j) F[i][j] = Fi[i][j] = mk<double>(0.0, 0.0);
    }
    return;
  }
  eff_alphaf(p, beta, phi, al, F);
  inv4(F, Fi);
}

// the block matrix of the forward (rows / columns 0, 2) and backward (1, 3)
// E parts of a field matrix (E_mat with mode None, dtmm/tmm.py:974-996)
__device__ inline void epn_of(const cpx<double> F[4][4], cpx<double> E[4][4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) E[i][j] = mk<double>(0.0, 0.0);
  E[0][0] = F[0][0]; E[0][2] = F[0][2]; E[2][0] = F[2][0]; E[2][2] = F[2][2];
  E[1][1] = F[0][1]; E[1][3] = F[0][3]; E[3][1] = F[2][1]; E[3][3] = F[2][3];
}

// 2x2 interface transmission t and reflection r at k from isotropic medium a
// into b for the forward (mode +1) or backward (-1) modes: with S = Fa^-1 Fb,
// St / Sr its transmitted / reflected blocks, A and Er the E parts of Fa's
// mode and opposite-mode columns and Et of Fb's, ei = St^-1 A^-1,
// t = Et ei, r = Er Sr ei (dtmm/tmm.py:850-878, :925-949, :1025-1048); zero
// where beta >= betamax (the reference's masked eigen-data)
__device__ inline void tr_k(double beta, double phi, cpx<double> ea, cpx<double> eb, double betamax, int mode,
                            cpx<double> t[2][2], cpx<double> r[2][2]) {
  cpx<double> al[4], Fa[4][4], Fai[4][4], Fb[4][4], Fbi[4][4];
  iso_k(beta, phi, ea, betamax, al, Fa, Fai);
  iso_k(beta, phi, eb, betamax, al, Fb, Fbi);
  const int m = mode < 0 ? 1 : 0, o = 1 - m;
  cpx<double> St[2][2], Sr[2][2], A[2][2], Er[2][2], Et[2][2], Sti[2][2], Ai[2][2], ei[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      cpx<double> st = mk<double>(0.0, 0.0), sr = mk<double>(0.0, 0.0);
      for (int q = 0; q < 4; ++q) {
        st = st + Fai[2 * i + m][q] * Fb[q][2 * j + m];
        sr = sr + Fai[2 * i + o][q] * Fb[q][2 * j + m];
      }
      St[i][j] = st;
      Sr[i][j] = sr;
      A[i][j] = Fa[2 * i][2 * j + m];
      Er[i][j] = Fa[2 * i][2 * j + o];
      Et[i][j] = Fb[2 * i][2 * j + m];
    }
  inv2(St, Sti);
  inv2(A, Ai);
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) ei[i][j] = Sti[i][0] * Ai[0][j] + Sti[i][1] * Ai[1][j];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      t[i][j] = Et[i][0] * ei[0][j] + Et[i][1] * ei[1][j];
      r[i][j] = mk<double>(0.0, 0.0);
      for (int q = 0; q < 2; ++q) r[i][j] = r[i][j] + Er[i][q] * (Sr[q][0] * ei[0][j] + Sr[q][1] * ei[1][j]);
    }
}

// tent weight of window w (of n x n) of ray `ray` at grid point (ky, kx), zero beyond betamax
// (dtmm/mode.py:11-50); 1 without windows
__device__ inline double win_weight(const WinParams& wp, const Grid& g, double ks, int n, int w, int ray, int ky,
                                    int kx) {
  if (n <= 1) return 1.0;
  const int i = w / n, j = w % n;
  const int xt = (i == 0) ? -1 : ((i == n - 1) ? 1 : 0);
  const int yt = (j == 0) ? -1 : ((j == n - 1) ? 1 : 0);
  const double l = 2.0 * M_PI / ks;
  const double bx = l * ((double)fsigned(kx, g.W) * (1.0 / g.W));
  const double by = l * ((double)fsigned(ky, g.H) * (1.0 / g.H));
  const double b = sqrt(bx * bx + by * by);
  if (!(b < wp.betamax)) return 0.0;
  return tent((bx - (win_center(wp, i) + wp.xoff[ray])) / wp.step, xt) *
         tent((by - (win_center(wp, j) + wp.yoff[ray])) / wp.step, yt);
}

// beta and (cos, sin) of phi at grid point k without the angle itself
__device__ inline void betacs_k(const Grid& g, double ks, int ky, int kx, double& beta, double& c, double& s) {
  const double xx = (double)fsigned(kx, g.W) * (1.0 / g.W);
  const double yy = (double)fsigned(ky, g.H) * (1.0 / g.H);
  const double r = sqrt(xx * xx + yy * yy);
  beta = (2.0 * M_PI / fabs(ks)) * r;
  if (r > 0.0) {
    c = xx / r;
    s = yy / r;
  } else {
    c = 1.0;  // phi = atan2(0, 0) = 0
    s = 0.0;
  }
}

// Closed forms of the isotropic medium's half steps (a = sqrt(eps - beta^2),
// eigenvalues (a, -a, a, -a), e+- = exp(+-i a kd)): E P F^-1 (first, field ->
// E of both directions, dtmm/matrix.py:110) or F P E^-1 (dtmm/matrix.py:121),
// the products of the field matrices written out, with the same cut: zero
// where beta >= betamax or a = 0.
__device__ inline void iso_half_step(bool first, cpx<double> eps, double beta, double c, double s, double kd,
                                     double betamax, cpx<double> M[4][4]) {
  const cpx<double> z = mk<double>(0.0, 0.0);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) M[i][j] = z;
  if (beta >= betamax) return;
  const cpx<double> a = csqrt_d(mk<double>(eps.re - beta * beta, eps.im));
  if (a.re == 0.0 && a.im == 0.0) return;
  const cpx<double> ep = cexp_i(a * kd), em = cexp_i(-a * kd);
  const double cc = c * c, ss = s * s, cs = c * s;
  if (first) {
    // with igp = a / eps, ia = 1 / a: P = igp c^2 + ia s^2, Q = cs (ia - igp), S = igp s^2 + ia c^2
    const cpx<double> igp = cdiv(a, eps), ia = cdiv(mk<double>(1.0, 0.0), a);
    const cpx<double> P = igp * cc + ia * ss, Q = (ia - igp) * cs, S = igp * ss + ia * cc;
    const cpx<double> hp = ep * 0.5, hm = em * 0.5;
    M[0][0] = hp; M[0][1] = hp * P;  M[0][3] = hp * Q;
    M[2][1] = -(hp * Q); M[2][2] = hp; M[2][3] = -(hp * S);
    M[1][0] = hm; M[1][1] = -(hm * P); M[1][3] = -(hm * Q);
    M[3][1] = hm * Q; M[3][2] = hm; M[3][3] = hm * S;
  } else {
    // with gp = eps / a: P = gp c^2 + a s^2, Q = cs (gp - a), S = gp s^2 + a c^2
    const cpx<double> gp = cdiv(eps, a);
    const cpx<double> P = gp * cc + a * ss, Q = (gp - a) * cs, S = gp * ss + a * cc;
    M[0][0] = ep; M[0][1] = em;
    M[1][0] = ep * P; M[1][1] = -(em * P); M[1][2] = ep * Q; M[1][3] = -(em * Q);
    M[2][2] = ep; M[2][3] = em;
    M[3][0] = -(ep * Q); M[3][1] = em * Q; M[3][2] = -(ep * S); M[3][3] = em * S;
  }
}

// complex entries of one table per (lam, ky, kx) (the engine's ktab_entries)
__device__ __forceinline__ int kt_entries(int what) {
  switch (what) {
    case KT_2IN: case KT_2OUT: case KT_2RIN: case KT_2X: return 8;
    case KT_2E: case KT_2TE: case KT_2R: case KT_2CE: case KT_2WIN: case KT_2BX: case KT_2H: case KT_2C1:
    case KT_2C2: return 4;
    default: return 16;
  }
}

// grid point (ky, kx) lies clearly beyond betamax at wavenumber ks: r^2 =
// (kx / W)^2 + (ky / H)^2 above (betamax ks / 2 pi)^2 with a relative margin
// far above the rounding of beta = (2 pi / ks) r, so the exact test beta >=
// betamax agrees; points near the limit take the exact test
__device__ __forceinline__ bool clearly_beyond(const Grid& g, double ks, double betamax, int ky, int kx) {
  const double xx = (double)fsigned(kx, g.W) * (1.0 / g.W);
  const double yy = (double)fsigned(ky, g.H) * (1.0 / g.H);
  const double q = betamax * fabs(ks) * (0.5 / M_PI);
  return xx * xx + yy * yy > q * q * (1.0 + 1e-9);
}

template <typename R>
__global__ void k_ktab(KTabParams p, Grid g, cpx<R>* __restrict__ tab) {
  const int HW = g.H * g.W;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nlam * HW) return;
  const int lam = t / HW, k = t - lam * HW;
  const int ky = k / g.W, kx = k - ky * g.W;
  const double ks = p.ks[lam];
  if (p.eps_dev != nullptr) p.eps = mk<double>(p.eps_dev[0], p.eps_dev[1]);
  if (p.eps_dev2 != nullptr) p.eps2 = mk<double>(p.eps_dev2[0], p.eps_dev2[1]);
  if (p.what == KT_DIAG || p.what == KT_D1 || p.what == KT_D2 || p.what == KT_D12) {
    if (clearly_beyond(g, ks, p.betamax, ky, kx)) {  // zero tables there
      if (p.what == KT_DIAG) {
        const size_t tt = ((size_t)lam * g.W + kx) * g.H + ky;
        tab[tt * 2 + 0] = tab[tt * 2 + 1] = mk<R>((R)0, (R)0);
      } else {
        cpx<R>* o = tab + (size_t)t * 16;
        for (int i = 0; i < 16; ++i) o[i] = mk<R>((R)0, (R)0);
      }
      return;
    }
    double beta, c, s;
    betacs_k(g, ks, ky, kx, beta, c, s);
    if (p.what == KT_DIAG) {
      const cpx<double> a = beta >= p.betamax ? mk<double>(0.0, 0.0) : csqrt_d(mk<double>(p.eps.re - beta * beta, p.eps.im));
      const bool cut = (beta >= p.betamax) || (a.re == 0.0 && a.im == 0.0);
      const cpx<double> z = mk<double>(0.0, 0.0);
      // column-major (lam, kx, ky) so that column passes read it coalesced
      const size_t tt = ((size_t)lam * g.W + kx) * g.H + ky;
      tab[tt * 2 + 0] = cvt<R>(cut ? z : cexp_i(a * (ks * p.d)));
      tab[tt * 2 + 1] = cvt<R>(cut ? z : cexp_i(-a * (ks * p.d)));
      return;
    }
    cpx<double> M[4][4];
    if (p.what == KT_D12) {
      cpx<double> M1[4][4], M2[4][4];
      iso_half_step(true, p.eps, beta, c, s, ks * p.d, p.betamax, M1);
      iso_half_step(false, p.eps2, beta, c, s, ks * p.d2, p.betamax, M2);
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          cpx<double> acc = mk<double>(0.0, 0.0);
          for (int m = 0; m < 4; ++m) acc = acc + M1[i][m] * M2[m][j];
          M[i][j] = acc;
        }
    } else {
      iso_half_step(p.what == KT_D1, p.eps, beta, c, s, ks * p.d, p.betamax, M);
    }
    cpx<R>* o = tab + (size_t)t * 16;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) o[i * 4 + j] = cvt<R>(M[i][j]);
    return;
  }
  // every table but C . D, D . C and C . D . C (cut at their own beta limit)
  // vanishes for beta >= betamax: those points are written as zeros without
  // the eigen-data
  if (p.what != KT_CFD && p.what != KT_CD && p.what != KT_DC) {
    double b0 = 2.0 * p.betamax, c0, s0;
    if (!clearly_beyond(g, ks, p.betamax, ky, kx)) betacs_k(g, ks, ky, kx, b0, c0, s0);
    if (b0 >= p.betamax) {
      const int ne = kt_entries(p.what);
      cpx<R>* o = tab + (size_t)t * ne;
      for (int i = 0; i < ne; ++i) o[i] = mk<R>((R)0, (R)0);
      return;
    }
  }
  double beta, phi;
  betaphi_k(g, ks, ky, kx, beta, phi);
  cpx<double> al[4], F[4][4], Fi[4][4];
  if (p.what == KT_WINMAT) {
    // window w = proj_mode of ray p.ray: tent(beta_x) tent(beta_y), zero beyond betamax
    const int n = p.nwin_axis, w = p.proj_mode;
    double c = 1.0;
    if (n > 1) {
      const int i = w / n, j = w % n;
      const int xt = (i == 0) ? -1 : ((i == n - 1) ? 1 : 0);
      const int yt = (j == 0) ? -1 : ((j == n - 1) ? 1 : 0);
      const double l = 2.0 * M_PI / ks;
      const double bx = l * ((double)fsigned(kx, g.W) * (1.0 / g.W));
      const double by = l * ((double)fsigned(ky, g.H) * (1.0 / g.H));
      const double b = sqrt(bx * bx + by * by);
      c = 0.0;
      if (b < p.win.betamax)
        c = tent((bx - (win_center(p.win, i) + p.win.xoff[p.ray])) / p.win.step, xt) *
            tent((by - (win_center(p.win, j) + p.win.yoff[p.ray])) / p.win.step, yt);
    }
    cpx<R>* o = tab + (size_t)t * 16;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) o[i * 4 + j] = cvt<R>(mk<double>(i == j ? c : 0.0, 0.0));
    return;
  }
  if (p.what == KT_CFD || p.what == KT_CD || p.what == KT_DC) {
    // D: the isotropic layer over d (cut at betamax); C: the beam's own mode
    // over -d/2 (KT_CFD) or -d, uncut (alphaffi, not the diffraction eigen-data)
    const double bmax = (p.what == KT_CFD && p.nwin_axis > 1) ? kDefaultBetamax : p.betamax;
    const double dc = p.what == KT_CFD ? p.d / 2 : p.d;
    eff_k(p, beta, phi, bmax, al, F, Fi);
    cpx<double> D[4][4], Cb[4][4], Fb[4][4], Fbi[4][4], alb[4], T[4][4];
    cpx<double> pd[4], pc[4];
    for (int m = 0; m < 4; ++m) pd[m] = cexp_i(al[m] * (ks * p.d));
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + F[i][m] * pd[m] * Fi[m][j];
        D[i][j] = s;
      }
    const int w = p.ray * p.nwin_axis * p.nwin_axis + p.proj_mode;  // window of this ray
    eff_alphaf(p, p.wbeta[w], p.wphi[w], alb, Fb);
    inv4(Fb, Fbi);
    for (int m = 0; m < 4; ++m) pc[m] = cexp_i(alb[m] * (-ks * dc));
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + Fb[i][m] * pc[m] * Fbi[m][j];
        Cb[i][j] = s;
      }
    cpx<R>* o = tab + (size_t)t * 16;
    if (p.what == KT_CD) {  // C . D
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          cpx<double> s = mk<double>(0.0, 0.0);
          for (int m = 0; m < 4; ++m) s = s + Cb[i][m] * D[m][j];
          o[i * 4 + j] = cvt<R>(s);
        }
      return;
    }
    for (int i = 0; i < 4; ++i)  // T = D . C
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + D[i][m] * Cb[m][j];
        T[i][j] = s;
      }
    if (p.what == KT_DC) {
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) o[i * 4 + j] = cvt<R>(T[i][j]);
      return;
    }
    for (int i = 0; i < 4; ++i)  // C . T
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + Cb[i][m] * T[m][j];
        o[i * 4 + j] = cvt<R>(s);
      }
    return;
  }
  if (p.what == KT_C1 || p.what == KT_C2) {
    // masked eigen-data of the effective medium over d, the beam's correction over -d (uncut)
    eff_k(p, beta, phi, p.betamax, al, F, Fi);
    cpx<double> E[4][4], Ei[4][4], D[4][4], Fb[4][4], Eb[4][4], Ebi[4][4], Cb[4][4], alb[4], pd[4], pc[4];
    epn_of(F, E);
    inv4(E, Ei);
    for (int m = 0; m < 4; ++m) pd[m] = cexp_i(al[m] * (ks * p.d));
    const bool first = p.what == KT_C1;
    for (int i = 0; i < 4; ++i)  // E P F^-1 or F P E^-1
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + (first ? E[i][m] : F[i][m]) * pd[m] * (first ? Fi[m][j] : Ei[m][j]);
        D[i][j] = s;
      }
    const int w = p.ray * p.nwin_axis * p.nwin_axis + p.proj_mode;  // window of this ray
    eff_alphaf(p, p.wbeta[w], p.wphi[w], alb, Fb);
    epn_of(Fb, Eb);
    inv4(Eb, Ebi);
    for (int m = 0; m < 4; ++m) pc[m] = cexp_i(alb[m] * (-ks * p.d));
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + Eb[i][m] * pc[m] * Ebi[m][j];
        Cb[i][j] = s;
      }
    cpx<R>* o = tab + (size_t)t * 16;
    for (int i = 0; i < 4; ++i)  // C . D or D . C
      for (int j = 0; j < 4; ++j) {
        cpx<double> s = mk<double>(0.0, 0.0);
        for (int m = 0; m < 4; ++m) s = s + (first ? Cb[i][m] * D[m][j] : D[i][m] * Cb[m][j]);
        o[i * 4 + j] = cvt<R>(s);
      }
    return;
  }
  if (p.what == KT_CEPN) {
    eff_k(p, beta, phi, p.betamax, al, F, Fi);
    const bool cut = beta >= p.betamax;
    const int w = p.ray * p.nwin_axis * p.nwin_axis + p.proj_mode;  // window of this ray
    cpx<double> alb[4], Fb[4][4];
    eff_alphaf(p, p.wbeta[w], p.wphi[w], alb, Fb);
    cpx<double> M[4][4];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) M[i][j] = mk<double>(0.0, 0.0);
    for (int m = 0; m < 2; ++m) {  // m = 0 forward (columns 0, 2), 1 backward (1, 3)
      cpx<double> J[2][2], Ji[2][2], Jb[2][2], Jbi[2][2], D[2][2], Cm[2][2], T[2][2];
      J[0][0] = F[0][m]; J[0][1] = F[0][m + 2]; J[1][0] = F[2][m]; J[1][1] = F[2][m + 2];
      Jb[0][0] = Fb[0][m]; Jb[0][1] = Fb[0][m + 2]; Jb[1][0] = Fb[2][m]; Jb[1][1] = Fb[2][m + 2];
      inv2(J, Ji);
      inv2(Jb, Jbi);
      const cpx<double> pd[2] = {cexp_i(al[m] * (ks * p.d)), cexp_i(al[m + 2] * (ks * p.d))};
      const cpx<double> pc[2] = {cexp_i(alb[m] * (-ks * p.d / 2)), cexp_i(alb[m + 2] * (-ks * p.d / 2))};
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
          D[i][j] = cut ? mk<double>(0.0, 0.0) : J[i][0] * pd[0] * Ji[0][j] + J[i][1] * pd[1] * Ji[1][j];
          Cm[i][j] = Jb[i][0] * pc[0] * Jbi[0][j] + Jb[i][1] * pc[1] * Jbi[1][j];
        }
      for (int i = 0; i < 2; ++i)  // T = D . C
        for (int j = 0; j < 2; ++j) T[i][j] = D[i][0] * Cm[0][j] + D[i][1] * Cm[1][j];
      for (int i = 0; i < 2; ++i)  // C . T into the rows / columns of the direction
        for (int j = 0; j < 2; ++j) M[2 * i + m][2 * j + m] = Cm[i][0] * T[0][j] + Cm[i][1] * T[1][j];
    }
    cpx<R>* o = tab + (size_t)t * 16;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) o[i * 4 + j] = cvt<R>(M[i][j]);
    return;
  }
  if (p.what == KT_PROJ) {
    iso_k(beta, phi, p.eps, p.betamax, al, F, Fi);
    // F . diag(modes) . F^-1 over the forward (or backward) pair (dtmm/diffract.py:242)
    const int m0 = p.proj_mode > 0 ? 0 : 1;
    cpx<R>* o = tab + (size_t)t * 16;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) o[i * 4 + j] = cvt<R>(F[i][m0] * Fi[m0][j] + F[i][m0 + 2] * Fi[m0 + 2][j]);
    return;
  }
  if (p.what == KT_2H) {
    // rows Hy, Hx from rows Ex, Ey of the forward modes: B A^-1 with A, B the
    // E and H rows of the field matrix's columns 0, 2 (zero beyond betamax)
    iso_k(beta, phi, p.eps, p.betamax, al, F, Fi);
    cpx<double> Am[2][2], Ai[2][2];
    Am[0][0] = F[0][0]; Am[0][1] = F[0][2]; Am[1][0] = F[2][0]; Am[1][1] = F[2][2];
    inv2(Am, Ai);
    cpx<R>* o = tab + (size_t)t * 4;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) o[i * 2 + j] = cvt<R>(F[2 * i + 1][0] * Ai[0][j] + F[2 * i + 1][2] * Ai[1][j]);
    return;
  }
  if (p.what == KT_2WIN) {
    const double c = win_weight(p.win, g, ks, p.nwin_axis, p.proj_mode, p.ray, ky, kx);
    cpx<R>* o = tab + (size_t)t * 4;
    o[0] = o[3] = cvt<R>(mk<double>(c, 0.0));
    o[1] = o[2] = cvt<R>(mk<double>(0.0, 0.0));
    return;
  }
  const int m = p.mode < 0 ? 1 : 0;  // the mode's columns m, m + 2
  if (p.what == KT_2CE || p.what == KT_2C1 || p.what == KT_2C2) {
    // C . E(d) . C: E(d) = j P(d) j^-1 of the medium (masked), C = jb P(-d/2) jb^-1
    // of the window's own beam (uncut), 2x2 of the mode (any effective medium);
    // KT_2C1 / KT_2C2: C over -d on one side only
    eff_k(p, beta, phi, p.betamax, al, F, Fi);
    const bool cut = beta >= p.betamax;
    const int w = p.ray * p.nwin_axis * p.nwin_axis + p.proj_mode;
    cpx<double> alb[4], Fb[4][4];
    eff_alphaf(p, p.wbeta[w], p.wphi[w], alb, Fb);
    cpx<double> J[2][2], Ji[2][2], Jb[2][2], Jbi[2][2], D[2][2], Cm[2][2], T2[2][2];
    J[0][0] = F[0][m]; J[0][1] = F[0][m + 2]; J[1][0] = F[2][m]; J[1][1] = F[2][m + 2];
    Jb[0][0] = Fb[0][m]; Jb[0][1] = Fb[0][m + 2]; Jb[1][0] = Fb[2][m]; Jb[1][1] = Fb[2][m + 2];
    inv2(J, Ji);
    inv2(Jb, Jbi);
    const cpx<double> pd[2] = {cexp_i(al[m] * (ks * p.d)), cexp_i(al[m + 2] * (ks * p.d))};
    const double dc = p.what == KT_2CE ? p.d / 2 : p.d;
    const cpx<double> pc[2] = {cexp_i(alb[m] * (-ks * dc)), cexp_i(alb[m + 2] * (-ks * dc))};
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        D[i][j] = cut ? mk<double>(0.0, 0.0) : J[i][0] * pd[0] * Ji[0][j] + J[i][1] * pd[1] * Ji[1][j];
        Cm[i][j] = Jb[i][0] * pc[0] * Jbi[0][j] + Jb[i][1] * pc[1] * Jbi[1][j];
      }
    if (p.what != KT_2CE) {
      cpx<R>* o = tab + (size_t)t * 4;
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          o[i * 2 + j] = cvt<R>(p.what == KT_2C1 ? Cm[i][0] * D[0][j] + Cm[i][1] * D[1][j]
                                                 : D[i][0] * Cm[0][j] + D[i][1] * Cm[1][j]);
      return;
    }
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) T2[i][j] = D[i][0] * Cm[0][j] + D[i][1] * Cm[1][j];
    cpx<R>* o = tab + (size_t)t * 4;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) o[i * 2 + j] = cvt<R>(Cm[i][0] * T2[0][j] + Cm[i][1] * T2[1][j]);
    return;
  }
  // 2x2 method: E-basis diffraction over d, e(d) * I for the isotropic medium
  // (dtmm/diffract.py:173 with alphaEEi; masked -> 0)
  iso_k(beta, phi, p.eps, p.betamax, al, F, Fi);
  cpx<double> Ed[2][2], Edi[2][2], Edm[2][2];
  Ed[0][0] = F[0][m]; Ed[0][1] = F[0][m + 2]; Ed[1][0] = F[2][m]; Ed[1][1] = F[2][m + 2];
  inv2(Ed, Edi);
  const cpx<double> pd0 = cexp_i(al[m] * (ks * p.d)), pd2 = cexp_i(al[m + 2] * (ks * p.d));
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) Edm[i][j] = Ed[i][0] * pd0 * Edi[0][j] + Ed[i][1] * pd2 * Edi[1][j];
  if (p.what == KT_2E) {
    cpx<R>* o = tab + (size_t)t * 4;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) o[i * 2 + j] = cvt<R>(Edm[i][j]);
    return;
  }
  cpx<double> T[2][2], Rm[2][2];
  const cpx<double> med_a = p.ta == 0 ? p.eps : (p.ta == 1 ? p.eps_in : p.eps_out);
  const cpx<double> med_b = p.tb == 0 ? p.eps : (p.tb == 1 ? p.eps_in : p.eps_out);
  if (p.with_t) {
    tr_k(beta, phi, med_a, med_b, p.betamax, p.mode, T, Rm);
  } else {
    T[0][0] = T[1][1] = mk<double>(1.0, 0.0);
    T[0][1] = T[1][0] = mk<double>(0.0, 0.0);
    Rm[0][0] = Rm[0][1] = Rm[1][0] = Rm[1][1] = mk<double>(0.0, 0.0);
  }
  // window sum and the window-weighted E2H of medium tb for each window's beam
  // (dtmm/tmm.py:1051): only the exit and reflection tables need them
  const int n = p.nwin_axis;
  const int nw = n * n;
  double wsum = 0.0;
  cpx<double> H[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) H[i][j] = mk<double>(0.0, 0.0);
  const bool exit_tab = p.what == KT_2OUT || p.what == KT_2X;
  if (exit_tab || p.what == KT_2R || p.what == KT_2RIN) {
    for (int w = 0; w < nw; ++w) {
      const int idx = p.ray * nw + w;
      if (n > 1 && p.wzero[idx]) continue;
      const double c = win_weight(p.win, g, ks, n, w, p.ray, ky, kx);
      if (n > 1 && c == 0.0) continue;
      wsum += c;
      if (!exit_tab) continue;
      cpx<double> alw[4], Fw[4][4];
      iso_alphaf(p.wbeta[idx], p.wphi[idx], med_b, alw, Fw);
      cpx<double> A[2][2], Ai[2][2];
      A[0][0] = Fw[0][m]; A[0][1] = Fw[0][m + 2]; A[1][0] = Fw[2][m]; A[1][1] = Fw[2][m + 2];
      inv2(A, Ai);
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          H[i][j] = H[i][j] + (Fw[2 * i + 1][m] * Ai[0][j] + Fw[2 * i + 1][m + 2] * Ai[1][j]) * c;
    }
  }
  if (p.what == KT_2IN || p.what == KT_2RIN) {
    // rows Ex, Ey of the forward projection in the input medium
    cpx<double> alp[4], Fp[4][4], Fpi[4][4], P[2][4];
    iso_k(beta, phi, p.eps_p, p.betamax, alp, Fp, Fpi);
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 4; ++j)
        P[i][j] = p.proj_in ? Fp[2 * i][0] * Fpi[0][j] + Fp[2 * i][2] * Fpi[2][j]
                            : mk<double>(j == 2 * i ? 1.0 : 0.0, 0.0);
    cpx<double> DT[2][2];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        DT[i][j] = p.what == KT_2IN ? Edm[i][0] * T[0][j] + Edm[i][1] * T[1][j] : Rm[i][j] * wsum;
    cpx<R>* o = tab + (size_t)t * 8;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 4; ++j) o[i * 4 + j] = cvt<R>(DT[i][0] * P[0][j] + DT[i][1] * P[1][j]);
    return;
  }
  if (p.what == KT_2BX) {
    // E(eps, d) . T(eps2 -> eps) . E(eps2, d2), forward modes
    cpx<double> al2[4], F2[4][4], F2i[4][4], Ed2[2][2], Ed2i[2][2], Edm2[2][2], T2[2][2], R2[2][2];
    iso_k(beta, phi, p.eps2, p.betamax, al2, F2, F2i);
    Ed2[0][0] = F2[0][0]; Ed2[0][1] = F2[0][2]; Ed2[1][0] = F2[2][0]; Ed2[1][1] = F2[2][2];
    inv2(Ed2, Ed2i);
    const cpx<double> q0 = cexp_i(al2[0] * (ks * p.d2)), q2 = cexp_i(al2[2] * (ks * p.d2));
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) Edm2[i][j] = Ed2[i][0] * q0 * Ed2i[0][j] + Ed2[i][1] * q2 * Ed2i[1][j];
    if (p.with_t) {
      tr_k(beta, phi, p.eps2, p.eps, p.betamax, 1, T2, R2);
    } else {
      T2[0][0] = T2[1][1] = mk<double>(1.0, 0.0);
      T2[0][1] = T2[1][0] = mk<double>(0.0, 0.0);
    }
    cpx<double> TE[2][2];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) TE[i][j] = T2[i][0] * Edm2[0][j] + T2[i][1] * Edm2[1][j];
    cpx<R>* o = tab + (size_t)t * 4;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) o[i * 2 + j] = cvt<R>(Edm[i][0] * TE[0][j] + Edm[i][1] * TE[1][j]);
    return;
  }
  if (p.what == KT_2TE || p.what == KT_2R) {
    cpx<R>* o = tab + (size_t)t * 4;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        const cpx<double> v = p.what == KT_2TE ? T[i][0] * Edm[0][j] + T[i][1] * Edm[1][j]
                                               : (Rm[i][0] * Edm[0][j] + Rm[i][1] * Edm[1][j]) * wsum;
        o[i * 2 + j] = cvt<R>(v);
      }
    return;
  }
  // KT_2OUT: [sum_w win_w ; sum_w win_w E2H_w] . T . E(d); KT_2X: the same without T . E(d); masked
  cpx<double> TD[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j)
      TD[i][j] = p.what == KT_2X ? mk<double>(i == j ? 1.0 : 0.0, 0.0) : T[i][0] * Edm[0][j] + T[i][1] * Edm[1][j];
  const bool masked = beta >= p.betamax;
  cpx<R>* o = tab + (size_t)t * 8;
  // rows: Ex, Hy, Ey, Hx of the output field; columns: Ex, Ey of the state
  for (int j = 0; j < 2; ++j) {
    cpx<double> ex = masked ? mk<double>(0.0, 0.0) : TD[0][j] * wsum;
    cpx<double> ey = masked ? mk<double>(0.0, 0.0) : TD[1][j] * wsum;
    cpx<double> hy = masked ? mk<double>(0.0, 0.0) : H[0][0] * TD[0][j] + H[0][1] * TD[1][j];
    cpx<double> hx = masked ? mk<double>(0.0, 0.0) : H[1][0] * TD[0][j] + H[1][1] * TD[1][j];
    o[0 * 2 + j] = cvt<R>(ex);
    o[1 * 2 + j] = cvt<R>(hy);
    o[2 * 2 + j] = cvt<R>(ey);
    o[3 * 2 + j] = cvt<R>(hx);
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_layer_col(ColParams p, Grid g, const cpx<R>* __restrict__ X,
                                                   cpx<R>* __restrict__ U) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int H = g.H, W = g.W, TC = p.tc;
  const int CM = p.cin > p.cout ? p.cin : p.cout;
  // tile element (y, c, xc) at (y * CM + c) * TC + xc: line (c, xc) is
  // l = c * TC + xc with unit line stride and element stride CM * TC
  cpx<R>* T = (cpx<R>*)smem_raw;              // [H][CM][TC]
  cpx<R>* Tm = T + (size_t)CM * H * TC;       // [H][CM][TC] (window work buffer)
  cpx<R>* tw = Tm + (size_t)CM * H * TC;      // [H]
  int* perm = (int*)(tw + H);                 // [H]
  const int es = CM * TC;
  const int img = blockIdx.y;
  const int x0 = blockIdx.x * TC;
  const int lam = img_lam(g, img), ray = img_ray(g, img);
  for (int t = threadIdx.x; t < H; t += blockDim.x) {
    tw[t] = ((const cpx<R>*)p.tw)[t];
    perm[t] = p.perm[t];
  }
  __syncthreads();
  // load (scatter into digit-reversed rows when transforming)
  const int nin = p.cin * H * TC;
  for (int t = threadIdx.x; t < nin; t += blockDim.x) {
    const int c = t / (H * TC), r = t - c * H * TC;
    const int y = r / TC, xc = r - y * TC;
    const int x = x0 + xc;
    cpx<R> v = (x < W) ? X[(((size_t)img * p.cin + c) * H + y) * W + x] : mk<R>(0, 0);
    const int ys = p.do_fwd ? perm[y] : y;
    T[((size_t)ys * CM + c) * TC + xc] = v;
  }
  __syncthreads();
  if (p.do_fwd) fft_dit<R, false>(T, es, 1, p.cin * TC, true, tw, p.plan);
  // k-space operator
  if (p.kop != KOP_NONE) {
    const int nk = H * TC;
    for (int t = threadIdx.x; t < nk; t += blockDim.x) {
      const int ky = t / TC, xc = t - ky * TC;
      const int kx = x0 + xc;
      if (kx >= W) continue;
      const size_t kidx = ((size_t)lam * H + ky) * W + kx;
      cpx<R>* v = T + (size_t)ky * es + xc;
      if (p.kop == KOP_DIAG) {
        const cpx<R>* e = (const cpx<R>*)p.ktab + (((size_t)lam * W + kx) * H + ky) * 2;
        const cpx<R> ep = e[0], em = e[1];
        for (int c = 0; c < p.cin; ++c) v[c * TC] = v[c * TC] * (((c & 1) == 0 || p.cin == 2) ? ep : em);
      } else {
        const cpx<R>* m = (const cpx<R>*)p.ktab + ray * p.ktab_ray_stride + kidx * p.cout * p.cin;
        cpx<R> vin[4], vout[4];
        for (int c = 0; c < p.cin; ++c) vin[c] = v[c * TC];
        for (int co = 0; co < p.cout; ++co) {
          cpx<R> s = mk<R>(0, 0);
          for (int ci = 0; ci < p.cin; ++ci) s = cfma(m[co * p.cin + ci], vin[ci], s);
          vout[co] = s;
        }
        for (int co = 0; co < p.cout; ++co) v[co * TC] = vout[co];
      }
    }
    __syncthreads();
  }
  const int C = p.cout;
  const R sc = (R)p.out_scale;
  for (int jj = 0; jj < p.ny; ++jj) {
    const int j = p.j_only >= 0 ? p.j_only : jj;
    cpx<R>* buf = T;
    if (p.cy != nullptr) {
      const R* cyj = (const R*)p.cy + (((size_t)ray * p.cy_rows + j) * g.nlam + lam) * H;
      for (int t = threadIdx.x; t < H * C * TC; t += blockDim.x) {
        const int y = t / (C * TC), r = t - y * C * TC;
        const size_t o = (size_t)y * es + r;
        Tm[o] = T[o] * cyj[y];
      }
      buf = Tm;
      __syncthreads();
    }
    if (p.inverse_out) fft_dif<R, true>(buf, es, 1, C * TC, true, tw, p.plan);
    cpx<R>* Uj = U + (size_t)jj * g.NI * C * H * W;
    for (int t = threadIdx.x; t < C * H * TC; t += blockDim.x) {
      const int c = t / (H * TC), r = t - c * H * TC;
      const int y = r / TC, xc = r - y * TC;
      const int x = x0 + xc;
      if (x >= W) continue;
      const int ys = p.inverse_out ? perm[y] : y;
      Uj[(((size_t)img * C + c) * H + y) * W + x] = buf[((size_t)ys * CM + c) * TC + xc] * sc;
    }
    __syncthreads();
  }
}

// Row pass, one row y of a group of G wavelengths (all polarisations) of one
// ray.  The (image, component) lines sit at an odd line stride and every FFT
// pass interleaves butterflies across lines (consecutive threads, consecutive
// lines), which keeps shared-memory access free of bank conflicts and turns
// twiddle reads into broadcasts.  The per-voxel step walks the digit-reversed
// slots q of the inverse transform's output (x = iperm[q]) and accumulates in
// the same slots, the input order of the forward transform.  Operator records
// are read once per block and window, phases once per wavelength.
// REAL: records are real (see k_voxel_op).
template <typename R, int C, bool REAL>
__global__ void __launch_bounds__(256, 3) k_layer_row(RowParams p, Grid g, const cpx<R>* __restrict__ U,
                                                   cpx<R>* __restrict__ X) {
  using T = typename std::conditional<REAL, R, cpx<R>>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int W = g.W, H = g.H;
  const int LS = W | 1;
  const int ngrp = (g.nlam + p.G - 1) / p.G;
  const int npg = (g.npol + p.PB - 1) / p.PB;
  const int y = blockIdx.x;
  const int pg = blockIdx.y % npg, rg = blockIdx.y / npg;
  const int ray = rg / ngrp, grp = rg - ray * ngrp;
  const int lam0 = grp * p.G, pol0 = pg * p.PB;
  const int G = min(p.G, g.nlam - lam0);
  const int NP = min(p.PB, g.npol - pol0);  // polarisations of this block
  const int nimg = G * NP, nlines = nimg * C;
  cpx<R>* acc = (cpx<R>*)smem_raw;                 // [lines][LS] (digit-reversed)
  cpx<R>* tmp = acc + (size_t)p.G * p.PB * C * LS; // [lines][LS]
  cpx<R>* tw = tmp + (size_t)p.G * p.PB * C * LS;  // [W]
  const int HW = H * W;
  const int nwin = p.nx * p.ny;
  for (int t = threadIdx.x; t < W; t += blockDim.x) tw[t] = ((const cpx<R>*)p.tw)[t];
  for (int t = threadIdx.x; t < nlines * LS; t += blockDim.x) acc[t] = mk<R>(0, 0);
  const R sc = (R)p.in_scale;  // det of each block's records
  __syncthreads();
  // line l <-> (image = (g, pol), component c): l = (g * NP + pol) * C + c
  for (int j = 0; j < p.ny; ++j) {
    // a single-window chain reads the one window row the column pass emitted
    const cpx<R>* Uj = U + (size_t)(p.win_only >= 0 ? 0 : j) * g.NI * C * HW;
    for (int i = 0; i < p.nx; ++i) {
      const int w = i * p.ny + j;
      if (p.win_only >= 0 && w != p.win_only) continue;
      if (p.wzero != nullptr && p.wzero[ray * nwin + w]) continue;
      // window-weighted rows (natural order, coalesced)
      for (int l = 0; l < nlines; ++l) {
        const int c = l % C, im = l / C;
        const int gl = im / NP, pol = pol0 + im - gl * NP;
        const int lam = lam0 + gl;
        const int img = (ray * g.npol + pol) * g.nlam + lam;
        const cpx<R>* src = Uj + (((size_t)img * C + c) * H + y) * W;
        const R* cxl = (p.cx && p.use_cx) ? (const R*)p.cx + (((size_t)ray * p.nx + i) * g.nlam + lam) * W : nullptr;
        cpx<R>* dst = tmp + (size_t)l * LS;
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
          cpx<R> v = src[x];
          dst[x] = cxl ? v * cxl[x] : v;
        }
      }
      __syncthreads();
      fft_dif<R, true>(tmp, 1, LS, nlines, true, tw, p.plan);
      // per-voxel operator of window w; records are stored in the row's
      // digit-reversed order (slot q), so these loads are coalesced
      const int rs = p.rec_stride;
      const T* opw = (const T*)p.op + (((size_t)ray * nwin + w) * HW + (size_t)y * W) * rs;
      constexpr int NR = C == 4 ? OP_REC : REC_BLOCK;
      for (int q = threadIdx.x; q < W; q += blockDim.x) {
        T rec[NR];
        load_recs<NR, T>(opw + (size_t)q * rs, rec);
        const T* ef = rec;
        const T* eb = rec + (C == 4 ? REC_BLOCK : 0);
        for (int gl = 0; gl < G; ++gl) {
          const R kph = (R)(p.ks[lam0 + gl] * p.dir);
          // projector form of each block: q = p1 scale, dp = p0 - p1
          cpx<R> qf, dpf, qb, dpb;
          {
            const cpx<R> f0 = phase_of(ef[4], kph), f1 = phase_of(ef[5], kph);
            qf = f1 * sc;
            dpf = f0 - f1;
          }
          if (C == 4) {
            const cpx<R> b0 = phase_of(eb[4], kph), b1 = phase_of(eb[5], kph);
            qb = b1 * sc;
            dpb = b0 - b1;
          }
          for (int pol = 0; pol < NP; ++pol) {
            const int l0 = (gl * NP + pol) * C;
            const cpx<R>* h = tmp + (size_t)l0 * LS + q;
            cpx<R>* a = acc + (size_t)l0 * LS + q;
            if (C == 4) {
              cpx<R> a0 = a[0], a1 = a[LS], a2 = a[2 * LS], a3 = a[3 * LS];
              apply_block<R, T>(ef, qf, dpf, h[0], h[2 * LS], a0, a2);
              apply_block<R, T>(eb, qb, dpb, h[LS], h[3 * LS], a1, a3);
              a[0] = a0; a[LS] = a1; a[2 * LS] = a2; a[3 * LS] = a3;
            } else {
              cpx<R> a0 = a[0], a1 = a[LS];
              apply_block<R, T>(ef, qf, dpf, h[0], h[LS], a0, a1);
              a[0] = a0; a[LS] = a1;
            }
          }
        }
      }
      __syncthreads();
    }
  }
  // forward row transform of the accumulator (digit-reversed in, natural out) and store
  fft_dit<R, false>(acc, 1, LS, nlines, true, tw, p.plan);
  for (int l = 0; l < nlines; ++l) {
    const int c = l % C, im = l / C;
    const int gl = im / NP, pol = pol0 + im - gl * NP;
    const int img = (ray * g.npol + pol) * g.nlam + lam0 + gl;
    cpx<R>* dst = X + (((size_t)img * C + c) * H + y) * W;
    const cpx<R>* src = acc + (size_t)l * LS;
    for (int x = threadIdx.x; x < W; x += blockDim.x) dst[x] = p.accumulate ? dst[x] + src[x] : src[x];
  }
}

// ---------------------------------------------------------------------------
// Plain row FFT of every (image, component, y) line, src -> dst (the same
// array for an in-place transform: a block reads its lines completely before
// it writes them, and no other block touches them).
// ---------------------------------------------------------------------------
template <typename R, bool INV>
__global__ void __launch_bounds__(256) k_fft_rows(const cpx<R>* src, cpx<R>* dst, int nlines, int W, FFTPlan plan,
                                                  const cpx<R>* __restrict__ twg, const int* __restrict__ permg,
                                                  double scale, int lpb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<R>* s = (cpx<R>*)smem_raw;
  cpx<R>* tw = s + (size_t)lpb * W;
  int* perm = (int*)(tw + W);
  for (int t = threadIdx.x; t < W; t += blockDim.x) {
    tw[t] = twg[t];
    perm[t] = permg[t];
  }
  __syncthreads();
  const int l0 = blockIdx.x * lpb;
  const int nl = min(lpb, nlines - l0);
  for (int t = threadIdx.x; t < nl * W; t += blockDim.x) {
    const int l = t / W, x = t - l * W;
    cpx<R> v = src[(size_t)(l0 + l) * W + x];
    s[l * W + (INV ? x : perm[x])] = v;
  }
  __syncthreads();
  if (INV)
    fft_dif<R, true>(s, 1, W, nl, false, tw, plan);
  else
    fft_dit<R, false>(s, 1, W, nl, false, tw, plan);
  const R sc = (R)scale;
  for (int t = threadIdx.x; t < nl * W; t += blockDim.x) {
    const int l = t / W, x = t - l * W;
    dst[(size_t)(l0 + l) * W + x] = s[l * W + (INV ? perm[x] : x)] * sc;
  }
}

// ---------------------------------------------------------------------------
// Between-pass helpers of the 4x4 multi-pass (reflection) iteration
// (dtmm/transfer.py:815-873).  Arrays are [image][4][H][W].
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ double poynting(const cpx<R> f[4]) {
  return (double)(f[0].re * f[1].re + f[0].im * f[1].im) - (double)(f[2].re * f[3].re + f[2].im * f[3].im);
}

struct NotchParams {
  int on;
  double x0, sigma;
  double den;  // 1 - exp(-x0 / sigma) (host)
  const double* ks;
};

// the notch of denoise_field at k: (1 - exp(-a / sigma)) / (1 - exp(-x0 / sigma)),
// a = |beta - x0| clipped to [0, x0] (beta as in betaphi_k)
__device__ __forceinline__ double notch_k(const NotchParams& n, const Grid& g, int lam, int ky, int kx) {
  if (!n.on) return 1.0;
  const double xx = (double)fsigned(kx, g.W) * (1.0 / g.W);
  const double yy = (double)fsigned(ky, g.H) * (1.0 / g.H);
  const double beta = (2.0 * M_PI / fabs(n.ks[lam])) * sqrt(xx * xx + yy * yy);
  double a = fabs(beta - n.x0);
  if (a > n.x0) a = n.x0;
  if (a < 0.0) a = 0.0;
  return (1.0 - exp(-a / n.sigma)) / n.den;
}

// k-space: f <- notch * P . f, optionally with the per-k intensity renormalisation
// of project_normalized_fft (dtmm/transfer.py:67-90).  One thread per (lam, k):
// the matrix and the notch once for every image of the wavelength.
// With iref (normalize only) the intensity to restore is iref's at each k
// instead of the field's own (the reference field's spectrum).
template <typename R>
__global__ void k_kproject(cpx<R>* __restrict__ f, const cpx<R>* __restrict__ P, Grid g, int normalize, NotchParams nt,
                           const cpx<R>* __restrict__ iref) {
  const int HW = g.H * g.W;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)g.nlam * HW) return;
  const int lam = (int)(t / HW), k = (int)(t - (size_t)lam * HW);
  const int ky = k / g.W, kx = k - ky * g.W;
  cpx<R> m[16];
  load_recs<16, cpx<R>>(P + ((size_t)lam * HW + k) * 16, m);
  const double notch = notch_k(nt, g, lam, ky, kx);
  const int per = g.nray * g.npol;
  for (int q = 0; q < per; ++q) {
    const size_t img = (size_t)q * g.nlam + lam;
    cpx<R> v[4], o[4];
    for (int c = 0; c < 4; ++c) v[c] = f[(img * 4 + c) * HW + k];
    for (int i = 0; i < 4; ++i) {
      cpx<R> s = mk<R>(0, 0);
      for (int j = 0; j < 4; ++j) s = cfma(m[i * 4 + j], v[j], s);
      o[i] = s;
    }
    double fact = 1.0;
    if (normalize) {
      double i1 = poynting(v), i2 = poynting(o);
      if (iref != nullptr) {
        cpx<R> rv[4];
        for (int c = 0; c < 4; ++c) rv[c] = iref[(img * 4 + c) * HW + k];
        i1 = poynting(rv);
      }
      if (i2 == 0.0) {
        i2 = 1.0;
        i1 = 0.0;
      }
      fact = i1 / i2;
      if (fact <= -1) fact = -1;
      if (fact >= 1) fact = 1;
      fact = fabs(fact);
    }
    fact *= notch;
    for (int c = 0; c < 4; ++c) f[(img * 4 + c) * HW + k] = o[c] * (R)fact;
  }
}

// per-image pixel sums of the z-Poynting component, FP64 accumulation:
// grid (chunks, images), block sums of each image's chunk of pixels into
// part[img * chunks + chunk]; k_total_sum adds the chunks in a fixed order
template <typename R>
__global__ void k_total_intensity(const cpx<R>* __restrict__ f, Grid g, double* part) {
  const int HW = g.H * g.W;
  const int img = blockIdx.y, chunk = blockIdx.x, nch = gridDim.x;
  const int k0 = (int)(((long long)HW * chunk) / nch), k1 = (int)(((long long)HW * (chunk + 1)) / nch);
  double s = 0.0;
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    cpx<R> v[4];
    for (int c = 0; c < 4; ++c) v[c] = f[((size_t)img * 4 + c) * HW + k];
    s += poynting(v);
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)img * nch + chunk] = red[0];
}

__global__ void k_total_sum(const double* part, int chunks, double* out, int n) {
  const int img = blockIdx.x * blockDim.x + threadIdx.x;
  if (img >= n) return;
  double s = 0.0;
  for (int c = 0; c < chunks; ++c) s += part[(size_t)img * chunks + c];
  out[img] = s;
}

// elementwise: out = a*x + b*y with per-image real factors (null = 1)
template <typename R>
__global__ void k_axpby(cpx<R>* out, const cpx<R>* x, const double* ax, double sx, const cpx<R>* y, const double* by,
                        double sy, Grid g, int C) {
  const size_t per = (size_t)C * g.H * g.W;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)g.NI * per) return;
  const int img = (int)(t / per);
  double fa = sx * (ax ? ax[img] : 1.0);
  cpx<R> r = x ? x[t] * (R)fa : mk<R>(0, 0);
  if (y) {
    double fb = sy * (by ? by[img] : 1.0);
    r = r + y[t] * (R)fb;
  }
  out[t] = r;
}

// "total" normalisation factor of each image: |clamp(i1 / i2, -1, 1)| with i2 =
// ik / hw the real-space total of a k-space grid sum ik; a zero i2 gives 0
// (normalize_field_total, dtmm/transfer.py:123-132); written over ik
__global__ void k_total_fact(const double* i1, double* ik, double hw, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double i2 = ik[t] / hw;
  double f = i2 == 0.0 ? 0.0 : i1[t] / i2;
  if (f <= -1.0) f = -1.0;
  if (f >= 1.0) f = 1.0;
  ik[t] = fabs(f);
}

// k-space: f <- notch * fact[image] * f (one thread per (lam, k), the notch
// once for every image of the wavelength)
template <typename R>
__global__ void k_kscale(cpx<R>* __restrict__ f, const double* fact, Grid g, NotchParams nt) {
  const int HW = g.H * g.W;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)g.nlam * HW) return;
  const int lam = (int)(t / HW), k = (int)(t - (size_t)lam * HW);
  const int ky = k / g.W, kx = k - ky * g.W;
  const double notch = notch_k(nt, g, lam, ky, kx);
  const int per = g.nray * g.npol;
  for (int q = 0; q < per; ++q) {
    const size_t img = (size_t)q * g.nlam + lam;
    const R s = (R)((fact ? fact[img] : 1.0) * notch);
    for (int c = 0; c < 4; ++c) {
      cpx<R>& v = f[(img * 4 + c) * HW + k];
      v = v * s;
    }
  }
}

// per-image ratio a / b (the total-intensity rescale of odd passes)
__global__ void k_ratio(const double* a, const double* b, double* out, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = a[t] / b[t];
}

// copy between precisions / layouts: dst[image][c][..] = src[image][c_map[c]][..]
template <typename RD, typename RS>
__global__ void k_convert(cpx<RD>* dst, const cpx<RS>* src, size_t n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = mk<RD>(to_r<RD>((double)src[t].re), to_r<RD>((double)src[t].im));
}

// FFT twiddles exp(-2 pi i t / N) (FP64, then rounded) and digit reversal
template <typename R>
__global__ void k_fft_tables(FFTPlan plan, cpx<R>* tw, int* perm) {
  const int n = plan.n;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)t / (double)n, &s, &c);
    tw[t] = mk<R>((R)c, (R)s);
    int m = t, pos = 0, stride = n;
    for (int q = plan.nr - 1; q >= 0; --q) {
      stride /= plan.r[q];
      pos += (m % plan.r[q]) * stride;
      m /= plan.r[q];
    }
    perm[t] = pos;
  }
}

// isotropic effective medium: mean over every voxel of (e0 + e1 + e2) / 3
// (effective_block with symmetry 0, dtmm/data.py:1364-1392), FP64
__global__ void k_eps_mean(const void* epsv, int eps_complex, long long s0, long long s1, long long s2, int L, int H,
                           int W, double* part) {
  const long long n = (long long)L * H * W;
  double sr = 0.0, si = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(t / ((long long)H * W));
    const long long r = t - (long long)l * H * W;
    const int y = (int)(r / W), x = (int)(r - (long long)y * W);
    const long long o = l * s0 + y * s1 + x * s2;
    if (eps_complex) {
      const cpx<double>* e = (const cpx<double>*)epsv + o;
      sr += (e[0].re + e[1].re + e[2].re) / 3.0;
      si += (e[0].im + e[1].im + e[2].im) / 3.0;
    } else {
      const double* e = (const double*)epsv + o;
      sr += (e[0] + e[1] + e[2]) / 3.0;
    }
  }
  __shared__ double red[2][256];
  red[0][threadIdx.x] = sr;
  red[1][threadIdx.x] = si;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      red[0][threadIdx.x] += red[0][threadIdx.x + st];
      red[1][threadIdx.x] += red[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x * 2 + 0] = red[0][0];
    part[blockIdx.x * 2 + 1] = red[1][0];
  }
}

// fixed-order sum of the block partials -> mean (re, im): one block of 256
// threads, each adding a fixed strided subset, then a tree
__global__ void k_eps_final(const double* part, int blocks, long long n, double* out) {
  double sr = 0, si = 0;
  for (int b = threadIdx.x; b < blocks; b += blockDim.x) {
    sr += part[2 * b];
    si += part[2 * b + 1];
  }
  __shared__ double red[2][256];
  red[0][threadIdx.x] = sr;
  red[1][threadIdx.x] = si;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      red[0][threadIdx.x] += red[0][threadIdx.x + st];
      red[1][threadIdx.x] += red[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = red[0][0] / (double)n;
    out[1] = red[1][0] / (double)n;
  }
}

// sqrt(eps_eff - beta_w^2) per window (real path)
// per (ray, window): a_w = sqrt(eps_eff - beta^2); with one real eps for
// every voxel (e0 = its first voxel) also eps11 - beta^2, its square root and
// eps11 (eps11 - beta^2 + delta), the window constants of the real-path solve
__global__ void k_window_aw(const double* wbeta, const double* eps_eff, double* aw, int n, const double* e0,
                            double* ev02, double* evs, double* c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  aw[i] = sqrt(eps_eff[0] - wbeta[i] * wbeta[i]);
  if (e0 != nullptr) {
    const double v = e0[0] - wbeta[i] * wbeta[i];
    ev02[i] = v;
    evs[i] = sqrt(v);
    c2[i] = e0[0] * (v + (e0[2] - e0[0]));
  }
}

// Per-call host scalars travel as kernel arguments (captured by value in a
// CUDA graph), 64 at a time.
struct Scalars64 {
  double v[64];
  int n, off;
};
__global__ void k_set_scalars(Scalars64 s, double* dst) {
  const int i = threadIdx.x;
  if (i < s.n) dst[s.off + i] = s.v[i];
}

// Partial sums of the voxels' lab-frame dielectric tensors R diag(epsv) R^T
// (dtmm/data.py:515-533; R = R_z(phi) R_y(theta) R_z(psi) of the voxel's
// Euler angles, dtmm/rotation.py:125-150) as (00, 11, 22, 01, 02, 12), re
// and im: 12 doubles per block
__global__ void k_eps_tensor_mean(const void* epsv, const double* epsa, int eps_complex, long long s0, long long s1,
                                  long long s2, long long a0, long long a1, long long a2, int L, int H, int W,
                                  double* part) {
  const long long n = (long long)L * H * W;
  double acc[12];
  for (int c = 0; c < 12; ++c) acc[c] = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(t / ((long long)H * W));
    const long long r = t - (long long)l * H * W;
    const int y = (int)(r / W), x = (int)(r - (long long)y * W);
    const long long o = l * s0 + y * s1 + x * s2;
    double er[3], ei[3] = {0.0, 0.0, 0.0};
    if (eps_complex) {
      const cpx<double>* e = (const cpx<double>*)epsv + o;
      for (int k = 0; k < 3; ++k) {
        er[k] = e[k].re;
        ei[k] = e[k].im;
      }
    } else {
      const double* e = (const double*)epsv + o;
      for (int k = 0; k < 3; ++k) er[k] = e[k];
    }
    const double* a = epsa + (l * a0 + y * a1 + x * a2);
    double sps, cps, st, ct, sp, cp;
    sincos(a[0], &sps, &cps);
    sincos(a[1], &st, &ct);
    sincos(a[2], &sp, &cp);
    double R[3][3];
    R[0][0] = ct * (cp * cps) - sp * sps;
    R[0][1] = -ct * (cp * sps) - sp * cps;
    R[0][2] = cp * st;
    R[1][0] = ct * (sp * cps) + cp * sps;
    R[1][1] = cp * cps - ct * (sp * sps);
    R[1][2] = st * sp;
    R[2][0] = -cps * st;
    R[2][1] = st * sps;
    R[2][2] = ct;
    const int pi[6] = {0, 1, 2, 0, 0, 1}, pj[6] = {0, 1, 2, 1, 2, 2};
    for (int c = 0; c < 6; ++c) {
      double vr = 0.0, vi = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double w = R[pi[c]][k] * R[pj[c]][k];
        vr += er[k] * w;
        vi += ei[k] * w;
      }
      acc[2 * c] += vr;
      acc[2 * c + 1] += vi;
    }
  }
  __shared__ double red[12][256];
  for (int c = 0; c < 12; ++c) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int c = 0; c < 12; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 12) part[blockIdx.x * 12 + threadIdx.x] = red[threadIdx.x][0];
}

// fixed-order sum of the tensor partials -> the mean tensor (12 doubles)
__global__ void k_eps_tensor_final(const double* part, int blocks, long long n, double* out) {
  if (threadIdx.x >= 12) return;
  double s = 0.0;
  for (int b = 0; b < blocks; ++b) s += part[b * 12 + threadIdx.x];
  out[threadIdx.x] = s / (double)n;
}

// cos, sin of the beam azimuths (one window per ray)
__global__ void k_sincos(const double* phi, double* c, double* sn, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sincos(phi[i], sn + i, c + i);
}

// ---------------------------------------------------------------------------
// Plane-wave input fields (the grid of illumination_data, dtmm/field.py:586):
// out[i][c][y][x] = coef[i][c] * ex[x] * ey[y] * window[y][x] with
//   FFT modes (k_planewave):  ex = exp(2 pi i mx x / W), ey = exp(2 pi i my y / H)
//                             (integer phase numerators reduced exactly, so
//                             sincospi sees an argument in [0, 2));
//   continuous (k_wave_window): ex = exp(i kx x), ey = exp(i ky y), the plane
//                             wave of dtmm/wave.py:376 normalised to 1 at the
//                             first pixel, times an optional real window.
// A block fills `rows` rows of one image: the W + rows phase factors are
// formed once in FP64 into shared memory (in the bulk precision), so the
// per-pixel work is complex products in R.
// ---------------------------------------------------------------------------
constexpr int kWaveRows = 8;

template <typename R>
__device__ __forceinline__ void wave_rows(cpx<R>* __restrict__ o, const cpx<R>* ex, const cpx<R>* ey,
                                          const cpx<R> c[4], const double* __restrict__ window, int y0, int ny,
                                          int W, long long HW) {
  for (int t = threadIdx.x; t < ny * W; t += blockDim.x) {
    const int r = t / W, x = t - r * W;
    const long long p = (long long)(y0 + r) * W + x;
    cpx<R> w = ex[x] * ey[r];
    if (window) w = w * to_r<R>(window[p]);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k * HW + p] = c[k] * w;
  }
}

template <typename R>
__global__ void k_planewave(cpx<R>* __restrict__ out, const cpx<double>* __restrict__ coef,
                            const int* __restrict__ my, const int* __restrict__ mx, int H, int W) {
  extern __shared__ __align__(16) unsigned char wave_smem[];
  cpx<R>* ex = (cpx<R>*)wave_smem;
  cpx<R>* ey = ex + W;
  const int img = blockIdx.y;
  const int y0 = blockIdx.x * kWaveRows, ny = min(kWaveRows, H - y0);
  const long long HW = (long long)H * W;
  const long long iy = ((long long)my[img] % H + H) % H, ix = ((long long)mx[img] % W + W) % W;
  for (int x = threadIdx.x; x < W; x += blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)((ix * x) % W) / (double)W, &s, &c);
    ex[x] = mk<R>(to_r<R>(c), to_r<R>(s));
  }
  for (int r = threadIdx.x; r < ny; r += blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)((iy * (y0 + r)) % H) / (double)H, &s, &c);
    ey[r] = mk<R>(to_r<R>(c), to_r<R>(s));
  }
  cpx<R> c[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) c[k] = cvt<R>(coef[(size_t)img * 4 + k]);
  __syncthreads();
  wave_rows<R>(out + (size_t)img * 4 * HW, ex, ey, c, nullptr, y0, ny, W, HW);
}

template <typename R>
__global__ void k_wave_window(cpx<R>* __restrict__ out, const cpx<double>* __restrict__ coef,
                              const double* __restrict__ kx, const double* __restrict__ ky,
                              const double* __restrict__ window, int H, int W) {
  extern __shared__ __align__(16) unsigned char wave_smem[];
  cpx<R>* ex = (cpx<R>*)wave_smem;
  cpx<R>* ey = ex + W;
  const int img = blockIdx.y;
  const int y0 = blockIdx.x * kWaveRows, ny = min(kWaveRows, H - y0);
  const long long HW = (long long)H * W;
  const double kxi = kx[img], kyi = ky[img];
  for (int x = threadIdx.x; x < W; x += blockDim.x) {
    double s, c;
    sincos(kxi * (double)x, &s, &c);
    ex[x] = mk<R>(to_r<R>(c), to_r<R>(s));
  }
  for (int r = threadIdx.x; r < ny; r += blockDim.x) {
    double s, c;
    sincos(kyi * (double)(y0 + r), &s, &c);
    ey[r] = mk<R>(to_r<R>(c), to_r<R>(s));
  }
  cpx<R> c[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) c[k] = cvt<R>(coef[(size_t)img * 4 + k]);
  __syncthreads();
  wave_rows<R>(out + (size_t)img * 4 * HW, ex, ey, c, window, y0, ny, W, HW);
}

// Field diffraction matrix of a homogeneous isotropic medium eps over d
// pixels (field_diffraction_matrix, dtmm/diffract.py:125-138):
// F . diag(exp(i alpha_m k0 d)) . F^-1 per grid k, over both directions
// (mode 0), the forward modes 0, 2 (+1) or the backward modes 1, 3 (-1);
// zero where beta >= betamax.  out[lam][ky][kx][4][4] in complex128, for
// wavelengths lam0 .. lam0 + kc.n - 1 (wavenumbers passed by value).
struct KsChunk {
  double ks[64];
  int n;
};

__global__ void k_field_dmat(KsChunk kc, int lam0, Grid g, cpx<double> eps, double d, int mode, double betamax,
                             cpx<double>* __restrict__ out) {
  const int HW = g.H * g.W;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= kc.n * HW) return;
  const int l = t / HW, k = t - l * HW;
  const int ky = k / g.W, kx = k - ky * g.W;
  const double ks = kc.ks[l];
  double beta, phi;
  betaphi_k(g, ks, ky, kx, beta, phi);
  cpx<double> al[4], F[4][4], Fi[4][4];
  iso_k(beta, phi, eps, betamax, al, F, Fi);
  cpx<double> ph[4];
  for (int m = 0; m < 4; ++m) {
    const bool keep = mode == 0 || (mode > 0 ? (m % 2 == 0) : (m % 2 == 1));
    ph[m] = keep ? cexp_i(al[m] * (ks * d)) : mk<double>(0.0, 0.0);
  }
  cpx<double>* o = out + ((size_t)(lam0 + l) * HW + k) * 16;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      cpx<double> acc = mk<double>(0.0, 0.0);
      for (int m = 0; m < 4; ++m) acc = acc + F[i][m] * ph[m] * Fi[m][j];
      o[i * 4 + j] = acc;
    }
}

// field[img] *= base[img] * sqrt(num[img] / den[img]) (num, den null: base only);
// the factor is formed once per block and applied in R
template <typename R>
__global__ void k_scale_fields(cpx<R>* __restrict__ f, long long per, const double* __restrict__ base,
                               const double* __restrict__ num, const double* __restrict__ den) {
  const int img = blockIdx.y;
  double fa = base ? base[img] : 1.0;
  if (num && den) fa *= sqrt(num[img] / den[img]);
  const R s = to_r<R>(fa);
  cpx<R>* o = f + (size_t)img * per;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < per; t += (long long)gridDim.x * blockDim.x)
    o[t] = o[t] * s;
}
}  // namespace dtmm
