// Types and helpers of a layer step shared by every kernel family: the
// image grid, the row / column pass parameters and the per-voxel operator
// application.
//
// Data layout in HBM
//   field / state arrays : [image][component][H][W] interleaved complex,
//                          image = (ray * npol + pol) * nlam + lam
//                          (the reference's ([rays],[pols],lambda,4,H,W) order)
//   window-row buffers   : [j][image][component][H][W]
//   layer operators      : [ray][window][H][W][record], 6 records per mode
//                          block (forward, then backward with both blocks)
#pragma once

#include "dtmm_common.cuh"

namespace dtmm {

// Records of one per-voxel layer operator, per mode block (forward modes 0,
// 2; backward 1, 3): the 2x2 block E of the block's E rows with its first
// column scaled by the scale of the pass over det(E), and the two phase
// arguments, (e0 s, e1, e2 s, e3, arg0, arg1) with s = scale / det(E).
// E' = E diag(s, 1) has det(E') = scale, so E' diag(p) adj(E') = scale E
// diag(p) E^-1.  A voxel keeps its records next to each other (REC_BLOCK
// or 2 REC_BLOCK of them), so they are read with vector loads.
constexpr int REC_BLOCK = 6;
constexpr int OP_REC = 2 * REC_BLOCK;  // records of both blocks

enum KOp { KOP_NONE = 0, KOP_DIAG = 1, KOP_MAT = 2 };

struct Grid {
  int H, W;       // grid
  int NI;         // images
  int nlam, npol, nray;
};

__device__ __forceinline__ int img_lam(const Grid& g, int img) { return img % g.nlam; }
__device__ __forceinline__ int img_ray(const Grid& g, int img) { return img / (g.nlam * g.npol); }

// fftfreq(n)[i] * n
__host__ __device__ __forceinline__ int fsigned(int i, int n) { return (i < (n + 1) / 2) ? i : i - n; }

// |beta_x| of FFT column x is below betamax: the same expression as the
// k-space tables' cut test at ky = 0 (the smallest beta of the column;
// correctly rounded operations only, so host and device agree)
__host__ __device__ inline bool in_band(int x, int n, double ks, double betamax) {
  const double xx = (double)fsigned(x, n) * (1.0 / n);
  return (2.0 * M_PI / fabs(ks)) * sqrt(xx * xx + 0.0 * 0.0) < betamax;
}

// largest |fsigned| index of an n-point axis inside the band (-1: none);
// formed on the host once per wavelength
__host__ __device__ inline int band_limit(int n, double ks, double betamax) {
  int lim = -1;
  for (int i = 0; i <= n / 2; ++i) {
    if (!in_band(i, n, ks, betamax)) break;
    lim = i;
  }
  return lim;
}

// ---------------------------------------------------------------------------
// Column pass of one layer step (all along ky, a tile of columns of one
// image): forward column FFT -> k-space operator -> for each window row j:
// cy_j * (.) -> inverse column FFT (scaled) -> U_j.
// Input X: [image][cin][H][W] (rows already transformed along x).
// ---------------------------------------------------------------------------
struct ColParams {
  int cin, cout;
  int kop;                 // KOp
  size_t ktab_ray_stride;  // elements between the tables of consecutive rays (0 = shared)
  const void* ktab;        // KOP_DIAG: [lam][H][W][2]; KOP_MAT: [lam][H][W][cout][cin]
  // band skip (register column pass, KOP_DIAG): the diagonal operator is zero
  // for beta >= betamax, so a tile whose columns all have |beta_x| >= betamax
  // at the image's wavelength produces zeros without any transform.
  // 1: such tiles write zeros; 2: they write nothing (the register row pass
  // reads those columns as zero without loading them)
  int band_skip;
  const double* blim;      // [lam] band limit: largest in-band |column frequency index| (-1: none)
  int tile_lo, tile_hi0;   // register column pass with band_skip 2: launched tiles [0, tile_lo) and
                           // tile_hi0 on (tile_lo 0: every tile)
  int ny;                  // window rows (1 = no windows)
  const void* cy;          // [ray][j][lam][H] (null = weight 1)
  int j_only;              // >= 0: emit only window row j_only (into U slot 0)
  int cy_rows;             // window rows in the cy table (ray stride = cy_rows * nlam * H)
  int do_fwd;              // 1: transform along y first (input spatial in y)
  int inverse_out;         // 1: inverse column FFT on the way out
  double out_scale;
  FFTPlan plan;
  const void* tw;          // twiddles of H
  const int* perm;         // digit reversal of H
  int tc;                  // columns per block
};

// ---------------------------------------------------------------------------
// Row pass of one layer step, one row y of a group of wavelengths and
// polarisations of one ray: for each window (i, j): cx_i * U_j -> inverse row
// FFT -> per-voxel operator of window (i, j) -> accumulate; then forward row
// FFT -> X.
// ---------------------------------------------------------------------------
struct RowParams {
  int C;                 // 4 (Epn) or 2 (E)
  const double* blim;    // [lam] band limit: columns with |frequency index| > limit read as zero
  int nx, ny;            // windows per axis (1, 1 without windows)
  const void* cx;        // [ray][i][lam][W] (null = weight 1)
  const int* wzero;      // [ray][nx*ny]
  const void* op;        // [ray][win][H][W][rec_stride] (offset to the block the pass uses)
  int rec_stride;        // records per voxel: REC_BLOCK, or OP_REC with both blocks
  const double* ks;      // [lam]
  double dir;            // propagation direction (+1 / -1)
  double in_scale;       // 1/W of the inverse row transform (and 1/H of the column one)
  FFTPlan plan;
  const void* tw;
  const int* perm;
  int G;                 // wavelengths per block
  int PB;                // polarisations per block
  int win_only;          // >= 0: only this window (its own sub-step chain), -1: all
  int use_cx;            // apply the window's beta_x weight (first sub-step of a chain)
  int accumulate;        // add the result to X instead of overwriting it
  int groups_inner;      // register row pass: blockIdx.x the group, blockIdx.y the row (else the reverse)
  int xr;                // register row pass variant with accumulators in registers, pixels a thread (0: none)
};

template <typename R>
__device__ __forceinline__ cpx<R> phase_of(cpx<R> arg, R k) {
  return cexp_i(mk<R>(arg.re * k, arg.im * k));
}
// exp(i arg k) of a real phase.  complex64 bulk: Cody-Waite reduction of
// x = arg k by 2 pi (2 pi split into a float head and tail) to |r| <= pi, then
// the SFU sine / cosine, whose absolute error there is about 4e-7; phase
// arguments of one layer step are small, so the reduction is exact in
// practice.  complex128 bulk: the FP64 library sincos.
template <typename R>
__device__ __forceinline__ cpx<R> phase_of(R arg, R k) {
  if constexpr (sizeof(R) == 4) {
    const float x = arg * k;
    const float q = rintf(x * 0.159154943f);  // x / (2 pi)
    float r = fmaf(-q, 6.28318548f, x);       // float(2 pi)
    r = fmaf(-q, -1.74845553e-7f, r);         // 2 pi - float(2 pi)
    float s, c;
    __sincosf(r, &s, &c);
    return mk<R>(c, s);
  } else {
    R s, c;
    sincos(arg * k, &s, &c);
    return mk<R>(c, s);
  }
}

// the n records of one voxel, in 16-byte loads when n records fill whole
// 16-byte words (every voxel's records then start on a 16-byte boundary),
// else in 8-byte loads (six FP32 records: 8-byte boundaries)
template <int N, typename T>
__device__ __forceinline__ void load_recs(const T* __restrict__ src, T (&r)[N]) {
  constexpr int B = N * (int)sizeof(T);
  if constexpr (B % 16 == 0) {
    union {
      float4 v[B / 16];
      T t[N];
    } u;
#pragma unroll
    for (int i = 0; i < B / 16; ++i) u.v[i] = ((const float4*)src)[i];
#pragma unroll
    for (int i = 0; i < N; ++i) r[i] = u.t[i];
  } else {
    static_assert(B % 8 == 0, "records fill 8-byte words");
    union {
      float2 v[B / 8];
      T t[N];
    } u;
#pragma unroll
    for (int i = 0; i < B / 8; ++i) u.v[i] = ((const float2*)src)[i];
#pragma unroll
    for (int i = 0; i < N; ++i) r[i] = u.t[i];
  }
}

template <int N, typename T>
__device__ __forceinline__ void store_recs(T* __restrict__ dst, const T (&r)[N]) {
  constexpr int B = N * (int)sizeof(T);
  if constexpr (B % 16 == 0) {
    union {
      float4 v[B / 16];
      T t[N];
    } u;
#pragma unroll
    for (int i = 0; i < N; ++i) u.t[i] = r[i];
#pragma unroll
    for (int i = 0; i < B / 16; ++i) ((float4*)dst)[i] = u.v[i];
  } else {
    static_assert(B % 8 == 0, "records fill 8-byte words");
    union {
      float2 v[B / 8];
      T t[N];
    } u;
#pragma unroll
    for (int i = 0; i < N; ++i) u.t[i] = r[i];
#pragma unroll
    for (int i = 0; i < B / 8; ++i) ((float2*)dst)[i] = u.v[i];
  }
}

// one 2x2 block of the per-voxel operator, out += E' diag(p0, p1) adj(E') h
// (E' the block's records, first column carrying scale / det, so det(E') =
// scale), in projector form: with c0 = (e0', e2') and r0 = (e3, -e1),
// E' diag(p0, p1) adj(E') = p1 scale I + (p0 - p1) c0 r0.  The caller forms
// q = p1 scale and dp = p0 - p1 once per voxel and wavelength.
template <typename R, typename T>
__device__ __forceinline__ void apply_block(const T e[4], cpx<R> q, cpx<R> dp, cpx<R> h0, cpx<R> h1, cpx<R>& a0,
                                            cpx<R>& a1) {
  const cpx<R> s = (e[3] * h0 - e[1] * h1) * dp;
  a0 = cfma(q, h0, a0) + e[0] * s;
  a1 = cfma(q, h1, a1) + e[2] * s;
}

}  // namespace dtmm
