// Row and column passes of a layer step with register line transforms
// (complex64 bulk, every side N = N1 * N2 that `reg_lanes` lists).
//
// Each (image, component) line is transformed by a group of N1 lanes
// (`TwoStep`); the groups synchronise with their own lane mask, so a warp may
// hold lines of different activity.  Work per block:
//   row pass     one row y of G wavelengths x PB polarisations of one ray:
//                for each window, the weighted row is inverse-transformed into
//                the line's row buffer, the per-voxel operator accumulates into
//                the line's accumulator, and the accumulator is transformed
//                forward and stored (natural order throughout);
//   column pass  TX columns x C components of one image: coalesced row loads
//                into a tile, forward column transforms, the diagonal k-space
//                operator, then per window row j: spectra * cy_j -> inverse
//                transform -> coalesced row stores.  With N2 % N1 == 0 the
//                spectra stay in registers and one tile serves as loads,
//                exchange and stores; otherwise they stay in tile A and the
//                exchange uses tile B (A itself for a single window row).
//
// The kernels are instantiated per side in separate translation units
// (dtmm_reg_*.cu) through DTMM_REG_DEFINE; the engine reaches them through the
// row_reg_<N> / col_reg_<N> functions declared at the end.
#pragma once

#include <type_traits>

#include "dtmm_layer.cuh"
#include "dtmm_regfft.cuh"

namespace dtmm {

// lanes [g * N1, g * N1 + N1) of the calling lane's group
template <int N1>
__device__ __forceinline__ unsigned group_mask() {
  if constexpr (N1 >= 32) {
    return 0xffffffffu;
  } else {
    const unsigned lane = threadIdx.x & 31u;
    return ((1u << N1) - 1u) << (lane & ~(unsigned)(N1 - 1));
  }
}

// row buffer stride (complex elements): with N1 = 4 or 8 several line groups
// share a half-warp, and a stride of W + 4 (W + 8) puts their exchange slots
// on disjoint banks; W is a multiple of 16 for every listed side
// wavelengths per row block at most (the engine caps row_group here)
constexpr int kMaxRowGroup = 64;

__host__ __device__ constexpr int reg_row_stride(int n1, int w) { return n1 == 4 ? w + 4 : (n1 == 8 ? w + 8 : w); }

// Band variants of the row pass.  The window rows arrive band-limited: every
// entry with |f_x| beyond the wavelength's band limit lim is zero.  Variant
// b > 0 loads only the entries m < KB and m >= N2 - KB of a lane (KB =
// row_band_slots) and runs the sparse step-1 DFT; it is exact when every
// wavelength of the launch has lim < KB N1 (the other entries then lie
// beyond the band: t + N1 m >= N1 KB for m >= KB on the positive side,
// W - (t + N1 m) > N1 KB for m < N2 - KB on the negative side).
__host__ __device__ constexpr int row_band_slots(int n2, int b) {
  return b == 0 ? 0 : ((b == 1 ? n2 / 8 : n2 / 4) > 1 ? (b == 1 ? n2 / 8 : n2 / 4) : 1);
}
__host__ __device__ constexpr bool row_band_ok(int n2, int b) { return b == 0 || 2 * row_band_slots(n2, b) < n2; }

// largest block of the register row pass for an n-point row (its launch bounds)
__host__ __device__ constexpr int reg_row_max_threads(int n) {
  return reg_lanes(n) > 0 && n / reg_lanes(n) >= 32 ? 512 : 256;
}

// the band variant of an n-point row for the largest band limit of a launch
__host__ __device__ constexpr int row_band_pick(int n, int lim) {
  const int n1 = reg_lanes(n), n2 = n1 > 0 ? n / n1 : 0;
  for (int b = 1; b <= 2; ++b)
    if (n1 > 0 && row_band_ok(n2, b) && lim < row_band_slots(n2, b) * n1) return b;
  return 0;
}

// Launch bounds: rows of up to 16 points per lane run at most 256 threads a
// block and keep at most 85 registers, so that six 128-thread blocks share an
// SM (measured 8 % faster than four at 117 registers for 256-point rows);
// 32 points per lane need the registers of a whole 512-thread block.
// XR > 0: the block holds exactly kXrLines lines (two images of the 4x4
// method) and W / XR threads, and each thread keeps the accumulators of its
// XR pixels in registers across the windows (no shared-memory
// read-modify-write per window); 128 registers a thread at most.
constexpr int kXrLines = 8;
template <typename R, int C, bool REAL, int N1, int N2, int BAND, int XR = 0>
__global__ void __launch_bounds__(XR > 0 ? (N1 * N2) / (XR > 0 ? XR : 1) : (N2 >= 32 ? 512 : 256),
                                  XR > 0 ? 4 : (N2 >= 32 ? 1 : 3))
    k_layer_row_reg(RowParams p, Grid g, const cpx<R>* __restrict__ U, cpx<R>* __restrict__ X) {
  static_assert(XR == 0 || C == 4, "register accumulators: the 4x4 method's two-image blocks");
  using T = typename std::conditional<REAL, R, cpx<R>>::type;
  using TS = TwoStep<N1, N2>;
  constexpr int W = N1 * N2;
  constexpr int LS = reg_row_stride(N1, W);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int H = g.H;
  const int ngrp = (g.nlam + p.G - 1) / p.G;
  const int npg = (g.npol + p.PB - 1) / p.PB;
  // groups_inner: the groups of one row are neighbours in the launch order,
  // so that the row's operator records (shared by every wavelength and
  // polarisation) come from HBM once and from L2 for the other groups
  const int y = p.groups_inner ? blockIdx.y : blockIdx.x;
  const int gi = p.groups_inner ? blockIdx.x : blockIdx.y;
  const int pg = gi % npg, rg = gi / npg;
  const int ray = rg / ngrp, grp = rg - ray * ngrp;
  const int lam0 = grp * p.G, pol0 = pg * p.PB;
  const int G = min(p.G, g.nlam - lam0);
  const int NP = min(p.PB, g.npol - pol0);  // polarisations of this block
  const int nlines = G * NP * C;
  cpx<R>* acc = (cpx<R>*)smem_raw;                  // [lines][LS]
  cpx<R>* tmp = acc + (size_t)p.G * p.PB * C * LS;  // [lines][LS] exchange and transformed rows
  cpx<R>* tw = tmp + (size_t)p.G * p.PB * C * LS;   // [W]  twiddles, lane-major (TwoStep::twiddle_entry)
  const int HW = H * W;
  const int nwin = p.nx * p.ny;
  for (int e = threadIdx.x; e < W; e += blockDim.x) tw[e] = TS::twiddle_entry((const cpx<R>*)p.tw, e);
  if (XR == 0)
    for (int e = threadIdx.x; e < nlines * LS; e += blockDim.x) acc[e] = mk<R>(0, 0);
  cpx<R> racc[XR > 0 ? XR : 1][kXrLines];
  if (XR > 0) {
#pragma unroll
    for (int k = 0; k < (XR > 0 ? XR : 1); ++k)
#pragma unroll
      for (int l = 0; l < kXrLines; ++l) racc[k][l] = mk<R>((R)0, (R)0);
  }
  // phase scale k0 * direction of each wavelength of the block (formed once, in FP64)
  __shared__ R s_kph[kMaxRowGroup];
  __shared__ int s_lim[kMaxRowGroup];  // band limit of each wavelength (columns beyond read as zero)
  for (int g2 = threadIdx.x; g2 < G; g2 += blockDim.x) {
    s_kph[g2] = (R)(p.ks[lam0 + g2] * p.dir);
    s_lim[g2] = (int)p.blim[lam0 + g2];
  }
  const R sc = (R)p.in_scale;  // det of each block's records
  __syncthreads();
  const int line = threadIdx.x / N1, t = threadIdx.x % N1;
  const bool active = line < nlines;
  const unsigned gm = group_mask<N1>();
  // the lane's twiddles W_N^(t k1) in registers when they are few
  constexpr bool TWREG = N2 <= 8;
  cpx<R> trow[TWREG ? N2 : 1];
  if (TWREG) {
#pragma unroll
    for (int k1 = 0; k1 < (TWREG ? N2 : 1); ++k1) trow[k1] = tw[k1 * N1 + t];
  }
  const int c = line % C, im = line / C;
  const int gl = im / NP, pol = pol0 + im - gl * NP;
  const int lam = lam0 + gl;
  const int img = (ray * g.npol + pol) * g.nlam + lam;
  cpx<R>* xl = tmp + (size_t)line * LS;
  for (int j = 0; j < p.ny; ++j) {
    // a single-window chain reads the one window row the column pass emitted
    const cpx<R>* Uj = U + (size_t)(p.win_only >= 0 ? 0 : j) * g.NI * C * HW;
    for (int i = 0; i < p.nx; ++i) {
      const int w = i * p.ny + j;
      if (p.win_only >= 0 && w != p.win_only) continue;
      if (p.wzero != nullptr && p.wzero[ray * nwin + w]) continue;
      if (active) {
        const cpx<R>* src = Uj + (((size_t)img * C + c) * H + y) * W;
        const R* cxl = (p.cx && p.use_cx) ? (const R*)p.cx + (((size_t)ray * p.nx + i) * g.nlam + lam) * W : nullptr;
        cpx<R> v[N2];
        const int lim = s_lim[gl];
        constexpr int KB = row_band_slots(N2, BAND);
#pragma unroll
        for (int m = 0; m < N2; ++m) {
          if (BAND == 0 || m < KB || m >= N2 - KB) {
            const int xk = t + N1 * m;
            const int fx = xk < (W + 1) / 2 ? xk : W - xk;  // |fsigned(xk)|
            cpx<R> a = fx <= lim ? src[xk] : mk<R>((R)0, (R)0);
            v[m] = cxl ? a * cxl[xk] : a;
          } else {
            v[m] = mk<R>((R)0, (R)0);
          }
        }
        TS::template step1<R, true, BAND == 0 ? full_mask(N2) : band_mask(N2, KB)>(v, xl, 1, TWREG ? trow : nullptr,
                                                                                    tw, t);
        __syncwarp(gm);
        cpx<R> u[TS::J][N1];
        TS::template step2<R, true>(u, xl, 1, t);
        __syncwarp(gm);  // every read of the exchange precedes the results that overwrite it
        TS::template store<R>(u, xl, 1, t);  // the 1/W of the inverse rides on the operator's 1/det
      }
      __syncthreads();
      const int rs = p.rec_stride;
      const T* opw = (const T*)p.op + (((size_t)ray * nwin + w) * HW + (size_t)y * W) * rs;
      // XU pixels per thread and round: their records are loaded together, so
      // that several rounds of global loads are in flight (long rows hold
      // few blocks per SM)
      constexpr int XU = (C == 2 && N2 >= 32) ? 4 : 1;
      constexpr int NR = C == 4 ? OP_REC : REC_BLOCK;  // records this pass reads per voxel
      if constexpr (XR > 0) {
        // pixels threadIdx.x + k W / XR; the block's two images b (G = 1 and
        // two polarisations share the phases, G = 2 has its own per image)
#pragma unroll
        for (int k = 0; k < (XR > 0 ? XR : 1); ++k) {
          const int x = threadIdx.x + k * (W / (XR > 0 ? XR : 1));
          T rec[NR];
          load_recs<NR, T>(opw + (size_t)x * rs, rec);
          const T* ef = rec;
          const T* eb = rec + REC_BLOCK;
          cpx<R> qf, dpf, qb, dpb;
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            if (b == 0 || G == 2) {
              const R kph = s_kph[G == 2 ? b : 0];
              const cpx<R> f0 = phase_of(ef[4], kph), f1 = phase_of(ef[5], kph);
              qf = f1 * sc;
              dpf = f0 - f1;
              const cpx<R> b0 = phase_of(eb[4], kph), b1 = phase_of(eb[5], kph);
              qb = b1 * sc;
              dpb = b0 - b1;
            }
            const cpx<R>* h = tmp + (size_t)(4 * b) * LS + x;
            apply_block<R, T>(ef, qf, dpf, h[0], h[2 * LS], racc[k][4 * b], racc[k][4 * b + 2]);
            apply_block<R, T>(eb, qb, dpb, h[LS], h[3 * LS], racc[k][4 * b + 1], racc[k][4 * b + 3]);
          }
        }
        __syncthreads();
        continue;
      }
      for (int x0 = threadIdx.x; x0 < W; x0 += XU * blockDim.x) {
        T rec[XU][NR];
#pragma unroll
        for (int k = 0; k < XU; ++k) {
          const int x = x0 + k * blockDim.x;
          if (x >= W) break;
          load_recs<NR, T>(opw + (size_t)x * rs, rec[k]);
        }
#pragma unroll
        for (int k = 0; k < XU; ++k) {
          const int x = x0 + k * blockDim.x;
          if (x >= W) break;
          const T* ef = rec[k];
          const T* eb = rec[k] + (C == 4 ? REC_BLOCK : 0);
          for (int g2 = 0; g2 < G; ++g2) {
            const R kph = s_kph[g2];
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
            for (int q = 0; q < NP; ++q) {
              const int l0 = (g2 * NP + q) * C;
              const cpx<R>* h = tmp + (size_t)l0 * LS + x;
              cpx<R>* a = acc + (size_t)l0 * LS + x;
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
      }
      __syncthreads();
    }
  }
  if constexpr (XR > 0) {  // the accumulators into the rows of the forward transform
#pragma unroll
    for (int k = 0; k < (XR > 0 ? XR : 1); ++k)
#pragma unroll
      for (int l = 0; l < kXrLines; ++l) acc[(size_t)l * LS + threadIdx.x + k * (W / (XR > 0 ? XR : 1))] = racc[k][l];
    __syncthreads();
  }
  if (active) {
    cpx<R> v[N2];
    const cpx<R>* al = acc + (size_t)line * LS;
#pragma unroll
    for (int m = 0; m < N2; ++m) v[m] = al[t + N1 * m];
    TS::template step1<R, false>(v, xl, 1, TWREG ? trow : nullptr, tw, t);
    __syncwarp(gm);
    cpx<R> u[TS::J][N1];
    TS::template step2<R, false>(u, xl, 1, t);
    cpx<R>* dst = X + (((size_t)img * C + c) * H + y) * W;
    if constexpr (TS::EVEN) {
      TS::template to_lane_order<R>(u, v);
#pragma unroll
      for (int m = 0; m < N2; ++m) dst[t + N1 * m] = p.accumulate ? dst[t + N1 * m] + v[m] : v[m];
    } else {
      __syncwarp(gm);
      TS::template store<R>(u, xl, 1, t, (R)1);
      __syncwarp(gm);
#pragma unroll
      for (int m = 0; m < N2; ++m) {
        const cpx<R> r = xl[t + N1 * m];
        dst[t + N1 * m] = p.accumulate ? dst[t + N1 * m] + r : r;
      }
    }
  }
}

// Plain row FFT of `nlines` lines of N = N1 * N2 points, natural order in
// and out, src -> dst (the same array for in place: a line's group reads it
// completely before it writes), times `scale`; blockDim / N1 lines per block.
template <typename R, int N1, int N2, bool INV>
__global__ void __launch_bounds__(256) k_fft_rows_reg(const cpx<R>* src, cpx<R>* dst, int nlines,
                                                     const cpx<R>* __restrict__ twg, R scale) {
  using TS = TwoStep<N1, N2>;
  constexpr int W = N1 * N2;
  constexpr int LS = reg_row_stride(N1, W);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<R>* tw = (cpx<R>*)smem_raw;  // [W] twiddles, lane-major
  cpx<R>* xb = tw + W;             // [lines per block][LS] exchange
  for (int e = threadIdx.x; e < W; e += blockDim.x) tw[e] = TS::twiddle_entry(twg, e);
  __syncthreads();
  const int lpb = blockDim.x / N1;
  const int li = threadIdx.x / N1, t = threadIdx.x % N1;
  const int line = blockIdx.x * lpb + li;
  if (li >= lpb || line >= nlines) return;  // whole lane groups leave together
  const unsigned gm = group_mask<N1>();
  cpx<R>* xl = xb + (size_t)li * LS;
  const cpx<R>* in = src + (size_t)line * W;
  cpx<R>* out = dst + (size_t)line * W;
  cpx<R> v[N2];
#pragma unroll
  for (int m = 0; m < N2; ++m) v[m] = in[t + N1 * m];
  TS::template step1<R, INV>(v, xl, 1, nullptr, tw, t);
  __syncwarp(gm);
  cpx<R> u[TS::J][N1];
  TS::template step2<R, INV>(u, xl, 1, t);
  if constexpr (TS::EVEN) {
    TS::template to_lane_order<R>(u, v);
#pragma unroll
    for (int m = 0; m < N2; ++m) out[t + N1 * m] = v[m] * scale;
  } else {
    __syncwarp(gm);
    TS::template store<R>(u, xl, 1, t, scale);
    __syncwarp(gm);
#pragma unroll
    for (int m = 0; m < N2; ++m) out[t + N1 * m] = xl[t + N1 * m];
  }
}

// tiles of the column pass: N2 % N1 == 0 keeps the spectra in registers (one
// tile); otherwise the spectra stay in tile A and, with several window rows,
// the exchange needs tile B
__host__ __device__ constexpr bool reg_even(int n) { return reg_lanes(n) > 0 && (n / reg_lanes(n)) % reg_lanes(n) == 0; }
__host__ __device__ constexpr int reg_col_tiles(int n, int ny) { return (!reg_even(n) && ny > 1) ? 2 : 1; }

// Column pass, k-space operator KOP_NONE, KOP_DIAG or KOP_MAT (C x C per k,
// exchanged through the tile; see the file comment).  BAND > 0 (KOP_DIAG
// only, N2 % N1 == 0): the diagonal table is zero beyond betamax, so after it
// a lane's spectrum entries outside m < KB, m >= N2 - KB are exact zeros
// whenever the H axis's band limit is below KB N1; the window-row inverse
// transforms then weight only those entries and run the sparse step 1.
template <typename R, int N1, int N2, int BAND>
__global__ void __launch_bounds__(256, 3) k_layer_col_reg(ColParams p, Grid g, const cpx<R>* __restrict__ X,
                                                         cpx<R>* __restrict__ U) {
  using TS = TwoStep<N1, N2>;
  constexpr int H = N1 * N2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int W = g.W, TX = p.tc, C = p.cin;
  const int RS = C * TX + 1;                       // tile row stride (odd)
  const int ntiles = reg_col_tiles(H, p.ny);
  cpx<R>* tileA = (cpx<R>*)smem_raw;               // [H][RS] loaded rows, then spectra along y
  cpx<R>* tileB = tileA + (size_t)(ntiles - 1) * H * RS;  // [H][RS] exchange and outgoing rows (= A with one tile)
  cpx<R>* tw = tileA + (size_t)ntiles * H * RS;    // [H] twiddles, lane-major (TwoStep::twiddle_entry)
  const int img = blockIdx.y;
  // tile_lo > 0: the launch covers the in-band tiles only, tiles [0, tile_lo)
  // and from tile_hi0 on (the others write nothing with band_skip 2)
  const int tile = (p.tile_lo > 0 && (int)blockIdx.x >= p.tile_lo) ? p.tile_hi0 + ((int)blockIdx.x - p.tile_lo)
                                                                    : (int)blockIdx.x;
  const int x0 = tile * TX;
  const int lam = img_lam(g, img), ray = img_ray(g, img);
  const int CT = C * TX;
  const int lc = threadIdx.x % CT, ystep = blockDim.x / CT;
  const int lcc = lc / TX, lxc = lc - lcc * TX;
  const bool lin = (int)threadIdx.x < ystep * CT && x0 + lxc < W;
  if (p.band_skip && p.kop == KOP_DIAG) {
    const int lim = (int)p.blim[lam];
    bool any = false;
    for (int xc = 0; xc < TX && x0 + xc < W; ++xc) {
      const int xk = x0 + xc;
      any = any || (xk < (W + 1) / 2 ? xk : W - xk) <= lim;
    }
    if (!any) {  // the whole block leaves together
      if (p.band_skip == 1) {
        for (int jj = 0; jj < p.ny; ++jj) {
          cpx<R>* udst = U + (size_t)jj * g.NI * C * H * W + ((size_t)img * C + lcc) * H * W + x0 + lxc;
          if (lin)
            for (int y = threadIdx.x / CT; y < H; y += ystep) udst[(size_t)y * W] = mk<R>((R)0, (R)0);
        }
      }
      return;
    }
  }
  for (int e = threadIdx.x; e < H; e += blockDim.x) tw[e] = TS::twiddle_entry((const cpx<R>*)p.tw, e);
  const cpx<R>* xsrc = X + ((size_t)img * C + lcc) * H * W + x0 + lxc;
  if (lin)
    for (int y = threadIdx.x / CT; y < H; y += ystep) tileA[y * RS + lc] = xsrc[(size_t)y * W];
  __syncthreads();
  const int l = threadIdx.x / N1, t = threadIdx.x % N1;
  const int nlines = C * TX;
  const bool active = l < nlines;
  const unsigned gm = group_mask<N1>();
  const int c = l / TX, xc = l - c * TX;
  const int kx = x0 + xc;
  cpx<R>* colA = tileA + l;  // line element e at colA[e * RS]
  cpx<R>* colB = tileB + l;
  const bool diag = active && p.kop == KOP_DIAG && kx < W;
  const cpx<R>* ek = diag ? (const cpx<R>*)p.ktab + (((size_t)lam * W + kx) * H) * 2 + ((((c & 1) == 0) || C == 2) ? 0 : 1)
                          : nullptr;
  const R sc = (R)p.out_scale;
  if constexpr (TS::EVEN) {
    // spectra in registers, lane order v[m] = X[t + N1 m]
    cpx<R> v[N2];
    if (active) {
#pragma unroll
      for (int m = 0; m < N2; ++m) v[m] = colA[(t + N1 * m) * RS];
      __syncwarp(gm);
      if (p.do_fwd) {
        TS::template step1<R, false>(v, colA, RS, nullptr, tw, t);
        __syncwarp(gm);
        cpx<R> u[TS::J][N1];
        TS::template step2<R, false>(u, colA, RS, t);
        TS::template to_lane_order<R>(u, v);
      }
      if (diag) {
#pragma unroll
        for (int m = 0; m < N2; ++m) v[m] = v[m] * ek[(t + N1 * m) * 2];
      }
      // the output scale once on the spectrum, not on every window row's result
#pragma unroll
      for (int m = 0; m < N2; ++m) v[m] = v[m] * sc;
    }
    if (p.kop == KOP_MAT) {
      // C x C matrix per k across the components of a column: through tile A
      __syncthreads();  // every line's forward exchange is done with the tile
      if (active) {
#pragma unroll
        for (int m = 0; m < N2; ++m) colA[(t + N1 * m) * RS] = v[m];
      }
      __syncthreads();
      if (active && kx < W) {
        const cpx<R>* mt = (const cpx<R>*)p.ktab + ray * p.ktab_ray_stride + (((size_t)lam * H) * W + kx) * C * C + c * C;
#pragma unroll
        for (int m = 0; m < N2; ++m) {
          const int k = t + N1 * m;
          const cpx<R>* mrow = mt + (size_t)k * W * C * C;
          const cpx<R>* in = tileA + (size_t)k * RS + xc;
          cpx<R> acc = mk<R>((R)0, (R)0);
          for (int j = 0; j < C; ++j) acc = cfma(mrow[j], in[j * TX], acc);
          v[m] = acc;
        }
      }
    }
    for (int jj = 0; jj < p.ny; ++jj) {
      const int j = p.j_only >= 0 ? p.j_only : jj;
      __syncthreads();  // the previous window's stores (and the forward exchange) are done with the tile
      if (active) {
        const R* cyj = p.cy ? (const R*)p.cy + (((size_t)ray * p.cy_rows + j) * g.nlam + lam) * H : nullptr;
        constexpr int KB = row_band_slots(N2, BAND);
        cpx<R> w[N2];
#pragma unroll
        for (int m = 0; m < N2; ++m) {
          if (BAND == 0 || m < KB || m >= N2 - KB)
            w[m] = cyj ? v[m] * cyj[t + N1 * m] : v[m];
          else
            w[m] = mk<R>((R)0, (R)0);
        }
        if (p.inverse_out) {
          TS::template step1<R, true, BAND == 0 ? full_mask(N2) : band_mask(N2, KB)>(w, colA, RS, nullptr, tw, t);
          __syncwarp(gm);
          cpx<R> u[TS::J][N1];
          TS::template step2<R, true>(u, colA, RS, t);
          __syncwarp(gm);
          TS::template store<R>(u, colA, RS, t);
        } else {
#pragma unroll
          for (int m = 0; m < N2; ++m) colA[(t + N1 * m) * RS] = w[m];
        }
      }
      __syncthreads();
      cpx<R>* udst = U + (size_t)jj * g.NI * C * H * W + ((size_t)img * C + lcc) * H * W + x0 + lxc;
      if (lin)
        for (int y = threadIdx.x / CT; y < H; y += ystep) udst[(size_t)y * W] = tileA[y * RS + lc];
    }
  } else {
    // spectra in tile A (natural order); exchange in tile B (tile A itself
    // with one window row: the line is in registers before the exchange)
    if (active && p.do_fwd) {
      cpx<R> v[N2];
#pragma unroll
      for (int m = 0; m < N2; ++m) v[m] = colA[(t + N1 * m) * RS];
      __syncwarp(gm);
      TS::template step1<R, false>(v, colB, RS, nullptr, tw, t);
      __syncwarp(gm);
      cpx<R> u[TS::J][N1];
      TS::template step2<R, false>(u, colB, RS, t);
      __syncwarp(gm);
      TS::template store<R>(u, colA, RS, t, (R)1);
    }
    if (diag) {
      __syncwarp(gm);
#pragma unroll
      for (int m = 0; m < N2; ++m) {
        const int k = t + N1 * m;
        colA[k * RS] = colA[k * RS] * ek[k * 2];
      }
    }
    if (p.kop == KOP_MAT) {
      // C x C matrix per k across the components of a column, in tile A:
      // every thread reads its k's components, the block syncs, then writes
      __syncthreads();
      cpx<R> r[N2];
      if (active && kx < W) {
        const cpx<R>* mt = (const cpx<R>*)p.ktab + ray * p.ktab_ray_stride + (((size_t)lam * H) * W + kx) * C * C + c * C;
#pragma unroll
        for (int m = 0; m < N2; ++m) {
          const int k = t + N1 * m;
          const cpx<R>* mrow = mt + (size_t)k * W * C * C;
          const cpx<R>* in = tileA + (size_t)k * RS + xc;
          cpx<R> acc = mk<R>((R)0, (R)0);
          for (int j = 0; j < C; ++j) acc = cfma(mrow[j], in[j * TX], acc);
          r[m] = acc;
        }
      }
      __syncthreads();
      if (active && kx < W) {
#pragma unroll
        for (int m = 0; m < N2; ++m) colA[(t + N1 * m) * RS] = r[m];
      }
    }
    for (int jj = 0; jj < p.ny; ++jj) {
      const int j = p.j_only >= 0 ? p.j_only : jj;
      __syncthreads();  // tile A complete; the previous window's stores have read tile B
      if (active) {
        cpx<R> v[N2];
        const R* cyj = p.cy ? (const R*)p.cy + (((size_t)ray * p.cy_rows + j) * g.nlam + lam) * H : nullptr;
#pragma unroll
        for (int m = 0; m < N2; ++m) {
          const cpx<R> a = colA[(t + N1 * m) * RS];
          v[m] = cyj ? a * cyj[t + N1 * m] : a;
        }
        __syncwarp(gm);
        if (p.inverse_out) {
          TS::template step1<R, true>(v, colB, RS, nullptr, tw, t);
          __syncwarp(gm);
          cpx<R> u[TS::J][N1];
          TS::template step2<R, true>(u, colB, RS, t);
          __syncwarp(gm);
          TS::template store<R>(u, colB, RS, t, sc);
        } else {
#pragma unroll
          for (int m = 0; m < N2; ++m) colB[(t + N1 * m) * RS] = v[m] * sc;
        }
      }
      __syncthreads();
      cpx<R>* udst = U + (size_t)jj * g.NI * C * H * W + ((size_t)img * C + lcc) * H * W + x0 + lxc;
      if (lin)
        for (int y = threadIdx.x / CT; y < H; y += ystep) udst[(size_t)y * W] = tileB[y * RS + lc];
    }
  }
}

// ---------------------------------------------------------------------------
// launch glue: one function per side, defined by DTMM_REG_DEFINE in the
// dtmm_reg_*.cu units.  Geometry (grid, threads, shared bytes) comes from the
// engine; a variant that is not instantiated returns cudaErrorNotSupported.
// ---------------------------------------------------------------------------
struct RegLaunch {
  dim3 grid;
  int threads;
  size_t smem;
  cudaStream_t st;
};

// row variants: every (C, REAL) for power-of-two sides, real records for the others
__host__ __device__ constexpr bool reg_row_variant(int n, bool real) { return reg_lanes(n) > 0 && (real || is_pow2(n)); }

template <int N1, int N2, int C, bool REAL, int BAND = 0, int XR = 0>
cudaError_t row_reg_variant(const RegLaunch& L, const RowParams& p, const Grid& g, const void* U, void* X) {
  auto kern = k_layer_row_reg<float, C, REAL, N1, N2, BAND, XR>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
  if (e != cudaSuccess) return e;
  kern<<<L.grid, L.threads, L.smem, L.st>>>(p, g, (const cpx<float>*)U, (cpx<float>*)X);
  return cudaGetLastError();
}

// real records with a band variant b (row_band_pick), every (C, REAL) dense
// (p.xr > 0: the register-accumulator variant, built for 256-point rows of
// the 4x4 method, XR = p.xr pixels a thread)
template <int N1, int N2, int C>
cudaError_t row_reg_real(int band, const RegLaunch& L, const RowParams& p, const Grid& g, const void* U, void* X) {
  if constexpr (N1 == 16 && N2 == 16 && C == 4) {
    if (p.xr == 2) {
      if (band == 1) return row_reg_variant<N1, N2, C, true, 1, 2>(L, p, g, U, X);
      if (band == 2) return row_reg_variant<N1, N2, C, true, 2, 2>(L, p, g, U, X);
      return row_reg_variant<N1, N2, C, true, 0, 2>(L, p, g, U, X);
    }
  }
  if constexpr (row_band_ok(N2, 1))
    if (band == 1) return row_reg_variant<N1, N2, C, true, 1>(L, p, g, U, X);
  if constexpr (row_band_ok(N2, 2))
    if (band == 2) return row_reg_variant<N1, N2, C, true, 2>(L, p, g, U, X);
  return row_reg_variant<N1, N2, C, true, 0>(L, p, g, U, X);
}

template <int N1, int N2>
cudaError_t row_reg_launch(int C, bool real, int band, const RegLaunch& L, const RowParams& p, const Grid& g,
                           const void* U, void* X) {
  constexpr int N = N1 * N2;
  if (C == 4 && real) return row_reg_real<N1, N2, 4>(band, L, p, g, U, X);
  if (C == 2 && real) return row_reg_real<N1, N2, 2>(band, L, p, g, U, X);
  if constexpr (is_pow2(N)) {
    if (C == 4) return row_reg_variant<N1, N2, 4, false>(L, p, g, U, X);
    if (C == 2) return row_reg_variant<N1, N2, 2, false>(L, p, g, U, X);
  }
  return cudaErrorNotSupported;
}

template <int N1, int N2, int BAND>
cudaError_t col_reg_variant(const RegLaunch& L, const ColParams& p, const Grid& g, const void* in, void* out) {
  auto kern = k_layer_col_reg<float, N1, N2, BAND>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
  if (e != cudaSuccess) return e;
  kern<<<L.grid, L.threads, L.smem, L.st>>>(p, g, (const cpx<float>*)in, (cpx<float>*)out);
  return cudaGetLastError();
}

// band variants (row_band_pick of the H axis) for the diagonal operator of
// sides with N2 % N1 == 0; the caller passes band 0 for any other operator
template <int N1, int N2>
cudaError_t col_reg_launch(int band, const RegLaunch& L, const ColParams& p, const Grid& g, const void* in, void* out) {
  if constexpr (N2 % N1 == 0) {
    if constexpr (row_band_ok(N2, 1))
      if (band == 1) return col_reg_variant<N1, N2, 1>(L, p, g, in, out);
    if constexpr (row_band_ok(N2, 2))
      if (band == 2) return col_reg_variant<N1, N2, 2>(L, p, g, in, out);
  }
  return col_reg_variant<N1, N2, 0>(L, p, g, in, out);
}

template <int N1, int N2>
cudaError_t fft_rows_reg_launch(bool inv, const RegLaunch& L, const void* src, void* dst, int nlines, const void* tw,
                                float scale) {
  auto kern = inv ? k_fft_rows_reg<float, N1, N2, true> : k_fft_rows_reg<float, N1, N2, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
  if (e != cudaSuccess) return e;
  kern<<<L.grid, L.threads, L.smem, L.st>>>((const cpx<float>*)src, (cpx<float>*)dst, nlines,
                                             (const cpx<float>*)tw, scale);
  return cudaGetLastError();
}

#define DTMM_REG_SIDES(X) \
  X(64) X(80) X(96) X(112) X(128) X(144) X(160) X(192) X(224) X(240) X(256) X(288) X(320) X(336) X(384) X(400) \
  X(432) X(448) X(480) X(512) X(1024)

#define DTMM_REG_DECLARE(N)                                                                                      \
  cudaError_t row_reg_##N(int C, bool real, int band, const RegLaunch& L, const RowParams& p, const Grid& g,     \
                          const void* U, void* X);                                                             \
  cudaError_t col_reg_##N(int band, const RegLaunch& L, const ColParams& p, const Grid& g, const void* in,       \
                          void* out);                                                                          \
  cudaError_t fft_rows_reg_##N(bool inv, const RegLaunch& L, const void* src, void* dst, int nlines, const void* tw, \
                               float scale);

#define DTMM_REG_DEFINE(N)                                                                                       \
  cudaError_t row_reg_##N(int C, bool real, int band, const RegLaunch& L, const RowParams& p, const Grid& g,     \
                          const void* U, void* X) {                                                            \
    return row_reg_launch<reg_lanes(N), N / reg_lanes(N)>(C, real, band, L, p, g, U, X);                       \
  }                                                                                                            \
  cudaError_t col_reg_##N(int band, const RegLaunch& L, const ColParams& p, const Grid& g, const void* in,       \
                          void* out) {                                                                         \
    return col_reg_launch<reg_lanes(N), N / reg_lanes(N)>(band, L, p, g, in, out);                             \
  }                                                                                                            \
  cudaError_t fft_rows_reg_##N(bool inv, const RegLaunch& L, const void* src, void* dst, int nlines, const void* tw, \
                               float scale) {                                                                  \
    return fft_rows_reg_launch<reg_lanes(N), N / reg_lanes(N)>(inv, L, src, dst, nlines, tw, scale);           \
  }

DTMM_REG_SIDES(DTMM_REG_DECLARE)

// dispatch on the side (cudaErrorNotSupported for a side without a transform)
inline cudaError_t row_reg_dispatch(int n, int C, bool real, int band, const RegLaunch& L, const RowParams& p,
                                    const Grid& g, const void* U, void* X) {
  switch (n) {
#define DTMM_REG_ROW_CASE(N) \
  case N: return row_reg_##N(C, real, band, L, p, g, U, X);
    DTMM_REG_SIDES(DTMM_REG_ROW_CASE)
#undef DTMM_REG_ROW_CASE
    default: return cudaErrorNotSupported;
  }
}

inline cudaError_t col_reg_dispatch(int n, int band, const RegLaunch& L, const ColParams& p, const Grid& g,
                                    const void* in, void* out) {
  switch (n) {
#define DTMM_REG_COL_CASE(N) \
  case N: return col_reg_##N(band, L, p, g, in, out);
    DTMM_REG_SIDES(DTMM_REG_COL_CASE)
#undef DTMM_REG_COL_CASE
    default: return cudaErrorNotSupported;
  }
}

inline cudaError_t fft_rows_reg_dispatch(int n, bool inv, const RegLaunch& L, const void* src, void* dst, int nlines,
                                         const void* tw, float scale) {
  switch (n) {
#define DTMM_REG_FFT_CASE(N) \
  case N: return fft_rows_reg_##N(inv, L, src, dst, nlines, tw, scale);
    DTMM_REG_SIDES(DTMM_REG_FFT_CASE)
#undef DTMM_REG_FFT_CASE
    default: return cudaErrorNotSupported;
  }
}

}  // namespace dtmm
