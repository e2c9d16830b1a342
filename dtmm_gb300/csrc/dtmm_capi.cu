// Host orchestration of one transfer_field call on the GPU, exported through
// the C ABI declared in include/dtmm_gb300.h.
//
// One call enqueues, on the caller's stream:
//   set-up      : FFT tables, effective medium, window statistics/tables
//   per pass    : k-space entry table, then per (sub)layer a fused column
//                 kernel and a fused row kernel, then the k-space exit table
//   between passes (4x4, npass > 1): projection / normalisation / notch
//                 filtering and the total-intensity rescale of the reference
//                 (dtmm/transfer.py:815-873)
// No host synchronisation happens inside the call; all scratch lives in the
// caller's workspace.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <mutex>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dtmm_gb300.h"
#include "dtmm_effmed.h"
#include "dtmm_kernels.cuh"
#include "dtmm_regkern.cuh"

using namespace dtmm;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(DTMM_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)
#define CKL(what)                                                                                    \
  do {                                                                                               \
    ++launches;                                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                             \
    if (e_ != cudaSuccess) return fail(DTMM_ECUDA, "launch %s: %s", what, cudaGetErrorString(e_)); \
  } while (0)

// radix schedule of one line transform: radix-8 (when `rad8`) or radix-4
// passes first, then 2, 3, 5, 7
bool make_plan(int n, FFTPlan& p, bool rad8 = false) {
  p.n = n;
  p.nr = 0;
  int m = n;
  while (rad8 && m % 8 == 0 && p.nr < kMaxPasses) { p.r[p.nr++] = 8; m /= 8; }
  while (m % 4 == 0 && p.nr < kMaxPasses) { p.r[p.nr++] = 4; m /= 4; }
  while (m % 2 == 0 && p.nr < kMaxPasses) { p.r[p.nr++] = 2; m /= 2; }
  const int odd[10] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31};
  for (int q : odd)
    while (m % q == 0 && p.nr < kMaxPasses) { p.r[p.nr++] = q; m /= q; }
  p.rbits = 0;
  for (int i = 0; i < p.nr; ++i) p.rbits |= (unsigned long long)p.r[i] << (5 * i);
  return m == 1 && n >= 1;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr int kPartBlocks = 1216;  // blocks of the effective-medium reduction
constexpr int kWinChunks = 64;     // blocks per window of the window statistics

// Workspace layout (byte offsets), shared by the size query and the call.
struct Layout {
  int C;        // state components (4 or 2)
  int ny, nx, nwin;
  int nlay_sub; // total sub-steps
  bool cache_ops;
  size_t cplx;  // bytes of one complex
  size_t HW;
  size_t small, part, twH, permH, twW, permW, cx, cy;
  size_t slots, slot_bytes, dslots, dslot_bytes;
  int nslots, ndslots;
  size_t F, X, U, field0, op, Xw, Xa;
  size_t fbeta, fphi, fmodes;  // diffraction = inf: per-wavelength grid beta / phi, sorted modes + counts
  size_t fA, famp;             // diffraction = inf: row DFTs and mode amplitudes (FP64)
  size_t r4part;               // reflection mode 4 with windows: the window's part of the field
  size_t r2in, r2out, y2;      // 2x2 k-space, npass > 1: reflected waves of the outer interfaces, exit state
  size_t r2;                   // 2x2 real space, npass > 1: reflected wave of every interface
  size_t w2;                   // 2x2 real space with windows: window part, sum, reflected part and sum
  size_t effb, awb;            // per block: effective eps (re, im) and the windows' sqrt(eps_eff - beta^2)
  size_t effx, efft;           // per block: anisotropic effective medium (10 doubles), mean lab-frame tensor (12)
  size_t ref, ref2, refw;      // 4x4 norm_ref: reference field, its E part, window part / sum / H part
  size_t fnorm;                // 4x4 norm_ref without norm FFT ("local"): the output medium's field matrix and inverse
  bool chains;  // nstep > 1 with windows: per-window sub-step chains
  size_t op_one;  // bytes of one layer's operators
  size_t total;
};

// some block's effective medium is uniaxial or biaxial (block_sym 1 / 2)
int nblocks(const dtmm_transfer_desc* d);
bool is_real2(const dtmm_transfer_desc* d);
// block b's effective medium is uniaxial or biaxial: the mean of symmetry 1
// / 2, or a given medium (symmetry 3) without three equal eigenvalues
bool blk_aniso_of(const dtmm_transfer_desc* d, int b) {
  if (d->block_sym == nullptr) return false;
  const int s = d->block_sym[b];
  if (s == 1 || s == 2) return true;
  if (s != 3 || d->block_eff == nullptr) return false;
  const double* r = d->block_eff + 9 * (size_t)b;
  return !(r[0] == r[2] && r[2] == r[4] && r[1] == r[3] && r[3] == r[5]);
}
bool aniso_eff(const dtmm_transfer_desc* d) {
  if (d->block_sym == nullptr) return false;
  const int nb = nblocks(d);
  for (int b = 0; b < nb; ++b)
    if (blk_aniso_of(d, b)) return true;
  return false;
}

// 4x4 with diffraction through the real-space chains: reflection modes 2-4,
// and mode 1 around an anisotropic effective medium
bool is_refl4(const dtmm_transfer_desc* d) {
  return d->method == 4 && d->diffraction >= 1 &&
         ((d->reflection >= 2 && d->reflection <= 4) || (d->reflection == 1 && aniso_eff(d)));
}

int check_desc(const dtmm_transfer_desc* d) {
  if (d == nullptr) return fail(DTMM_EINVAL, "null descriptor");
  if (d->height < 1 || d->width < 1) return fail(DTMM_EINVAL, "grid must be at least 1x1");
  if (d->height > 16384 || d->width > 16384) return fail(DTMM_ENOTSUP, "grid side above 16384");
  if (d->nlam < 1 || d->npol < 1 || d->nray < 1) return fail(DTMM_EINVAL, "empty image axes");
  if (d->method != 4 && d->method != 2) return fail(DTMM_EINVAL, "method must be 4 (4x4) or 2 (2x2)");
  if (d->nlayers < 1) return fail(DTMM_EINVAL, "no layers");
  if (d->layer_block) {  // before anything reads the block count
    for (int l = 0; l < d->nlayers; ++l) {
      const int prev = l ? d->layer_block[l - 1] : 0;
      if (d->layer_block[l] != prev && d->layer_block[l] != prev + 1)
        return fail(DTMM_EINVAL, "layer_block must start at 0 and grow by 0 or 1 from layer to layer");
    }
  }
  if (d->block_sym) {
    for (int b = 0; b < nblocks(d); ++b) {
      if (d->block_sym[b] < 0 || d->block_sym[b] > 3)
        return fail(DTMM_EINVAL, "block_sym must be 0 (isotropic), 1 (uniaxial), 2 (biaxial) or 3 (given)");
      if (d->block_sym[b] == 3 && d->block_eff == nullptr)
        return fail(DTMM_EINVAL, "block_sym 3 needs block_eff");
    }
  }
  // reflection mode 2 without diffraction: the per-voxel 4x4 transfer (npass 1);
  // diffraction = inf (DTMM_DIFFRACTION_FULL): every eigenwave exactly (4x4, npass 1,
  // any reflection mode: the reference takes the same path for all of them;
  // 2x2 with reflection 0 or 2, any npass)
  const bool local4 = d->method == 4 && d->diffraction == 0 && (d->reflection == 2 || d->reflection == 4);
  const bool full4 = d->method == 4 && d->diffraction == DTMM_DIFFRACTION_FULL;
  const bool full2 = d->method == 2 && d->diffraction == DTMM_DIFFRACTION_FULL;
  // reflection modes 2-4 with diffraction: real-space steps around the
  // corrected diffraction matrices (tables per ray: they follow its beam)
  const bool refl4 = is_refl4(d);
  // the reference's 2x2 reflection 1 moves the field to k-space, and its modal
  // step transforms that field once more (dtmm/transfer.py:1091-1098, :1172)
  if (full2 && d->reflection == 1)
    return fail(DTMM_ENOTSUP, "2x2 with diffraction = inf is supported with reflection 0 or 2");
  // the modal DFT kernels take one grid row per (image, component) line
  if ((full4 || full2) && (long long)d->nray * d->npol * d->nlam * (full4 ? 4 : 2) > 65535)
    return fail(DTMM_ENOTSUP, "diffraction = inf is supported for at most %d images", full4 ? 16383 : 32767);
  // 2x2 without diffraction: real space (reflection 0 or 2) or k-space with
  // the interfaces' betamax cut only (reflection 1)
  const bool nodiff2 = d->method == 2 && d->diffraction == 0;
  if ((d->diffraction < 0 && !full4 && !full2) || (d->diffraction < 1 && !local4 && !full4 && !full2 && !nodiff2))
    return fail(DTMM_ENOTSUP, "diffraction must be >= 1 on this path (0 with 4x4 reflection mode 2 or 4, or "
                              "with 2x2; or inf)");
  if (d->method == 4 && (d->reflection < 1 || d->reflection > 4))
    return fail(DTMM_EINVAL, "4x4 reflection mode must be 1..4");
  if (d->method == 4 && d->reflection != 1 && !local4 && !full4 && !refl4)
    return fail(DTMM_ENOTSUP, "4x4 accepts reflection 1 with diffraction >= 1, 2-4 with diffraction >= 1, 2 and 4 "
                              "with diffraction 0, and any mode with diffraction = inf (reflection %d, diffraction "
                              "%d given)", d->reflection, d->diffraction);
  if (d->method == 2 && (d->reflection < 0 || d->reflection > 2))
    return fail(DTMM_EINVAL, "Invalid reflection. The 2x2 method supports reflection mode 0,1 or 2.");
  if (d->npass < 1) return fail(DTMM_EINVAL, "npass must be >= 1");
  if (d->method == 2 && d->npass > 1 && d->reflection == 0)
    return fail(DTMM_EINVAL, "Reflection mode `0` not compatible with npass > 1");
  // the reference's tracked reflection step applies its first diffraction
  // matrix, which it does not form without diffraction (dtmm/propagate_2x2.py:61)
  if (d->method == 2 && d->npass > 1 && d->reflection == 1 && d->diffraction == 0)
    return fail(DTMM_ENOTSUP, "2x2 reflection 1 without diffraction is not supported with npass > 1 (the "
                              "reference's tracked reflections need diffraction matrices)");
  if (d->precision != DTMM_PRECISION_MIXED && d->precision != DTMM_PRECISION_DOUBLE)
    return fail(DTMM_EINVAL, "unknown precision");
  // the reference's reference field takes int(diffraction) windows (dtmm/propagate_2x2.py:330)
  if (d->method == 4 && d->npass > 1 && d->norm_ref && d->diffraction == DTMM_DIFFRACTION_FULL)
    return fail(DTMM_ENOTSUP, "norm_ref is built for finite diffraction");
  if (d->nlayers < 1) return fail(DTMM_EINVAL, "no layers");
  if (!d->thickness || !d->nstep || !d->ks || !d->beta || !d->phi) return fail(DTMM_EINVAL, "null host array");
  if (!d->epsv || !d->epsa) return fail(DTMM_EINVAL, "null material pointer");
  for (int l = 0; l < d->nlayers; ++l) {
    if (d->nstep[l] < 1) return fail(DTMM_EINVAL, "nstep must be >= 1");
    // the k-space sweep cuts every step at betamax; the reference's sub-steps
    // without diffraction matrices do not
    if (nodiff2 && d->reflection == 1 && d->nstep[l] > 1)
      return fail(DTMM_ENOTSUP, "2x2 reflection 1 without diffraction supports nstep = 1");
  }
  if (d->block_sym) {
    // the 2x2 k-space sweep folds the isotropic medium's window corrections into its voxel
    // records; its reflection-0 step runs in real space instead, reflection 1 (interfaces
    // between the effective media, tracked reflections) is not built
    if (aniso_eff(d) && d->method == 2 && !is_real2(d) && d->diffraction != DTMM_DIFFRACTION_FULL)
      return fail(DTMM_ENOTSUP, "2x2 effective layers of uniaxial or biaxial symmetry are supported with reflection "
                                "0 or 2, or with diffraction = inf");
  }
  if (d->layer_block) {
    // the reflections of the inner interfaces between different effective media are not kept
    if (d->method == 2 && !(d->reflection == 2 || (d->diffraction == 0 && d->reflection == 0)) && d->npass > 1 &&
        d->layer_block[d->nlayers - 1] > 0)
      return fail(DTMM_ENOTSUP, "2x2 reflection 0 / 1 with several optical blocks is supported with npass = 1");
  }
  FFTPlan p;
  if (!make_plan(d->height, p) || !make_plan(d->width, p))
    return fail(DTMM_ENOTSUP, "grid sides must factor into primes up to 31 (got %dx%d)", d->height, d->width);
  if (d->betamax <= 0) return fail(DTMM_EINVAL, "betamax must be > 0");
  if (d->row_group < 0 || d->col_tile < 0 || d->fft_schedule < 0 || d->fft_schedule > 3)
    return fail(DTMM_EINVAL, "invalid tuning fields");
  return DTMM_OK;
}

// blocks of the layer list (layer_block null: one)
int nblocks(const dtmm_transfer_desc* d) {
  return (d->layer_block && d->nlayers > 0) ? d->layer_block[d->nlayers - 1] + 1 : 1;
}

// 2x2 in real space: reflection mode 2, or no diffraction without reflections
// -- and reflection 0 with diffraction around an anisotropic effective medium
// (the reference's k-space step, here on the real-space field)
bool is_real2(const dtmm_transfer_desc* d) {
  return d->method == 2 &&
         (d->reflection == 2 || (d->diffraction == 0 && d->reflection == 0) ||
          (d->reflection == 0 && d->diffraction >= 1 && aniso_eff(d)));
}

Layout layout_of(const dtmm_transfer_desc* d) {
  Layout L{};
  const size_t H = d->height, W = d->width;
  const size_t NI = (size_t)d->nray * d->npol * d->nlam;
  L.HW = H * W;
  L.C = d->method == 4 ? 4 : 2;
  L.cplx = d->precision == DTMM_PRECISION_DOUBLE ? 16 : 8;
  const size_t rsz = L.cplx / 2;
  const int n = d->diffraction;
  L.nx = L.ny = n > 1 ? n : 1;
  L.nwin = L.nx * L.ny;
  L.nlay_sub = 0;
  for (int l = 0; l < d->nlayers; ++l) L.nlay_sub += d->nstep[l];
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  const size_t nrw = (size_t)d->nray * L.nwin;
  L.small = take(sizeof(double) * (2 * d->nlam + 4 * d->nray + 9 * nrw + 4 + 3 * NI + 8));
  L.effb = take(sizeof(double) * 2 * nblocks(d));
  L.awb = take(sizeof(double) * nrw * nblocks(d));
  L.effx = take(sizeof(double) * 10 * nblocks(d));
  L.efft = take(sizeof(double) * 12 * nblocks(d));
  const bool refl4 = is_refl4(d);
  const bool real_space = d->method == 4 && (d->diffraction == 0 || d->diffraction == DTMM_DIFFRACTION_FULL || refl4);
  if (d->diffraction == DTMM_DIFFRACTION_FULL) {
    // beta, phi and the sorted mode list per wavelength and grid point, the
    // row DFTs and the mode amplitudes (FP64)
    const size_t grid = (size_t)d->nlam * L.HW;
    L.fbeta = take(sizeof(double) * grid);
    L.fphi = take(sizeof(double) * grid);
    L.fmodes = take(sizeof(int) * (grid + d->nlam));
    L.fA = take(16 * NI * 4 * L.HW);
    L.famp = take(16 * NI * 4 * L.HW);
  }
  const bool real2 = is_real2(d);
  if (real_space && d->npass == 1 && !refl4) {  // the per-voxel / modal sweep alone needs nothing more
    L.total = off;
    return L;
  }
  L.part = take(sizeof(double) * std::max<size_t>(2 * kPartBlocks, 4 * kWinChunks * nrw));
  L.twH = take(L.cplx * H);
  L.permH = take(sizeof(int) * H);
  L.twW = take(L.cplx * W);
  L.permW = take(sizeof(int) * W);
  L.cx = take(rsz * d->nray * L.nx * d->nlam * W);
  L.cy = take(rsz * d->nray * L.ny * d->nlam * H);
  const size_t kt = (size_t)d->nlam * L.HW;
  const bool passes = d->npass > 1;
  // k-space table slots: entry / exit / projection tables (reused across
  // passes when they repeat) and the inter-layer diagonal tables
  L.nslots = passes ? (d->method == 2 ? 8 : 6) : (real2 ? 4 : 3);
  // 4x4 tables (one per ray for the window / beam tables of reflection modes
  // 2-4), the 2x2 exit table 4x2 per ray
  L.slot_bytes = L.cplx * kt * std::max<size_t>(16 * (refl4 ? (size_t)d->nray : 1), 8 * (size_t)d->nray);
  L.slots = take(L.slot_bytes * L.nslots);
  L.ndslots = 2;
  L.dslot_bytes = L.cplx * kt * 2;
  L.dslots = take(L.dslot_bytes * L.ndslots);
  const size_t field = L.cplx * NI * 4 * L.HW;
  L.F = take(field);
  L.X = take(field);
  L.U = take(field * (size_t)(L.ny > 1 ? L.ny : 1));
  L.field0 = take(passes && d->method == 4 ? field : 0);
  L.chains = false;
  if (L.nwin > 1)
    for (int l = 0; l < d->nlayers; ++l)
      if (d->nstep[l] > 1) L.chains = true;
  L.Xw = take(L.chains ? field : 0);
  L.Xa = take(L.chains ? field : 0);
  L.r4part = take(refl4 && L.nwin > 1 ? field : 0);  // reflection mode 4: one window's part
  const size_t field2 = field / 2;
  const bool kpass2 = d->method == 2 && !real2 && passes;
  L.r2in = take(kpass2 ? field2 : 0);
  L.r2out = take(kpass2 ? field2 : 0);
  L.y2 = take(kpass2 ? field2 : 0);
  L.r2 = take(real2 && passes ? field2 * (size_t)(d->nlayers + 1) : 0);
  L.w2 = take(real2 && L.nwin > 1 ? 4 * field2 : 0);
  const bool refd = d->method == 4 && passes && d->norm_ref;
  L.ref = take(refd ? field : 0);
  L.ref2 = take(refd ? field2 : 0);
  L.refw = take(refd ? 3 * field2 : 0);
  L.fnorm = take(refd && d->norm_total ? 32 * sizeof(cpx<double>) : 0);
  // the real-space and modal paths keep no operator records
  L.op_one = (real_space || real2 || d->diffraction == DTMM_DIFFRACTION_FULL) ? 0 : L.cplx * nrw * OP_REC * L.HW;
  const size_t limit = d->op_cache_bytes ? d->op_cache_bytes : ((size_t)48 << 30);
  L.cache_ops = passes && L.op_one * (size_t)d->nlayers <= limit;
  // per-layer cache, or two buffers that alternate between the layer being
  // swept and the next layer's operators computed beside it
  L.op = take(L.op_one * (L.cache_ops ? (size_t)d->nlayers : 2));
  L.total = off;
  return L;
}

// host-side window offsets: the beam offset folded to the nearest multiple of
// the window spacing (dtmm/mode.py:54-70)
double fold(double off, double d) {
  double a = std::fmod(off, d);
  if (a != 0.0 && ((a < 0) != (d < 0))) a += d;  // numpy.mod sign convention
  double b = std::fmod(off, -d);
  if (b != 0.0 && ((b < 0) != (-d < 0))) b += -d;
  return std::fabs(a) > std::fabs(b) ? b : a;
}

// optional device-time accounting (dtmm_transfer_timed)
// Side stream of each caller stream, created on first use and kept for the
// process (at most kMaxSide of them; beyond that the overlap is skipped).
// The per-layer operators (FP64 eigen-solve) run there ahead of the row /
// column passes (FP32), so the FP64 pipe works while the FFT passes of the
// previous layer run.  When the caller's stream is being captured into a
// graph the stream is created with this thread's capture mode relaxed for
// the call, and the fork / join become edges of the graph.
constexpr size_t kMaxSide = 256;
std::mutex g_side_mu;
std::vector<std::pair<std::pair<int, cudaStream_t>, cudaStream_t>> g_side;

cudaStream_t side_stream(cudaStream_t origin) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_side_mu);
  for (auto& e : g_side)
    if (e.first.first == dev && e.first.second == origin) return e.second;
  if (g_side.size() >= kMaxSide) return nullptr;
  cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
  if (cudaThreadExchangeStreamCaptureMode(&mode) != cudaSuccess) return nullptr;
  cudaStream_t s = nullptr;
  const cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaThreadExchangeStreamCaptureMode(&mode);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  g_side.push_back({{dev, origin}, s});
  return s;
}

struct Prof {
  std::vector<cudaEvent_t> ev[3];  // row, col, op: begin/end pairs
  int launches = 0;
  ~Prof() {
    for (auto& v : ev)
      for (cudaEvent_t e : v) cudaEventDestroy(e);
  }
  void mark(int kind, cudaStream_t st) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, st);
    ev[kind].push_back(e);
  }
  double total(int kind) const {
    double ms = 0;
    for (size_t i = 0; i + 1 < ev[kind].size(); i += 2) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[kind][i], ev[kind][i + 1]);
      ms += t;
    }
    return ms;
  }
};
enum { PROF_ROW = 0, PROF_COL = 1, PROF_OP = 2 };

template <typename R>
struct Engine {
  Prof* prof = nullptr;
  int launches = 0;
  FullParams fullp{};  // diffraction = inf: mode tables (full_prepare)
  int blim_max = 1 << 30;   // largest band limit of the W axis over the wavelengths (set by setup)
  int blimH_max = 1 << 30;  // the same for the H axis
  // k-space table cache of this call: (kind, thickness, medium) -> slot
  struct Slot {
    int what = -1;
    double d = 0, e = 0;
    int mode = 0;
    int blk = -1;  // block of the effective medium (-1: independent of it)
    long long used = 0;
  };
  Slot slot[8], dslot[2];
  long long tick = 0;
  void mark(int kind) {
    if (prof) prof->mark(kind, st);
  }
  void mark_on(int kind, cudaStream_t s) {
    if (prof) prof->mark(kind, s);
  }
  // the operators' side stream (null: operators on the caller's stream) and
  // the events of this call, released when the call has enqueued everything
  cudaStream_t st2 = nullptr;
  std::vector<cudaEvent_t> own_events;
  ~Engine() {
    for (cudaEvent_t e : own_events) cudaEventDestroy(e);
  }
  // an event recorded now on stream s
  int record(cudaStream_t s, cudaEvent_t& e) {
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    own_events.push_back(e);
    CK(cudaEventRecord(e, s));
    return DTMM_OK;
  }
  // stream `waiter` waits for everything enqueued so far on stream `s`
  int wait_for(cudaStream_t waiter, cudaStream_t s) {
    cudaEvent_t e;
    int rc = record(s, e);
    if (rc) return rc;
    CK(cudaStreamWaitEvent(waiter, e, 0));
    return DTMM_OK;
  }
  const dtmm_transfer_desc& d;
  const dtmm_transfer_io& io;
  const Layout& L;
  unsigned char* ws;
  cudaStream_t st;
  Grid g;
  FFTPlan pH, pW;
  int NI;

  Engine(const dtmm_transfer_desc& d_, const dtmm_transfer_io& io_, const Layout& L_, unsigned char* ws_,
         cudaStream_t st_)
      : d(d_), io(io_), L(L_), ws(ws_), st(st_) {}

  cpx<R>* P(size_t off) const { return (cpx<R>*)(ws + off); }
  template <typename T>
  T* A(size_t off) const { return (T*)(ws + off); }

  // small area: ks | beta | phi | xoff | yoff | wbeta | wphi | wzero(int) | wcos | wsin | waw | wev02 |
  // wevs | wc2 | eps_eff(2) | i0 | i0f | fact
  double* ks() const { return A<double>(L.small); }
  double* rbeta() const { return ks() + d.nlam; }
  double* rphi() const { return rbeta() + d.nray; }
  double* xoff() const { return rphi() + d.nray; }
  double* yoff() const { return xoff() + d.nray; }
  double* wbeta() const { return yoff() + d.nray; }
  double* wphi() const { return wbeta() + (size_t)d.nray * L.nwin; }
  int* wzero() const { return (int*)(wphi() + (size_t)d.nray * L.nwin); }
  double* wcos() const { return (double*)(wzero()) + (size_t)d.nray * L.nwin; }
  double* wsin() const { return wcos() + (size_t)d.nray * L.nwin; }
  double* waw() const { return wsin() + (size_t)d.nray * L.nwin; }
  double* wev02() const { return waw() + (size_t)d.nray * L.nwin; }
  double* wevs() const { return wev02() + (size_t)d.nray * L.nwin; }
  double* wc2() const { return wevs() + (size_t)d.nray * L.nwin; }
  double* epseff() const { return wc2() + (size_t)d.nray * L.nwin; }
  double* i0() const { return epseff() + 4; }
  double* i0f() const { return i0() + NI; }
  double* fact() const { return i0f() + NI; }
  double* blim() const { return fact() + NI; }  // [lam] band limits of the W axis
  // per optical block: effective eps (re, im) and the windows' sqrt(eps_eff - beta^2)
  double* effb(int b) const { return A<double>(L.effb) + 2 * b; }
  double* effx(int b) const { return A<double>(L.effx) + 10 * b; }
  double* efft(int b) const { return A<double>(L.efft) + 12 * b; }
  // block b's effective medium is uniaxial or biaxial
  bool blk_aniso(int b) const { return b >= 0 && blk_aniso_of(&d, b); }
  // block b's effective medium is given (block_eff)
  bool blk_given(int b) const { return d.block_sym != nullptr && b >= 0 && d.block_sym[b] == 3; }
  double* awb(int b) const { return A<double>(L.awb) + (size_t)b * d.nray * L.nwin; }
  int blk_of(int l) const { return d.layer_block ? d.layer_block[l] : 0; }
  // the block whose effective medium the k-space tables fetched now use
  int cur_blk = 0;

  int launch_rows(cpx<R>* data, int C, bool inv, double scale) {
    const int nlines = NI * C * d.height;
    if constexpr (sizeof(R) == 4) {
      if (d.fft_schedule <= 1 && reg_lanes(d.width) > 0) {
        RegLaunch rl;
        const int n1 = reg_lanes(d.width), lpb = 256 / n1;
        rl.threads = lpb * n1;
        rl.smem = (size_t)(d.width + lpb * reg_row_stride(n1, d.width)) * sizeof(cpx<R>);
        rl.grid = dim3((unsigned)((nlines + lpb - 1) / lpb));
        rl.st = st;
        const cudaError_t e = fft_rows_reg_dispatch(d.width, inv, rl, data, data, nlines, P(L.twW), (float)scale);
        ++launches;
        if (e != cudaSuccess) return fail(DTMM_ECUDA, "launch k_fft_rows_reg: %s", cudaGetErrorString(e));
        return DTMM_OK;
      }
    }
    int lpb = 4096 / d.width;
    if (lpb < 1) lpb = 1;
    if (lpb > 16) lpb = 16;
    const size_t smem = (size_t)lpb * d.width * sizeof(cpx<R>) + d.width * (sizeof(cpx<R>) + sizeof(int));
    const int blocks = (nlines + lpb - 1) / lpb;
    if (inv) {
      CK(cudaFuncSetAttribute(k_fft_rows<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_fft_rows<R, true><<<blocks, 256, smem, st>>>(data, data, nlines, d.width, pW, P(L.twW), A<int>(L.permW),
                                                     scale, lpb);
    } else {
      CK(cudaFuncSetAttribute(k_fft_rows<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_fft_rows<R, false><<<blocks, 256, smem, st>>>(data, data, nlines, d.width, pW, P(L.twW), A<int>(L.permW),
                                                      scale, lpb);
    }
    CKL("k_fft_rows");
    return DTMM_OK;
  }

  int tile_cols(int cm, bool two) const {
    const size_t per = (size_t)cm * d.height * sizeof(cpx<R>) * (two ? 2 : 1);
    int tc = 1;
    while (tc < 16 && per * (tc * 2) <= 72 * 1024) tc *= 2;
    if (d.col_tile > 0 && per * d.col_tile <= 200 * 1024) tc = d.col_tile;
    if (tc > d.width) tc = d.width;
    return tc;
  }

  // register-transform column pass: complex64 bulk, sides listed by reg_lanes
  bool col_reg() const { return sizeof(R) == 4 && d.fft_schedule <= 1 && reg_lanes(d.height) > 0; }

  int launch_col_reg(ColParams& p, const cpx<R>* in, cpx<R>* out, int C) {
    if constexpr (sizeof(R) != 4) {
      return fail(DTMM_ENOTSUP, "register column transform is complex64 only");
    } else {
      const int n1 = reg_lanes(d.height);
      const size_t tiles = reg_col_tiles(d.height, p.ny);
      int tx = std::max(1, 256 / (C * n1));
      // tiles of H x (C tx + 1) complex: about 3 blocks per SM by default
      size_t cap = tiles == 2 ? 72 * 1024 : 100 * 1024;
      if (d.col_tile > 0 && d.col_tile * C * n1 <= 256) {  // the kernel's launch bound
        tx = d.col_tile;
        cap = 160 * 1024;
      }
      if (tx > d.width) tx = d.width;
      while (tx > 1 && tiles * d.height * (C * tx + 1) * sizeof(cpx<R>) > cap) tx /= 2;
      p.tc = tx;
      RegLaunch rl;
      rl.smem = tiles * d.height * (C * tx + 1) * sizeof(cpx<R>) + d.height * sizeof(cpx<R>);
      rl.threads = std::max(32, ((C * tx * n1 + 31) / 32) * 32);
      const int ntile = (d.width + tx - 1) / tx;
      p.tile_lo = 0;
      p.tile_hi0 = 0;
      int nlaunch = ntile;
      if (p.band_skip == 2 && p.kop == KOP_DIAG && blim_max >= 0) {
        // tiles holding a column with |frequency index| <= the largest band limit
        const int lo = (blim_max + 1 + tx - 1) / tx;        // columns 0 .. lim
        const int hi0 = std::max(lo, (d.width - blim_max) / tx);  // columns W - lim .. W - 1
        if (lo + (ntile - hi0) < ntile) {
          p.tile_lo = lo;
          p.tile_hi0 = hi0;
          nlaunch = lo + (ntile - hi0);
        }
      }
      rl.grid = dim3(nlaunch, NI);
      rl.st = st;
      mark(PROF_COL);
      // the diagonal table is cut at betamax: band variants of the inverse transforms
      const int band = p.kop == KOP_DIAG ? row_band_pick(d.height, blimH_max) : 0;
      const cudaError_t e = col_reg_dispatch(d.height, band, rl, p, g, in, out);
      mark(PROF_COL);
      ++launches;
      if (e != cudaSuccess) return fail(DTMM_ECUDA, "launch k_layer_col_reg: %s", cudaGetErrorString(e));
      return DTMM_OK;
    }
  }

  int launch_col(const cpx<R>* in, cpx<R>* out, int cin, int cout, int kop, const void* ktab, int ny,
                 const R* cy, bool do_fwd, bool inverse_out, double scale, size_t ktab_ray_stride = 0,
                 int j_only = -1) {
    ColParams p;
    p.ktab_ray_stride = ktab_ray_stride;
    // the engine's diagonal tables are cut at d.betamax; the register row
    // pass reads out-of-band columns as zero, so skipped tiles need no writes
    p.band_skip = row_reg() ? 2 : 1;
    p.blim = blim();
    p.j_only = j_only;
    p.cy_rows = L.ny;
    p.cin = cin;
    p.cout = cout;
    p.kop = kop;
    p.ktab = ktab;
    p.ny = ny;
    p.cy = cy;
    p.do_fwd = do_fwd;
    p.inverse_out = inverse_out;
    p.out_scale = scale;
    p.plan = pH;
    p.tw = P(L.twH);
    p.perm = A<int>(L.permH);
    const int cm = cin > cout ? cin : cout;
    if (col_reg() && cin == cout) return launch_col_reg(p, in, out, cin);
    p.tc = tile_cols(cm, true);
    const size_t smem = 2 * (size_t)cm * d.height * p.tc * sizeof(cpx<R>) + d.height * (sizeof(cpx<R>) + sizeof(int));
    CK(cudaFuncSetAttribute(k_layer_col<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((d.width + p.tc - 1) / p.tc, NI);
    mark(PROF_COL);
    k_layer_col<R><<<grid, 256, smem, st>>>(p, g, in, out);
    mark(PROF_COL);
    CKL("k_layer_col");
    return DTMM_OK;
  }

  bool real_ops() const { return d.real_path && !d.eps_complex && !d.biaxial; }
  // one real eps for every voxel: the real-path solve's window constants are tables
  bool uniform_real() const {
    return real_ops() && d.epsv_strides[0] == 0 && d.epsv_strides[1] == 0 && d.epsv_strides[2] == 0;
  }

  // wavelengths per row block: as many as fit ~100 KB of shared memory
  int row_group() const {
    const size_t per = 2 * (size_t)d.npol * L.C * (d.width | 1) * sizeof(cpx<R>);
    // about 16 lines per block (measured best for 256-pixel rows), within ~100 KB
    int G = 16 / (d.npol * L.C);
    if (G < 1) G = 1;
    if ((size_t)G * per > 100 * 1024) G = (int)((100 * 1024) / per);
    if (d.row_group > 0 && (size_t)d.row_group * per <= 200 * 1024) G = d.row_group;
    if (G < 1) G = 1;
    if (G > d.nlam) G = d.nlam;
    return G;
  }

  template <int C, bool REAL>
  int launch_row_t(const RowParams& p, const cpx<R>* Ub, cpx<R>* Xb) {
    const size_t smem = 2 * (size_t)p.G * p.PB * C * (d.width | 1) * sizeof(cpx<R>) + d.width * (sizeof(cpx<R>) + sizeof(int));
    if (smem > 220 * 1024) return fail(DTMM_ENOTSUP, "row of %d pixels too large for one block", d.width);
    CK(cudaFuncSetAttribute(k_layer_row<R, C, REAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // a multiple of the line count (fixed line per thread in the FFT passes)
    const int nl = p.G * p.PB * C;
    int threads = nl <= 256 ? (256 / nl) * nl : 256;
    if (d.width < 256 && nl <= 32) threads = std::max(nl, ((d.width + 31) / 32) * 32 / nl * nl);
    const int ngrp = (d.nlam + p.G - 1) / p.G;
    const int npg = (d.npol + p.PB - 1) / p.PB;
    dim3 grid(d.height, d.nray * ngrp * npg);
    mark(PROF_ROW);
    k_layer_row<R, C, REAL><<<grid, threads, smem, st>>>(p, g, Ub, Xb);
    mark(PROF_ROW);
    CKL("k_layer_row");
    return DTMM_OK;
  }

  // register-transform row pass: complex64 bulk, sides listed by reg_lanes
  // (complex operator records only for power-of-two sides)
  bool row_reg() const {
    return sizeof(R) == 4 && d.fft_schedule <= 1 && reg_row_variant(d.width, real_ops());
  }

  int row_group_reg() const {
    const int perG = d.npol * L.C;  // lines per wavelength
    const int n1 = reg_lanes(d.width);
    const size_t line_bytes = 2 * (size_t)reg_row_stride(n1, d.width) * sizeof(cpx<R>);
    // about 8 lines per block measured best (256-pixel rows, 4x4, 2 polarisations)
    int G = std::max(1, 8 / perG);
    if (d.row_group > 0) G = d.row_group;
    while (G > 1 && ((size_t)G * perG * line_bytes > 110 * 1024 || G * perG * n1 > reg_row_max_threads(d.width))) --G;
    return std::min(std::min(G, d.nlam), kMaxRowGroup);
  }

  int launch_row_reg(const RowParams& p, const cpx<R>* Ub, cpx<R>* Xb, int C, bool re) {
    if constexpr (sizeof(R) != 4) {
      return fail(DTMM_ENOTSUP, "register row transform is complex64 only");
    } else {
      const int n1 = reg_lanes(d.width);
      const int nl = p.G * p.PB * C;
      const size_t smem =
          2 * (size_t)nl * reg_row_stride(n1, d.width) * sizeof(cpx<R>) + d.width * sizeof(cpx<R>);
      if (smem > 220 * 1024 || nl * n1 > reg_row_max_threads(d.width))
        return fail(DTMM_ENOTSUP, "row of %d pixels too large for one block", d.width);
      RegLaunch rl;
      rl.smem = smem;
      rl.threads = std::max(((nl * n1 + 31) / 32) * 32, 32);
      const int ngrp = (d.nlam + p.G - 1) / p.G;
      const int npg = (d.npol + p.PB - 1) / p.PB;
      // one layer's operator records beyond half of L2 (128 MB): the groups of
      // a row run next to each other and share the row's records in L2
      const size_t rec_bytes = (re ? sizeof(R) : sizeof(cpx<R>)) * (size_t)d.nray * L.nwin * p.rec_stride * L.HW;
      RowParams q = p;
      q.groups_inner = rec_bytes > ((size_t)64 << 20) ? 1 : 0;
      // 256-point rows of the 4x4 method, two images a block in every block:
      // accumulators in registers, two pixels a thread
      q.xr = (C == 4 && re && d.width == 256 && nl == kXrLines && d.nlam % p.G == 0 && d.npol % p.PB == 0) ? 2 : 0;
      rl.grid = q.groups_inner ? dim3(d.nray * ngrp * npg, d.height) : dim3(d.height, d.nray * ngrp * npg);
      rl.st = st;
      mark(PROF_ROW);
      const int band = re ? row_band_pick(d.width, blim_max) : 0;
      const cudaError_t e = row_reg_dispatch(d.width, C, re, band, rl, q, g, Ub, Xb);
      mark(PROF_ROW);
      ++launches;
      if (e != cudaSuccess) return fail(DTMM_ECUDA, "launch k_layer_row_reg: %s", cudaGetErrorString(e));
      return DTMM_OK;
    }
  }

  int launch_row(const cpx<R>* Ub, cpx<R>* Xb, const void* op, double dir, int win_only = -1, bool use_cx = true,
                 bool accumulate = false) {
    RowParams p;
    p.blim = blim();
    p.win_only = win_only;
    p.use_cx = use_cx ? 1 : 0;
    p.accumulate = accumulate ? 1 : 0;
    p.PB = d.npol;
    p.C = L.C;
    p.nx = L.nx;
    p.ny = L.ny;
    p.cx = L.nx > 1 ? (const void*)A<R>(L.cx) : nullptr;
    p.wzero = L.nwin > 1 ? wzero() : nullptr;
    p.op = op;
    // records per voxel: both mode blocks for 4x4 and for 2x2 passes that alternate in direction
    p.rec_stride = (d.method == 4 || d.npass > 1) ? OP_REC : REC_BLOCK;
    p.ks = ks();
    p.dir = dir;
    p.in_scale = 1.0 / ((double)d.width * (double)d.height);
    p.plan = pW;
    p.tw = P(L.twW);
    p.perm = A<int>(L.permW);
    const bool re = real_ops();
    if (row_reg()) {
      p.G = row_group_reg();
      const int n1 = reg_lanes(d.width);
      if (2 * (size_t)d.npol * L.C * reg_row_stride(n1, d.width) * sizeof(cpx<R>) > 200 * 1024 ||
          d.npol * L.C * n1 > reg_row_max_threads(d.width))
        p.PB = 1;
      return launch_row_reg(p, Ub, Xb, L.C, re);
    }
    p.G = row_group();
    if (2 * (size_t)d.npol * L.C * (d.width | 1) * sizeof(cpx<R>) > 200 * 1024) p.PB = 1;
    if (L.C == 4) return re ? launch_row_t<4, true>(p, Ub, Xb) : launch_row_t<4, false>(p, Ub, Xb);
    return re ? launch_row_t<2, true>(p, Ub, Xb) : launch_row_t<2, false>(p, Ub, Xb);
  }

  int launch_ktab(int what, double dd, cpx<R>* tab, int proj_mode = 1, double eps_re = 0, double eps_im = 0,
                  bool eff = true) {
    KTabParams p;
    memset(&p, 0, sizeof(p));
    p.what = what;
    p.proj_mode = proj_mode;
    p.eps_dev = eff ? effb(cur_blk) : nullptr;
    p.effx = (eff && blk_aniso(cur_blk)) ? effx(cur_blk) : nullptr;
    p.eps_dev2 = nullptr;
    if (what == KT_D12 || what == KT_2BX) {  // the block before the boundary and its half step
      p.eps_dev2 = effb(proj_mode);
      p.d2 = eps_re;
    }
    p.eps = mk<double>(eps_re, eps_im);
    p.d = dd;
    p.betamax = d.betamax;
    p.ks = ks();
    p.with_t = d.reflection ? 1 : 0;
    p.eps_in = mk<double>(d.nin * d.nin, 0.0);
    p.eps_out = mk<double>(d.nout * d.nout, 0.0);
    p.eps_p = mk<double>(d.nin * d.nin, 0.0);
    p.nwin_axis = L.nx;
    p.wbeta = wbeta();
    p.wphi = wphi();
    p.wzero = wzero();
    p.win = winp();
    // 2x2 tables: proj_mode carries the mode (and for KT_2CE the window, 2 w +
    // (mode < 0)); entry interfaces go from the input medium into the effective
    // one, exit interfaces from the effective medium into the output medium
    // (forward) or back into the input medium (backward)
    p.mode = 1;
    p.ta = 1;
    p.tb = 0;
    // without diffraction the input is projected for the beam direction first
    // (transmitted_field_direct, dtmm/transfer.py:1075-1078)
    p.proj_in = d.diffraction > 0 ? 1 : 0;
    if (what == KT_2E || what == KT_2TE || what == KT_2R || what == KT_2OUT || what == KT_2X) {
      p.mode = proj_mode < 0 ? -1 : 1;
      p.ta = 0;
      p.tb = p.mode > 0 ? 2 : 1;
    } else if (what == KT_2CE || what == KT_2C1 || what == KT_2C2) {
      p.mode = (proj_mode & 1) ? -1 : 1;
      p.proj_mode = proj_mode >> 1;
    }
    const int n = d.nlam * d.height * d.width;
    // the exit / reflection tables and the window / beam tables depend on the
    // ray's windows: one slab per ray
    const bool per_ray = what == KT_2OUT || what == KT_WINMAT || what == KT_CFD || what == KT_CEPN ||
                         what == KT_CD || what == KT_DC || what == KT_2RIN || what == KT_2R || what == KT_2X ||
                         what == KT_2CE || what == KT_2WIN || what == KT_C1 || what == KT_C2 || what == KT_2C1 ||
                         what == KT_2C2;
    const int rays = per_ray ? d.nray : 1;
    const size_t slab = (size_t)n * ktab_entries(what);
    for (int r = 0; r < rays; ++r) {
      p.ray = r;
      k_ktab<R><<<(n + 127) / 128, 128, 0, st>>>(p, g, tab + (size_t)r * slab);
      CKL("k_ktab");
    }
    return DTMM_OK;
  }

  // complex entries of one k-space table per (lam, ky, kx)
  static int ktab_entries(int what) {
    switch (what) {
      case KT_2IN: case KT_2OUT: case KT_2RIN: case KT_2X: return 8;
      case KT_2E: case KT_2TE: case KT_2R: case KT_2CE: case KT_2WIN: case KT_2BX: case KT_2H: case KT_2C1:
      case KT_2C2: return 4;
      default: return 16;
    }
  }

  // table of kind `what` for thickness dd (medium eps_re for projections),
  // built once per call and reused while its slot is not needed for another
  int table(int what, double dd, const cpx<R>*& out, int proj_mode = 1, double eps_re = 0.0) {
    const bool diag = what == KT_DIAG;
    Slot* sl = diag ? dslot : slot;
    const int n = diag ? L.ndslots : L.nslots;
    const int blk = (what == KT_PROJ || what == KT_WINMAT || what == KT_2WIN || what == KT_2H) ? -1 : cur_blk;
    int pick = 0;
    for (int i = 0; i < n; ++i) {
      if (sl[i].what == what && sl[i].d == dd && sl[i].e == eps_re && sl[i].mode == proj_mode && sl[i].blk == blk) {
        sl[i].used = ++tick;
        out = P((diag ? L.dslots : L.slots) + (size_t)i * (diag ? L.dslot_bytes : L.slot_bytes));
        return DTMM_OK;
      }
      if (sl[i].used < sl[pick].used) pick = i;
    }
    cpx<R>* dst = P((diag ? L.dslots : L.slots) + (size_t)pick * (diag ? L.dslot_bytes : L.slot_bytes));
    int rc = (what == KT_PROJ || what == KT_2H) ? launch_ktab(what, dd, dst, proj_mode, eps_re, 0.0, false)
                                                : launch_ktab(what, dd, dst, proj_mode, eps_re);
    if (rc) return rc;
    sl[pick].what = what;
    sl[pick].d = dd;
    sl[pick].e = eps_re;
    sl[pick].mode = proj_mode;
    sl[pick].blk = blk;
    sl[pick].used = ++tick;
    out = dst;
    return DTMM_OK;
  }

  const cpx<R>* kdiag_cur = nullptr;
  // thickness factor of the diagonal tables between sub-steps: the pass
  // direction (4x4: the backward modes' phase follows the signed thickness);
  // 2x2: 1 (the e+ entry serves both directions), 0 without diffraction
  double kdir = 1.0;
  // (e+, e-) table of the merged half steps
  int diag_table(double dd) { return table(KT_DIAG, dd, kdiag_cur); }

  WinParams winp() const {
    WinParams w;
    w.n = d.diffraction;
    w.betamax = d.betamax;
    w.step = 0;
    if (d.diffraction > 1) {
      // numpy.linspace(-betamax, betamax, n): step = ax[1] - ax[0]
      const double st = (2.0 * d.betamax) / (d.diffraction - 1);
      const double a0 = -d.betamax, a1 = -d.betamax + 1 * st;
      w.step = (d.diffraction - 1 == 1) ? (d.betamax - a0) : (a1 - a0);
    }
    w.xoff = xoff();
    w.yoff = yoff();
    w.ks = ks();
    return w;
  }

  int voxel_ops(int layer, double dsub, cpx<R>* op, cudaStream_t s = nullptr) {
    if (s == nullptr) s = st;
    OpParams p;
    memset(&p, 0, sizeof(p));
    p.eps_dev = effb(blk_of(layer));
    p.permW = row_reg() ? nullptr : A<int>(L.permW);
    p.epsv = d.epsv;
    p.epsa = d.epsa;
    for (int i = 0; i < 3; ++i) {
      p.ev_s[i] = d.epsv_strides[i];
      p.ea_s[i] = d.epsa_strides[i];
    }
    p.eps_complex = d.eps_complex;
    p.layer = layer;
    p.d = dsub;
    p.wbeta = wbeta();
    p.wphi = wphi();
    p.wcos = wcos();
    p.wsin = wsin();
    p.waw = awb(blk_of(layer));
    p.nwin = L.nwin;
    // both mode blocks for 4x4, and for 2x2 passes that alternate in direction
    p.four = d.method == 4 || d.npass > 1;
    p.scale = 1.0 / ((double)d.width * (double)d.height);
    p.uncorrected = d.method == 2 && d.diffraction == 0;
    p.nray = d.nray;
    // every ray of a voxel in one thread (its trigonometry computed once)
    // while that still leaves at least 4 blocks per SM
    const int blocks = (int)((L.HW + 127) / 128);
    int rpt = d.nray;
    while (rpt > 1 && (long long)blocks * ((d.nray + rpt - 1) / rpt) < 608) rpt = (rpt + 1) / 2;
    p.rays_per_thread = rpt;
    dim3 grid((unsigned)blocks, (unsigned)((d.nray + rpt - 1) / rpt));
    mark_on(PROF_OP, s);
    p.wev02 = uniform_real() ? wev02() : nullptr;
    p.wevs = wevs();
    p.wc2 = wc2();
    if (real_ops()) {
      if (p.four)
        k_voxel_op<R, true, true, false><<<grid, 128, 0, s>>>(p, g, op);
      else
        k_voxel_op<R, true, false, false><<<grid, 128, 0, s>>>(p, g, op);
    } else if (d.biaxial) {
      if (p.four)
        k_voxel_op<R, false, true, true><<<grid, 128, 0, s>>>(p, g, op);
      else
        k_voxel_op<R, false, false, true><<<grid, 128, 0, s>>>(p, g, op);
    } else {
      if (p.four)
        k_voxel_op<R, false, true, false><<<grid, 128, 0, s>>>(p, g, op);
      else
        k_voxel_op<R, false, false, false><<<grid, 128, 0, s>>>(p, g, op);
    }
    mark_on(PROF_OP, s);
    CKL("k_voxel_op");
    return DTMM_OK;
  }

  // 4x4 reflection mode 2 without diffraction: the per-voxel transfer layer
  // by layer (input -> field_out, then in place), each layer's result also
  // into the bulk output when asked
  // Parameters of the per-voxel kernels (reflection mode 2 without
  // diffraction, and diffraction = inf) for layer l; d is set per layer.
  Local4Params local_params() {
    Local4Params p;
    p.epsv = d.epsv;
    p.epsa = d.epsa;
    for (int i = 0; i < 3; ++i) {
      p.ev_s[i] = d.epsv_strides[i];
      p.ea_s[i] = d.epsa_strides[i];
    }
    p.eps_complex = d.eps_complex;
    p.ks = ks();
    p.beta = rbeta();
    p.phi = rphi();
    p.bstride = 1;
    p.op = 0;
    return p;
  }

  // diffraction = inf: beta, phi and the sorted in-band mode list of every
  // wavelength (once per call)
  int full_prepare(FullParams& fp) {
    fp.ks = ks();
    fp.betamax = d.betamax;
    fp.beta = A<double>(L.fbeta);
    fp.phi = A<double>(L.fphi);
    fp.modes = A<int>(L.fmodes);
    fp.count = fp.modes + (size_t)d.nlam * L.HW;
    int limx = -1;
    for (int i = 0; i < d.nlam; ++i) limx = std::max(limx, band_limit(d.width, d.ks[i], d.betamax));
    fp.limx = std::max(limx, 0);
    fp.S = 2 * fp.limx + 1 >= d.width ? d.width : 2 * fp.limx + 1;
    fp.C = L.C;
    CK(cudaMemsetAsync(fp.count, 0, sizeof(int) * d.nlam, st));
    const dim3 gk((unsigned)((L.HW + 127) / 128), (unsigned)d.nlam);
    k_full_betaphi<<<gk, 128, 0, st>>>(fp, g);
    CKL("k_full_betaphi");
    k_full_rank<<<gk, 128, 0, st>>>(fp, g);
    CKL("k_full_rank");
    return DTMM_OK;
  }

  // diffraction = inf, one layer (signed by dir) from src into dst (may be
  // src): per sub-step the mode amplitudes of the current field, then their
  // plane waves through the voxels.  The layer list already holds the
  // sub-step thickness d / nstep (dtmm/transfer.py:926-975) and
  // propagate_4x4_full divides it by nsteps once more
  // (dtmm/propagate_4x4.py:521): each sub-step advances d / nstep^2.
  int full_layer(const FullParams& fp, Local4Params& q, int l, double dir, const cpx<R>* src, cpx<R>* dst) {
    q.layer = l;
    q.nst = d.nstep[l];
    q.d = dir * d.thickness[l] / ((double)d.nstep[l] * d.nstep[l]);
    cpx<double>* Ab = A<cpx<double>>(L.fA);
    cpx<double>* amp = A<cpx<double>>(L.famp);
    const dim3 gk((unsigned)((L.HW + 127) / 128), (unsigned)d.nlam);
    for (int s = 0; s < d.nstep[l]; ++s) {
      const cpx<R>* in = s == 0 ? src : (const cpx<R>*)dst;
      k_full_rowdft<R><<<dim3((unsigned)d.height, (unsigned)(NI * 4)), 128, 0, st>>>(fp, g, in, Ab);
      CKL("k_full_rowdft");
      k_full_coldft<<<dim3((unsigned)((L.HW + 127) / 128), (unsigned)(NI * 4)), 128, 0, st>>>(fp, g, Ab, amp);
      CKL("k_full_coldft");
      k_full_apply<R><<<gk, 128, 0, st>>>(fp, q, g, amp, dst);
      CKL("k_full_apply");
    }
    return DTMM_OK;
  }

  // reflection mode 2 without diffraction, one layer (signed by dir) from src
  // into dst (may be src), also into slab when given
  int local_layer(Local4Params& p, int l, double dir, const cpx<R>* src, cpx<R>* dst, cpx<R>* slab) {
    p.layer = l;
    p.nst = d.nstep[l];
    p.d = dir * d.thickness[l] / d.nstep[l];
    const dim3 grid((unsigned)((L.HW + 127) / 128), (unsigned)d.nray);
    k_local4<R><<<grid, 128, 0, st>>>(p, g, src, dst, slab);
    CKL("k_local4");
    return DTMM_OK;
  }

  // the per-voxel operator `op` (F P F^-1, E P F^-1 or F P E^-1) of every
  // voxel over thickness dd (one step) for the beam of window w of ray 0,
  // in place
  int local_step(Local4Params& p, int l, double dd, int w, int op, cpx<R>* f) {
    p.layer = l;
    p.nst = 1;
    p.d = dd;
    p.op = op;
    p.beta = wbeta() + w;
    p.phi = wphi() + w;
    p.bstride = L.nwin;
    const dim3 grid((unsigned)((L.HW + 127) / 128), (unsigned)d.nray);
    k_local4<R><<<grid, 128, 0, st>>>(p, g, f, f, nullptr);
    CKL("k_local4");
    return DTMM_OK;
  }

  // reflection modes 2 and 4 with diffraction, one layer of sub-steps ds
  // (signed) on F: per window (one for diffraction 1) the part of the field
  // in the window, then per sub-step a per-voxel half step, the corrected
  // diffraction matrix over ds, the second half step; the parts summed.
  // Mode 4: F P F^-1, the corrected field diffraction matrix, F P F^-1
  // (dtmm/propagate_4x4.py:55-77, :233-287); mode 2: E P F^-1, the corrected
  // E matrices of the forward and backward modes, F P E^-1
  // (dtmm/propagate_4x4.py:18-52, :156-230).
  // Mode 3 (its field lives in k-space between layers in the reference; the
  // same operators on the real-space field): C . D over ds/2, F P F^-1 over
  // ds, D . C over ds/2 (dtmm/propagate_4x4.py:135-153, :447-512).
  int refl_chain(Local4Params& p, int l, double ds, int w, cpx<R>* f) {
    const size_t rs = (size_t)d.nlam * L.HW * 16;  // one 4x4 table per ray
    int rc;
    if (d.reflection == 1) {
      // mode 1 around an anisotropic effective medium (its k-space field here
      // in real space, every step being linear): C . E P F^-1 over ds/2,
      // E P E^-1 over ds, F P E^-1 . C over ds/2 (dtmm/propagate_4x4.py:80-101,
      // :357-442)
      const cpx<R>* c1;
      const cpx<R>* c2;
      if ((rc = table(KT_C1, ds / 2, c1, w))) return rc;
      if ((rc = diffract(f, f, c1, rs))) return rc;
      if ((rc = local_step(p, l, ds, w, 3, f))) return rc;
      if ((rc = table(KT_C2, ds / 2, c2, w))) return rc;
      return diffract(f, f, c2, rs);
    }
    if (d.reflection == 3) {
      const cpx<R>* cd;
      const cpx<R>* dc;
      if ((rc = table(KT_CD, ds / 2, cd, w))) return rc;
      if ((rc = diffract(f, f, cd, rs))) return rc;
      if ((rc = local_step(p, l, ds, w, 0, f))) return rc;
      if ((rc = table(KT_DC, ds / 2, dc, w))) return rc;
      return diffract(f, f, dc, rs);
    }
    const bool two = d.reflection == 2;
    const cpx<R>* cfd;
    if ((rc = table(two ? KT_CEPN : KT_CFD, ds, cfd, w))) return rc;
    if ((rc = local_step(p, l, ds / 2, w, two ? 1 : 0, f))) return rc;
    if ((rc = diffract(f, f, cfd, rs))) return rc;
    return local_step(p, l, ds / 2, w, two ? 2 : 0, f);
  }

  int refl4_layer(Local4Params& p, int l, double ds) {
    cpx<R>* F = P(L.F);
    const int nst = d.nstep[l];
    int rc;
    if (L.nwin == 1) {
      for (int s = 0; s < nst; ++s)
        if ((rc = refl_chain(p, l, ds, 0, F))) return rc;
      return DTMM_OK;
    }
    const size_t bytes = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    cpx<R>* acc = P(L.X);
    cpx<R>* part = P(L.r4part);
    CK(cudaMemsetAsync(acc, 0, bytes, st));
    for (int w = 0; w < L.nwin; ++w) {
      const cpx<R>* win;
      if ((rc = table(KT_WINMAT, 0.0, win, w))) return rc;
      if ((rc = diffract(part, F, win, (size_t)d.nlam * L.HW * 16))) return rc;
      for (int s = 0; s < nst; ++s)
        if ((rc = refl_chain(p, l, ds, w, part))) return rc;
      if ((rc = axpby(acc, acc, nullptr, 1.0, part, nullptr, 1.0))) return rc;
    }
    CK(cudaMemcpyAsync(F, acc, bytes, cudaMemcpyDeviceToDevice, st));
    return DTMM_OK;
  }

  // One pass of the real-space 4x4 paths over F (in place): layer order and
  // thickness sign alternate with the pass as in dtmm/transfer.py:735-747;
  // with bulk (npass 1) each layer's result also into its slab
  int sweep_real4(int pass, cpx<R>* bulk) {
    const double dir = (pass % 2 == 0) ? 1.0 : -1.0;
    std::vector<int> order;
    layer_order(pass % 2 == 0 ? 1 : -1, order);
    cpx<R>* F = P(L.F);
    Local4Params p = local_params();
    const size_t bytes = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    int rc;
    for (int l : order) {
      cur_blk = blk_of(l);
      if (d.diffraction == DTMM_DIFFRACTION_FULL)
        rc = full_layer(fullp, p, l, dir, F, F);
      else if (d.diffraction == 0)
        rc = local_layer(p, l, dir, F, F, nullptr);
      else
        rc = refl4_layer(p, l, dir * d.thickness[l] / d.nstep[l]);
      if (rc) return rc;
      if (bulk) CK(cudaMemcpyAsync(bulk + (size_t)(l + 1) * NI * 4 * L.HW, F, bytes, cudaMemcpyDeviceToDevice, st));
    }
    return DTMM_OK;
  }

  // 4x4 with diffraction = inf, npass 1: input -> field_out, then in place;
  // each layer's result also into the bulk output when asked
  int run_full4() {
    int rc = scalars();
    if (rc) return rc;
    cpx<R>* fin = (cpx<R>*)io.field_in;
    cpx<R>* fout = (cpx<R>*)io.field_out;
    cpx<R>* bulk = (cpx<R>*)io.bulk;
    if ((rc = full_prepare(fullp))) return rc;
    Local4Params q = local_params();
    const size_t bytes = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    for (int l = 0; l < d.nlayers; ++l) {
      if ((rc = full_layer(fullp, q, l, 1.0, l == 0 ? (const cpx<R>*)fin : (const cpx<R>*)fout, fout))) return rc;
      if (bulk) CK(cudaMemcpyAsync(bulk + (size_t)(l + 1) * NI * 4 * L.HW, fout, bytes, cudaMemcpyDeviceToDevice, st));
    }
    return DTMM_OK;
  }

  // 4x4 reflection mode 2 without diffraction, npass 1: the per-voxel
  // transfer layer by layer (input -> field_out, then in place), each
  // layer's result also into the bulk output when asked
  int run_local4() {
    int rc = scalars();
    if (rc) return rc;
    cpx<R>* fin = (cpx<R>*)io.field_in;
    cpx<R>* fout = (cpx<R>*)io.field_out;
    cpx<R>* bulk = (cpx<R>*)io.bulk;
    Local4Params p = local_params();
    for (int l = 0; l < d.nlayers; ++l) {
      cpx<R>* slab = bulk ? bulk + (size_t)(l + 1) * NI * 4 * L.HW : nullptr;
      if ((rc = local_layer(p, l, 1.0, l == 0 ? (const cpx<R>*)fin : (const cpx<R>*)fout, fout, slab))) return rc;
    }
    return DTMM_OK;
  }

  // host scalars -> workspace: ks | beta | phi | window offsets
  int scalars() {
    std::vector<double> h(d.nlam + 4 * d.nray);
    for (int i = 0; i < d.nlam; ++i) h[i] = d.ks[i];
    const double dwin = d.diffraction > 1 ? 2.0 * d.betamax / (d.diffraction - 1) : 1.0;
    for (int r = 0; r < d.nray; ++r) {
      h[d.nlam + r] = d.beta[r];
      h[d.nlam + d.nray + r] = d.phi[r];
      h[d.nlam + 2 * d.nray + r] = fold(d.beta[r] * std::cos(d.phi[r]), dwin);
      h[d.nlam + 3 * d.nray + r] = fold(d.beta[r] * std::sin(d.phi[r]), dwin);
    }
    for (size_t o = 0; o < h.size(); o += 64) {
      Scalars64 sc;
      sc.n = (int)std::min<size_t>(64, h.size() - o);
      sc.off = (int)o;
      for (int i = 0; i < sc.n; ++i) sc.v[i] = h[o + i];
      k_set_scalars<<<1, 64, 0, st>>>(sc, ks());
      CKL("k_set_scalars");
    }
    return DTMM_OK;
  }

  int setup() {
    int rc = scalars();
    if (rc) return rc;
    {  // band limits of the W axis per wavelength (host, by value)
      blim_max = -1;
      blimH_max = -1;
      for (int i = 0; i < d.nlam; ++i) blimH_max = std::max(blimH_max, band_limit(d.height, d.ks[i], d.betamax));
      for (int o = 0; o < d.nlam; o += 64) {
        Scalars64 sc;
        sc.n = std::min(64, d.nlam - o);
        sc.off = o;
        for (int i = 0; i < sc.n; ++i) {
          const int lim = band_limit(d.width, d.ks[o + i], d.betamax);
          blim_max = std::max(blim_max, lim);
          sc.v[i] = (double)lim;
        }
        k_set_scalars<<<1, 64, 0, st>>>(sc, blim());
        CKL("k_set_scalars");
      }
    }
    // FFT tables
    k_fft_tables<R><<<(d.height + 255) / 256, 256, 0, st>>>(pH, P(L.twH), A<int>(L.permH));
    CKL("k_fft_tables");
    k_fft_tables<R><<<(d.width + 255) / 256, 256, 0, st>>>(pW, P(L.twW), A<int>(L.permW));
    CKL("k_fft_tables");
    // effective medium of every optical block: the mean eps of its voxels
    for (int l0 = 0; l0 < d.nlayers;) {
      int l1 = l0 + 1;
      while (l1 < d.nlayers && blk_of(l1) == blk_of(l0)) ++l1;
      // one eps for every voxel (all strides 0): the mean of that voxel
      const bool one = d.epsv_strides[0] == 0 && d.epsv_strides[1] == 0 && d.epsv_strides[2] == 0;
      const long long nvox = one ? 1 : (long long)(l1 - l0) * d.height * d.width;
      int blocks = (int)((nvox + 1023) / 1024);
      if (blocks > kPartBlocks) blocks = kPartBlocks;
      const char* e0 = (const char*)d.epsv + (size_t)l0 * d.epsv_strides[0] * (d.eps_complex ? 16 : 8);
      if (blk_given(blk_of(l0))) {  // a given medium: its first eigenvalue (the isotropic one when all are equal)
        const double* r = d.block_eff + 9 * (size_t)blk_of(l0);
        Scalars64 sc;
        sc.n = 2;
        sc.off = 0;
        sc.v[0] = r[0];
        sc.v[1] = r[1];
        k_set_scalars<<<1, 64, 0, st>>>(sc, effb(blk_of(l0)));
        CKL("k_set_scalars");
        l0 = l1;
        continue;
      }
      k_eps_mean<<<blocks, 256, 0, st>>>(e0, d.eps_complex, d.epsv_strides[0], d.epsv_strides[1], d.epsv_strides[2],
                                         one ? 1 : l1 - l0, one ? 1 : d.height, one ? 1 : d.width, A<double>(L.part));
      CKL("k_eps_mean");
      k_eps_final<<<1, 256, 0, st>>>(A<double>(L.part), blocks, nvox, effb(blk_of(l0)));
      CKL("k_eps_final");
      if (blk_aniso(blk_of(l0))) {  // the mean lab-frame tensor
        const bool onea = one && d.epsa_strides[0] == 0 && d.epsa_strides[1] == 0 && d.epsa_strides[2] == 0;
        const long long nv = onea ? 1 : (long long)(l1 - l0) * d.height * d.width;
        int tb = (int)((nv + 1023) / 1024);
        if (tb > kPartBlocks / 6) tb = kPartBlocks / 6;
        k_eps_tensor_mean<<<tb, 256, 0, st>>>(e0, d.epsa + (size_t)l0 * d.epsa_strides[0], d.eps_complex,
                                              d.epsv_strides[0], d.epsv_strides[1], d.epsv_strides[2],
                                              d.epsa_strides[0], d.epsa_strides[1], d.epsa_strides[2],
                                              onea ? 1 : l1 - l0, onea ? 1 : d.height, onea ? 1 : d.width,
                                              A<double>(L.part));
        CKL("k_eps_tensor_mean");
        k_eps_tensor_final<<<1, 32, 0, st>>>(A<double>(L.part), tb, nv, efft(blk_of(l0)));
        CKL("k_eps_tensor_final");
      }
      l0 = l1;
    }
    bool means = false;  // some block's medium is the eigen-frame of its mean tensor
    for (int b = 0; b < nblocks(&d); ++b) means = means || (blk_aniso(b) && !blk_given(b));
    if (aniso_eff(&d)) {
      const int nb = nblocks(&d);
      std::vector<double> t(12 * (size_t)nb), x(10 * (size_t)nb, 0.0);
      if (means) {  // the eigen-frame of each anisotropic block's mean tensor, on the host
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone)
          return fail(DTMM_ENOTSUP, "effective layers of uniaxial or biaxial symmetry are not supported in a stream "
                                    "capture (their eigen-frame is found on the host)");
        CK(cudaMemcpyAsync(t.data(), efft(0), sizeof(double) * t.size(), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
      for (int b = 0; b < nb; ++b) {
        if (!blk_aniso(b)) continue;
        double* xb = x.data() + 10 * (size_t)b;
        if (blk_given(b)) {  // the given eigenvalues and angles
          xb[0] = 3.0;
          for (int i = 0; i < 9; ++i) xb[1 + i] = d.block_eff[9 * (size_t)b + i];
        } else {
          eff_medium(t.data() + 12 * (size_t)b, d.block_sym[b], !d.eps_complex, xb);
        }
      }
      for (size_t o = 0; o < x.size(); o += 64) {
        Scalars64 sc;
        sc.n = (int)std::min<size_t>(64, x.size() - o);
        sc.off = (int)o;
        for (int i = 0; i < sc.n; ++i) sc.v[i] = x[o + i];
        k_set_scalars<<<1, 64, 0, st>>>(sc, effx(0));
        CKL("k_set_scalars");
      }
    }
    // windows
    if (d.diffraction > 1) {
      WinParams w = winp();
      // partial sums over many blocks, then the per-window means
      dim3 gs(kWinChunks, L.ny, d.nray);  // one block row per window row j
      k_window_stats<<<gs, 256, 0, st>>>(w, g, A<double>(L.part));
      CKL("k_window_stats");
      k_window_final<<<(L.nwin * d.nray + 127) / 128, 128, 0, st>>>(A<double>(L.part), kWinChunks, wbeta(), wphi(),
                                                                    wzero(), wcos(), wsin(), L.nwin * d.nray);
      CKL("k_window_final");
      dim3 gt(8, d.nlam, d.nray);
      k_window_tables<R><<<gt, 256, 0, st>>>(w, g, A<R>(L.cx), A<R>(L.cy));
      CKL("k_window_tables");
    } else {
      CK(cudaMemcpyAsync(wbeta(), rbeta(), sizeof(double) * d.nray, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(wphi(), rphi(), sizeof(double) * d.nray, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemsetAsync(wzero(), 0, sizeof(int) * d.nray, st));
      k_sincos<<<(d.nray + 127) / 128, 128, 0, st>>>(wphi(), wcos(), wsin(), d.nray);
      CKL("k_sincos");
    }
    for (int b = 0; b < nblocks(&d); ++b) {
      k_window_aw<<<(L.nwin * d.nray + 127) / 128, 128, 0, st>>>(wbeta(), effb(b), awb(b), L.nwin * d.nray,
                                                                uniform_real() ? (const double*)d.epsv : nullptr,
                                                                wev02(), wevs(), wc2());
      CKL("k_window_aw");
    }
    return DTMM_OK;
  }

  // layer order of one pass
  void layer_order(int dir, std::vector<int>& out) const {
    out.clear();
    for (int q = 0; q < d.nlayers; ++q) out.push_back(dir > 0 ? q : d.nlayers - 1 - q);
  }

  // One layer of `nst` sub-steps of thickness ds (signed by dir).  `in` holds
  // the state entering the layer (rows transformed along x), cin components;
  // the entry k-space operator is (kop0, ktab0).  Result: state in *out.
  // Without windows, or with one sub-step, every sub-step is one column and
  // one row pass.  With windows and several sub-steps each window follows its
  // own chain through the sub-steps (the reference applies the window once,
  // then all sub-steps to that part), and the chains are summed.
  int layer(const cpx<R>* in, int cin, int kop0, const void* ktab0, size_t ktab0_ray, cpx<R>*& out, const void* op,
            double dir, int nst, double ds) {
    int rc;
    const int C = L.C;
    cpx<R>* U = P(L.U);
    const R* cy = L.ny > 1 ? A<R>(L.cy) : nullptr;
    if (L.nwin == 1 || nst == 1) {
      cpx<R>* X = P(L.X);
      for (int s = 0; s < nst; ++s) {
        if (s == 0) {
          if ((rc = launch_col(in, U, cin, C, kop0, ktab0, L.ny, cy, true, true, 1.0, ktab0_ray))) return rc;
        } else {
          if ((rc = diag_table(kdir * ds))) return rc;
          if ((rc = launch_col(X, U, C, C, KOP_DIAG, kdiag_cur, 1, nullptr, true, true, 1.0))) return rc;
        }
        if ((rc = launch_row(U, X, op, dir))) return rc;
      }
      out = X;
      return DTMM_OK;
    }
    cpx<R>* Xw = P(L.Xw);
    cpx<R>* Xa = P(L.Xa);
    for (int w = 0; w < L.nwin; ++w) {
      const int j = w % L.ny;
      for (int s = 0; s < nst; ++s) {
        cpx<R>* dst = (s + 1 == nst) ? Xa : Xw;
        if (s == 0) {
          if ((rc = launch_col(in, U, cin, C, kop0, ktab0, 1, cy, true, true, 1.0, ktab0_ray, j))) return rc;
        } else {
          if ((rc = diag_table(kdir * ds))) return rc;
          if ((rc = launch_col(Xw, U, C, C, KOP_DIAG, kdiag_cur, 1, nullptr, true, true, 1.0))) return rc;
        }
        if ((rc = launch_row(U, dst, op, dir, w, s == 0, s + 1 == nst && w > 0))) return rc;
      }
    }
    out = Xa;
    return DTMM_OK;
  }

  // Operators of the layers of one sweep (layer order `order`, sub-step
  // thickness ds[q]).  With a side stream they are computed there ahead of
  // use: every layer at once into the per-layer cache (first pass; later
  // passes reuse it), or one layer ahead into two alternating buffers, the
  // side stream waiting until the passes that last read a buffer are queued
  // before it overwrites it.  Without a side stream: on the caller's stream
  // just before use.
  struct OpFeed {
    std::vector<cudaEvent_t> ready;  // per position q: operators of order[q] complete
    cudaEvent_t freed[2] = {nullptr, nullptr};
  };

  cpx<R>* op_buffer(size_t q, int l) const {
    return L.cache_ops ? (cpx<R>*)(ws + L.op + L.op_one * (size_t)l) : (cpx<R>*)(ws + L.op + L.op_one * (q % 2));
  }

  int feed_begin(int pass, const std::vector<int>& order, const std::vector<double>& ds, OpFeed& f) {
    f.ready.assign(order.size(), nullptr);
    if (L.cache_ops && pass > 0) return DTMM_OK;  // reused
    if (st2 == nullptr) st2 = side_stream(st);
    if (st2 == nullptr) return DTMM_OK;
    int rc = wait_for(st2, st);  // inputs of the operators (setup, earlier passes)
    if (rc) return rc;
    const size_t n = L.cache_ops ? order.size() : std::min<size_t>(1, order.size());
    for (size_t q = 0; q < n; ++q)
      if ((rc = feed_one(q, order, ds, f))) return rc;
    return DTMM_OK;
  }

  int feed_one(size_t q, const std::vector<int>& order, const std::vector<double>& ds, OpFeed& f) {
    int rc;
    if (!L.cache_ops && q >= 2) CK(cudaStreamWaitEvent(st2, f.freed[q % 2], 0));
    if ((rc = voxel_ops(order[q], ds[q], op_buffer(q, order[q]), st2))) return rc;
    return record(st2, f.ready[q]);
  }

  // before layer position q: its operators (computed now on the caller's
  // stream when there is no side stream), the next layer's queued beside it
  int feed_get(int pass, size_t q, const std::vector<int>& order, const std::vector<double>& ds, OpFeed& f,
               const void*& op) {
    int rc;
    op = op_buffer(q, order[q]);
    if (L.cache_ops && pass > 0) return DTMM_OK;
    if (st2 == nullptr) return voxel_ops(order[q], ds[q], (cpx<R>*)op);
    if (!L.cache_ops && q + 1 < order.size() && (rc = feed_one(q + 1, order, ds, f))) return rc;
    CK(cudaStreamWaitEvent(st, f.ready[q], 0));
    return DTMM_OK;
  }

  // after layer position q has been queued: its buffer may be overwritten
  int feed_done(size_t q, OpFeed& f) {
    if (st2 == nullptr || L.cache_ops) return DTMM_OK;
    return record(st, f.freed[q % 2]);
  }

  // state F (real space, 4 components) -> propagated through all layers -> F
  int sweep4(int pass, cpx<R>* bulk) {
    const double dir = (pass % 2 == 0) ? 1.0 : -1.0;
    kdir = dir;
    std::vector<int> order;
    layer_order(pass % 2 == 0 ? 1 : -1, order);
    cpx<R>* F = P(L.F);
    cpx<R>* U = P(L.U);
    int rc;
    std::vector<double> dsub(order.size());
    for (size_t q = 0; q < order.size(); ++q) dsub[q] = d.thickness[order[q]] / d.nstep[order[q]];
    OpFeed feed;
    if ((rc = feed_begin(pass, order, dsub, feed))) return rc;
    if ((rc = launch_rows(F, 4, false, 1.0))) return rc;
    const cpx<R>* cur = F;
    double dprev = 0.0;
    for (size_t q = 0; q < order.size(); ++q) {
      const int l = order[q];
      const int nst = d.nstep[l];
      const double ds = dsub[q];
      const void* op;
      if ((rc = feed_get(pass, q, order, dsub, feed, op))) return rc;
      int kop;
      const void* ktab;
      const int bprev = cur_blk;
      cur_blk = blk_of(l);
      if (q == 0) {
        const cpx<R>* t1;
        if ((rc = table(KT_D1, dir * ds / 2, t1))) return rc;
        kop = KOP_MAT;
        ktab = t1;
      } else if (cur_blk != bprev) {
        // a boundary between blocks of different effective media: the two
        // half steps as one matrix per k
        const cpx<R>* t12;
        if ((rc = table(KT_D12, dir * ds / 2, t12, bprev, dir * dprev / 2))) return rc;
        kop = KOP_MAT;
        ktab = t12;
      } else {
        if ((rc = diag_table(dir * 0.5 * (dprev + ds)))) return rc;
        kop = KOP_DIAG;
        ktab = kdiag_cur;
      }
      cpx<R>* out = nullptr;
      if ((rc = layer(cur, 4, kop, ktab, 0, out, op, dir, nst, ds))) return rc;
      if ((rc = feed_done(q, feed))) return rc;
      // keep the layer result out of the buffers the next layer writes
      if (out != P(L.X) && q + 1 < order.size() && L.chains) {
        CK(cudaMemcpyAsync(P(L.X), out, sizeof(cpx<R>) * (size_t)NI * 4 * L.HW, cudaMemcpyDeviceToDevice, st));
        out = P(L.X);
      }
      cur = out;
      dprev = ds;
      if (bulk) {
        // bulk[l + 1] = ifft2(D2 . X) (dtmm/transfer.py:758-764, :878-880)
        cpx<R>* slab = bulk + (size_t)(l + 1) * NI * 4 * L.HW;
        const cpx<R>* t2;
        if ((rc = table(KT_D2, dir * ds / 2, t2))) return rc;
        if ((rc = launch_col(cur, slab, 4, 4, KOP_MAT, t2, 1, nullptr, true, true, 1.0 / d.height))) return rc;
        if ((rc = launch_rows(slab, 4, true, 1.0 / d.width))) return rc;
      }
    }
    const cpx<R>* t2;
    if ((rc = table(KT_D2, dir * dprev / 2, t2))) return rc;
    if ((rc = launch_col(cur, U, 4, 4, KOP_MAT, t2, 1, nullptr, true, true, 1.0 / d.height))) return rc;
    if ((rc = launch_rows(U, 4, true, 1.0 / d.width))) return rc;
    CK(cudaMemcpyAsync(F, U, sizeof(cpx<R>) * (size_t)NI * 4 * L.HW, cudaMemcpyDeviceToDevice, st));
    return DTMM_OK;
  }

  // per-image grid sums of the z-Poynting component of f into out[image]:
  // chunk sums of every image (as many chunks as the partials buffer holds,
  // at most 32), added in a fixed order
  int total_intensity(const cpx<R>* f, double* out) {
    const size_t cap = std::max<size_t>(2 * kPartBlocks, 4 * (size_t)kWinChunks * d.nray * L.nwin);
    const int chunks = (int)std::max<size_t>(1, std::min<size_t>(32, cap / (size_t)NI));
    k_total_intensity<R><<<dim3((unsigned)chunks, (unsigned)NI), 256, 0, st>>>(f, g, A<double>(L.part));
    CKL("k_total_intensity");
    k_total_sum<<<(NI + 255) / 256, 256, 0, st>>>(A<double>(L.part), chunks, out, NI);
    CKL("k_total_sum");
    return DTMM_OK;
  }

  // f (real space) -> notch * P . fft2(f) [with per-k normalisation] -> ifft2 -> f
  int project(cpx<R>* f, const cpx<R>* Ptab, bool normalize, double sigma) {
    int rc;
    cpx<R>* K = P(L.U);
    if ((rc = launch_rows(f, 4, false, 1.0))) return rc;
    if ((rc = launch_col(f, K, 4, 4, KOP_NONE, nullptr, 1, nullptr, true, false, 1.0))) return rc;
    NotchParams nt;
    nt.on = 1;
    nt.x0 = d.nin;
    nt.sigma = sigma;
    nt.den = 1.0 - std::exp(-d.nin / sigma);
    nt.ks = ks();
    const size_t n = (size_t)d.nlam * L.HW;  // one thread per (wavelength, k)
    k_kproject<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(K, Ptab, g, normalize ? 1 : 0, nt, nullptr);
    CKL("k_kproject");
    if ((rc = launch_col(K, f, 4, 4, KOP_NONE, nullptr, 1, nullptr, false, true, 1.0 / d.height))) return rc;
    return launch_rows(f, 4, true, 1.0 / d.width);
  }

  // f (real space) -> notch * fact * ifft2(P . fft2(f)) with fact the clamped
  // ratio of the total intensities of f and of the projection
  // (project_normalized_total, dtmm/transfer.py:123-155, then the notch of
  // denoise_field): the projection's intensity summed in k-space (the
  // Poynting form is sesquilinear, so the grid sum of a transform is H W times
  // the real-space sum)
  int project_total(cpx<R>* f, const cpx<R>* Ptab, double sigma) {
    int rc;
    cpx<R>* K = P(L.U);
    if ((rc = total_intensity(f, i0f()))) return rc;
    if ((rc = launch_rows(f, 4, false, 1.0))) return rc;
    if ((rc = launch_col(f, K, 4, 4, KOP_NONE, nullptr, 1, nullptr, true, false, 1.0))) return rc;
    NotchParams off;
    off.on = 0;
    off.den = 1.0;
    off.ks = ks();
    const size_t n = (size_t)d.nlam * L.HW;  // one thread per (wavelength, k)
    k_kproject<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(K, Ptab, g, 0, off, nullptr);
    CKL("k_kproject");
    if ((rc = total_intensity(K, fact()))) return rc;
    k_total_fact<<<(NI + 255) / 256, 256, 0, st>>>(i0f(), fact(), (double)L.HW, NI);
    CKL("k_total_fact");
    NotchParams nt;
    nt.on = 1;
    nt.x0 = d.nin;
    nt.sigma = sigma;
    nt.den = 1.0 - std::exp(-d.nin / sigma);
    nt.ks = ks();
    k_kscale<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(K, fact(), g, nt);
    CKL("k_kscale");
    if ((rc = launch_col(K, f, 4, 4, KOP_NONE, nullptr, 1, nullptr, false, true, 1.0 / d.height))) return rc;
    return launch_rows(f, 4, true, 1.0 / d.width);
  }

  // f <- ifft2(P . fft2(src))
  // ray_stride: elements between the tables of consecutive rays (0 = shared)
  int diffract(cpx<R>* f, const cpx<R>* src, const cpx<R>* Ptab, size_t ray_stride = 0, int C = 4) {
    int rc;
    const size_t bytes = sizeof(cpx<R>) * (size_t)NI * C * L.HW;
    if (f != src) CK(cudaMemcpyAsync(f, src, bytes, cudaMemcpyDeviceToDevice, st));
    if ((rc = launch_rows(f, C, false, 1.0))) return rc;
    if ((rc = launch_col(f, P(L.U), C, C, KOP_MAT, Ptab, 1, nullptr, true, true, 1.0 / d.height, ray_stride)))
      return rc;
    if ((rc = launch_rows(P(L.U), C, true, 1.0 / d.width))) return rc;
    CK(cudaMemcpyAsync(f, P(L.U), bytes, cudaMemcpyDeviceToDevice, st));
    return DTMM_OK;
  }

  int axpby(cpx<R>* out, const cpx<R>* x, const double* ax, double sx, const cpx<R>* y, const double* by, double sy,
            int C = 4) {
    const size_t n = (size_t)NI * C * L.HW;
    k_axpby<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, x, ax, sx, y, by, sy, g, C);
    CKL("k_axpby");
    return DTMM_OK;
  }

  int run4() {
    int rc;
    cpx<R>* fin = (cpx<R>*)io.field_in;
    cpx<R>* fout = (cpx<R>*)io.field_out;
    cpx<R>* F = P(L.F);
    const size_t bytes = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    const int npass = d.npass;
    // out= given: keep only its backward-propagating part (dtmm/transfer.py:674)
    if (io.out_given) {
      const cpx<R>* pback;
      if ((rc = table(KT_PROJ, 0.0, pback, -1, d.nin * d.nin))) return rc;
      if ((rc = diffract(fout, fout, pback))) return rc;
    } else {
      CK(cudaMemsetAsync(fout, 0, bytes, st));
    }
    cpx<R>* field0 = nullptr;
    const cpx<R>* pin = nullptr;
    const cpx<R>* pout = nullptr;
    // norm_ref: the reference field starts as the caller's input (dtmm/transfer.py:710-711)
    const bool use_ref = npass > 1 && d.norm_ref;
    cpx<R>* ref = use_ref ? P(L.ref) : nullptr;
    if (use_ref) CK(cudaMemcpyAsync(ref, fin, bytes, cudaMemcpyDeviceToDevice, st));
    if (npass > 1) {
      if ((rc = table(KT_PROJ, 0.0, pin, 1, d.nin * d.nin))) return rc;
      field0 = P(L.field0);
      if ((rc = diffract(field0, fin, pin))) return rc;
      if ((rc = total_intensity(field0, i0()))) return rc;
    }
    CK(cudaMemcpyAsync(F, fin, bytes, cudaMemcpyDeviceToDevice, st));
    cpx<R>* bulk = (cpx<R>*)io.bulk;
    // the real-space paths (no diffraction, or diffraction = inf) sweep F in
    // place; the reference's bulk slabs alias its pass-end field there, which
    // this path does not restate
    const bool real_space =
        d.diffraction == 0 || d.diffraction == DTMM_DIFFRACTION_FULL || d.reflection >= 2 || aniso_eff(&d);
    if (real_space && bulk && npass > 1)
      return fail(DTMM_ENOTSUP, "ret_bulk with npass > 1 is built for reflection mode 1 with diffraction >= 1");
    if (d.diffraction == DTMM_DIFFRACTION_FULL && (rc = full_prepare(fullp))) return rc;
    for (int i = 0; i < npass; ++i) {
      // the reference field goes through the even passes whose normalisation uses it
      if (use_ref && i % 2 == 0 && i != npass - 1 && (rc = ref_pass(ref))) return rc;
      if ((rc = real_space ? sweep_real4(i, bulk) : sweep4(i, bulk))) return rc;
      if (npass > 1) {
        const double sigma = d.smooth * (npass - i) / npass;
        if (i % 2 == 0) {
          if (i == 0 && (rc = axpby(F, F, nullptr, 1.0, fout, nullptr, -1.0))) return rc;
          if (i != npass - 1) {
            if ((rc = table(KT_PROJ, 0.0, pout, 1, d.nout * d.nout))) return rc;
            if (use_ref)
              rc = d.norm_total ? project_local(F, ref, pout, sigma) : project_ref(F, ref, pout, sigma);
            else
              rc = d.norm_total ? project_total(F, pout, sigma) : project(F, pout, true, sigma);
            if (rc) return rc;
          }
          if ((rc = axpby(fout, fout, nullptr, 1.0, F, nullptr, 1.0))) return rc;
          CK(cudaMemcpyAsync(F, fout, bytes, cudaMemcpyDeviceToDevice, st));
        } else {
          CK(cudaMemcpyAsync(fin, F, bytes, cudaMemcpyDeviceToDevice, st));
          if (i != npass - 1) {
            if ((rc = table(KT_PROJ, 0.0, pin, 1, d.nin * d.nin))) return rc;
            if ((rc = project(F, pin, false, sigma))) return rc;
            if ((rc = total_intensity(F, i0f()))) return rc;
            k_ratio<<<(NI + 255) / 256, 256, 0, st>>>(i0(), i0f(), fact(), NI);
            CKL("k_ratio");
            if ((rc = axpby(F, F, fact(), 1.0, nullptr, nullptr, 0.0))) return rc;
            if ((rc = axpby(fout, fout, fact(), 1.0, nullptr, nullptr, 0.0))) return rc;
            if ((rc = axpby(fin, fin, fact(), 1.0, nullptr, nullptr, 0.0))) return rc;
            if ((rc = axpby(F, field0, nullptr, 1.0, F, nullptr, -1.0))) return rc;
            if ((rc = axpby(fin, fin, nullptr, 1.0, F, nullptr, 1.0))) return rc;
            if (use_ref) CK(cudaMemcpyAsync(ref, F, bytes, cudaMemcpyDeviceToDevice, st));  // dtmm/transfer.py:868-869
          }
        }
      } else {
        CK(cudaMemcpyAsync(fout, F, bytes, cudaMemcpyDeviceToDevice, st));
      }
    }
    return DTMM_OK;
  }

  // The reference field of norm_ref (DTMM_NORM_FFT | DTMM_NORM_REF): its E
  // part through every layer of a forward pass as the 2x2 method's mode 2
  // without reflections (per window: E P E^-1 half steps around the
  // corrected E diffraction matrix, dtmm/transfer.py:770-775 with
  // dtmm/propagate_2x2.py:286-377), then its H part from E in the output
  // medium (jones2H, dtmm/transfer.py:805-806, :255-267).
  int ref_pass(cpx<R>* ref) {
    int rc = DTMM_OK;
    cpx<R>* E2 = P(L.ref2);
    cpx<R>* P2 = P(L.refw);
    cpx<R>* A2 = P2 + (size_t)NI * 2 * L.HW;
    cpx<R>* H2 = A2 + (size_t)NI * 2 * L.HW;
    const size_t n2 = (size_t)NI * 2 * L.HW;
    const size_t bytes2 = sizeof(cpx<R>) * n2;
    const size_t ray4 = (size_t)d.nlam * L.HW * 4;
    k_epart<R><<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(ref, E2, g);
    CKL("k_epart");
    Local2Params p = local2_params();
    p.mode = 1;
    p.lin = -1;
    chain_refl = 0;
    const int save_blk = cur_blk;
    for (int l = 0; l < d.nlayers; ++l) {
      cur_blk = blk_of(l);
      p.lout = l;
      const int nst = d.nstep[l];
      const double dd = d.thickness[l] / nst;
      if (L.nwin == 1) {
        if ((rc = chain2(p, 0, 0, nst, dd, E2, nullptr, nullptr))) break;
        continue;
      }
      CK(cudaMemsetAsync(A2, 0, bytes2, st));
      for (int w = 0; w < L.nwin; ++w) {
        const cpx<R>* wt;
        if ((rc = table(KT_2WIN, 0.0, wt, w))) break;
        if ((rc = diffract(P2, E2, wt, ray4, 2))) break;
        if ((rc = chain2(p, w, 0, nst, dd, P2, nullptr, nullptr))) break;
        if ((rc = axpby(A2, A2, nullptr, 1.0, P2, nullptr, 1.0, 2))) break;
      }
      if (rc) break;
      CK(cudaMemcpyAsync(E2, A2, bytes2, cudaMemcpyDeviceToDevice, st));
    }
    chain_refl = -1;
    cur_blk = save_blk;
    if (rc) return rc;
    const cpx<R>* th;
    if ((rc = table(KT_2H, 0.0, th, 1, d.nout * d.nout))) return rc;
    if ((rc = diffract(H2, E2, th, 0, 2))) return rc;
    k_join_eh<R><<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(ref, E2, H2, g);
    CKL("k_join_eh");
    return DTMM_OK;
  }

  // The even passes' normalisation with the reference field: ref scaled by
  // sqrt(nin / nout) in place, the intensities at each k from fft2(ref), and
  // -- as the reference's call, whose output array is the field, leaves it --
  // the projection of fft2(fft2(ref)) with the notch, back to real space in f
  // (dtmm/transfer.py:78-90, :824-834)
  int project_ref(cpx<R>* f, cpx<R>* ref, const cpx<R>* Ptab, double sigma) {
    int rc;
    cpx<R>* X = P(L.X);
    cpx<R>* U = P(L.U);
    const size_t bytes = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    if ((rc = axpby(ref, ref, nullptr, std::sqrt(d.nin / d.nout), nullptr, nullptr, 0.0))) return rc;
    CK(cudaMemcpyAsync(X, ref, bytes, cudaMemcpyDeviceToDevice, st));
    if ((rc = launch_rows(X, 4, false, 1.0))) return rc;
    if ((rc = launch_col(X, U, 4, 4, KOP_NONE, nullptr, 1, nullptr, true, false, 1.0))) return rc;  // U = fft2(ref)
    CK(cudaMemcpyAsync(X, U, bytes, cudaMemcpyDeviceToDevice, st));
    if ((rc = launch_rows(X, 4, false, 1.0))) return rc;
    if ((rc = launch_col(X, f, 4, 4, KOP_NONE, nullptr, 1, nullptr, true, false, 1.0))) return rc;  // f = fft2(U)
    NotchParams nt;
    nt.on = 1;
    nt.x0 = d.nin;
    nt.sigma = sigma;
    nt.den = 1.0 - std::exp(-d.nin / sigma);
    nt.ks = ks();
    const size_t n = (size_t)d.nlam * L.HW;
    k_kproject<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f, Ptab, g, 1, nt, U);
    CKL("k_kproject");
    if ((rc = launch_col(f, X, 4, 4, KOP_NONE, nullptr, 1, nullptr, false, true, 1.0 / d.height))) return rc;
    if ((rc = launch_rows(X, 4, true, 1.0 / d.width))) return rc;
    CK(cudaMemcpyAsync(f, X, bytes, cudaMemcpyDeviceToDevice, st));
    return DTMM_OK;
  }

  // The "local" normalisation with the reference field (norm_ref with
  // norm_total, the reference's DTMM_NORM_REF alone): f projected in k-space
  // (no per-k normalisation), per pixel the polarizer split of the
  // reference field (k_local_norm), then the notch (dtmm/transfer.py:103-136,
  // :824-835)
  int project_local(cpx<R>* f, cpx<R>* ref, const cpx<R>* Ptab, double sigma) {
    int rc;
    cpx<R>* K = P(L.U);
    const size_t n = (size_t)d.nlam * L.HW;
    const size_t npix = (size_t)NI * L.HW;
    if ((rc = axpby(ref, ref, nullptr, std::sqrt(d.nin / d.nout), nullptr, nullptr, 0.0))) return rc;
    if ((rc = launch_rows(f, 4, false, 1.0))) return rc;
    if ((rc = launch_col(f, K, 4, 4, KOP_NONE, nullptr, 1, nullptr, true, false, 1.0))) return rc;
    NotchParams off;
    off.on = 0;
    off.den = 1.0;
    off.ks = ks();
    k_kproject<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(K, Ptab, g, 0, off, nullptr);
    CKL("k_kproject");
    if ((rc = launch_col(K, f, 4, 4, KOP_NONE, nullptr, 1, nullptr, false, true, 1.0 / d.height))) return rc;
    if ((rc = launch_rows(f, 4, true, 1.0 / d.width))) return rc;
    cpx<double>* fn = A<cpx<double>>(L.fnorm);
    k_iso_fnorm<<<1, 32, 0, st>>>(d.nout * d.nout, fn);
    CKL("k_iso_fnorm");
    k_local_norm<R><<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(f, ref, fn, g);
    CKL("k_local_norm");
    // the notch of denoise_field
    if ((rc = launch_rows(f, 4, false, 1.0))) return rc;
    if ((rc = launch_col(f, K, 4, 4, KOP_NONE, nullptr, 1, nullptr, true, false, 1.0))) return rc;
    NotchParams nt;
    nt.on = 1;
    nt.x0 = d.nin;
    nt.sigma = sigma;
    nt.den = 1.0 - std::exp(-d.nin / sigma);
    nt.ks = ks();
    k_kscale<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(K, nullptr, g, nt);
    CKL("k_kscale");
    if ((rc = launch_col(K, f, 4, 4, KOP_NONE, nullptr, 1, nullptr, false, true, 1.0 / d.height))) return rc;
    return launch_rows(f, 4, true, 1.0 / d.width);
  }

  // byte offset of the backward-mode records in a voxel's operator records
  size_t back_records() const { return (size_t)REC_BLOCK * (real_ops() ? sizeof(R) : sizeof(cpx<R>)); }

  // 2x2 method in k-space (reflection 0 or 1; dtmm/propagate_2x2.py:19-87,
  // :193-284 driven by dtmm/transfer.py:1074-1183) over npass passes that
  // alternate in direction.  The inner interfaces join identical effective
  // media (t = 1, r = 0 within betamax), so with npass > 1 only the reflected
  // waves of the two outer interfaces are kept between passes, x-transformed
  // ([image][2][H][W], rows along x in k-space): each pass after the first
  // enters the stack with the wave its entry interface reflected in the
  // previous pass; forward passes add the field leaving the stack to
  // field_out, backward passes to field_in, which first becomes the input's
  // forward part (dtmm/transfer.py:1075-1080).  Without diffraction
  // (reflection 1) the voxels' operators are the plain E P E^-1 and the
  // k-space steps only the interfaces' betamax cut.
  int run2() {
    int rc;
    cpx<R>* fin = (cpx<R>*)io.field_in;
    cpx<R>* fout = (cpx<R>*)io.field_out;
    cpx<R>* F = P(L.F);
    cpx<R>* U = P(L.U);
    const size_t bytes4 = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    const size_t bytes2 = bytes4 / 2;
    const int npass = d.npass;
    const double hd = d.diffraction == 0 ? 0.0 : 1.0;  // half steps of the effective medium
    const size_t ray8 = (size_t)d.nlam * L.HW * 8, ray4 = (size_t)d.nlam * L.HW * 4;
    const double ih = 1.0 / d.height, iw = 1.0 / d.width;
    cpx<R>* Rin = npass > 1 ? P(L.r2in) : nullptr;
    cpx<R>* Rout = npass > 1 ? P(L.r2out) : nullptr;
    // ret_bulk (no windows): slab l + 1 collects block layer l's field and its
    // H part, E2H of the voxel for the ray's beam (dtmm/propagate_2x2.py:48-53, :80-85)
    cpx<R>* bulk = (cpx<R>*)io.bulk;
    const size_t n4 = (size_t)NI * 4 * L.HW;
    if (bulk) CK(cudaMemsetAsync(bulk + n4, 0, bytes4 * (size_t)d.nlayers, st));
    Local2Params pb = local2_params();
    pb.beta = rbeta();
    pb.phi = rphi();
    pb.bstride = 1;
    // the layer's field in real space (x-transformed state through its half
    // step E(dh) of mode `mode`, or as it is) added to its slab
    auto bulk_add = [&](int l, int mode, const cpx<R>* xs, double dh, bool half) -> int {
      int rc2;
      if (half) {
        const cpx<R>* te;
        if ((rc2 = table(KT_2E, dh, te, mode))) return rc2;
        if ((rc2 = launch_col(xs, U, 2, 2, KOP_MAT, te, 1, nullptr, true, true, 1.0 / d.height))) return rc2;
      } else {
        CK(cudaMemcpyAsync(U, xs, bytes4 / 2, cudaMemcpyDeviceToDevice, st));
      }
      if ((rc2 = launch_rows(U, 2, true, 1.0 / d.width))) return rc2;
      pb.lout = l;
      pb.mode = mode;
      return local2(pb, L2_BULK, U, nullptr, bulk + (size_t)(l + 1) * n4);
    };
    if (npass > 1) {
      const cpx<R>* pin;
      if ((rc = table(KT_PROJ, 0.0, pin, 1, d.nin * d.nin))) return rc;
      if ((rc = diffract(fin, fin, pin))) return rc;
    }
    kdir = hd;
    for (int i = 0; i < npass; ++i) {
      const int dir = i % 2 == 0 ? 1 : -1;
      std::vector<int> order;
      layer_order(dir, order);
      std::vector<double> dsub(order.size());
      for (size_t q = 0; q < order.size(); ++q) dsub[q] = d.thickness[order[q]] / d.nstep[order[q]];
      OpFeed feed;
      if ((rc = feed_begin(i, order, dsub, feed))) return rc;
      const cpx<R>* cur = F;
      int cin;
      const cpx<R>* t1;
      if (i == 0) {
        // entry: the input's forward part through the interface n_in -> effective,
        // half step; its reflection kept for the next pass
        CK(cudaMemcpyAsync(F, fin, bytes4, cudaMemcpyDeviceToDevice, st));
        if (d.diffraction == 0) {
          k_project_beam<R><<<dim3((unsigned)((L.HW + 127) / 128), (unsigned)d.nray), 128, 0, st>>>(
              F, rbeta(), rphi(), d.nin * d.nin, g);
          CKL("k_project_beam");
        }
        if ((rc = launch_rows(F, 4, false, 1.0))) return rc;
        if (npass > 1) {
          const cpx<R>* rt;
          if ((rc = table(KT_2RIN, 0.0, rt))) return rc;
          if ((rc = launch_col(F, Rin, 4, 2, KOP_MAT, rt, 1, nullptr, true, true, ih, ray8))) return rc;
        }
        cur_blk = blk_of(order[0]);
        if ((rc = table(KT_2IN, hd * dsub[0] / 2, t1))) return rc;
        cin = 4;
      } else {
        // entry: the wave reflected back into the stack in the previous pass
        cpx<R>* Rs = dir > 0 ? Rin : Rout;
        CK(cudaMemcpyAsync(F, Rs, bytes2, cudaMemcpyDeviceToDevice, st));
        cur_blk = blk_of(order[0]);
        if ((rc = table(KT_2E, dir * hd * dsub[0] / 2, t1, dir))) return rc;
        cin = 2;
      }
      double dprev = 0.0;
      for (size_t q = 0; q < order.size(); ++q) {
        const int l = order[q];
        const double ds = dsub[q];
        // backward: the field entering layer l from above (the reflected wave
        // at the top, else the layer above through its half step)
        if (bulk && dir < 0 && (rc = bulk_add(l, -1, cur, -hd * dprev / 2, q > 0))) return rc;
        const void* op;
        if ((rc = feed_get(i, q, order, dsub, feed, op))) return rc;
        if (dir < 0) op = (const char*)op + back_records();
        int kop;
        const void* ktab;
        const int bprev = cur_blk;
        cur_blk = blk_of(l);
        if (q == 0) {
          kop = KOP_MAT;
          ktab = t1;
        } else if (cur_blk != bprev) {
          // a boundary between blocks: half step, interface between the two
          // effective media, half step (npass 1)
          const cpx<R>* tb;
          if ((rc = table(KT_2BX, hd * ds / 2, tb, bprev, hd * dprev / 2))) return rc;
          kop = KOP_MAT;
          ktab = tb;
        } else {
          if ((rc = diag_table(hd * 0.5 * (dprev + ds)))) return rc;
          kop = KOP_DIAG;
          ktab = kdiag_cur;
        }
        cpx<R>* out = nullptr;
        if ((rc = layer(cur, cin, kop, ktab, 0, out, op, (double)dir, d.nstep[l], ds))) return rc;
        if ((rc = feed_done(q, feed))) return rc;
        if (out != P(L.X) && q + 1 < order.size() && L.chains) {
          CK(cudaMemcpyAsync(P(L.X), out, bytes2, cudaMemcpyDeviceToDevice, st));
          out = P(L.X);
        }
        cur = out;
        cin = 2;
        dprev = ds;
        if (bulk && dir > 0 && (rc = bulk_add(l, 1, cur, hd * ds / 2, true))) return rc;
      }
      if (dir > 0) {
        // exit: half step, interface effective -> n_out, windows and E -> H, into field_out
        const cpx<R>* t2;
        if ((rc = table(KT_2OUT, hd * dprev / 2, t2, 1))) return rc;
        if ((rc = launch_col(cur, U, 2, 4, KOP_MAT, t2, 1, nullptr, true, true, ih, ray8))) return rc;
        if ((rc = launch_rows(U, 4, true, iw))) return rc;
        if (i == 0)
          CK(cudaMemcpyAsync(fout, U, bytes4, cudaMemcpyDeviceToDevice, st));
        else if ((rc = axpby(fout, fout, nullptr, 1.0, U, nullptr, 1.0)))
          return rc;
        if (i + 1 < npass) {  // the wave the exit interface reflects back
          const cpx<R>* tr;
          if ((rc = table(KT_2R, hd * dprev / 2, tr, 1))) return rc;
          if ((rc = launch_col(cur, Rout, 2, 2, KOP_MAT, tr, 1, nullptr, true, true, ih, ray4))) return rc;
        }
      } else {
        // exit into n_in: t . (half step) + the input's reflection kept at the
        // entry, windows and E -> H of the backward modes, added to field_in
        cpx<R>* Y = P(L.y2);
        const cpx<R>* te;
        if ((rc = table(KT_2TE, -hd * dprev / 2, te, -1))) return rc;
        if ((rc = launch_col(cur, Y, 2, 2, KOP_MAT, te, 1, nullptr, true, true, ih))) return rc;
        if ((rc = axpby(Y, Y, nullptr, 1.0, Rin, nullptr, 1.0, 2))) return rc;
        if (i + 1 < npass) {
          const cpx<R>* tr;
          if ((rc = table(KT_2R, -hd * dprev / 2, tr, -1))) return rc;
          if ((rc = launch_col(cur, Rin, 2, 2, KOP_MAT, tr, 1, nullptr, true, true, ih, ray4))) return rc;
        }
        const cpx<R>* tx;
        if ((rc = table(KT_2X, 0.0, tx, -1))) return rc;
        if ((rc = launch_col(Y, U, 2, 4, KOP_MAT, tx, 1, nullptr, true, true, ih, ray8))) return rc;
        if ((rc = launch_rows(U, 4, true, iw))) return rc;
        if ((rc = axpby(fin, fin, nullptr, 1.0, U, nullptr, 1.0))) return rc;
      }
    }
    return DTMM_OK;
  }

  // 2x2 method in real space: reflection mode 2 (per-voxel interfaces and the
  // corrected E diffraction matrix between half steps, n x n windows each
  // through its own chain; dtmm/propagate_2x2.py:91-190, :286-377) and no
  // diffraction without reflections (the voxels' E P E^-1 alone).  The layer
  // list is n_in, the block's layers, n_out (dtmm/transfer.py:926-1005); with
  // npass > 1 every interface keeps its reflected wave between passes.
  Local2Params local2_params() {
    Local2Params p;
    p.epsv = d.epsv;
    p.epsa = d.epsa;
    for (int i = 0; i < 3; ++i) {
      p.ev_s[i] = d.epsv_strides[i];
      p.ea_s[i] = d.epsa_strides[i];
    }
    p.eps_complex = d.eps_complex;
    p.nin2 = d.nin * d.nin;
    p.nout2 = d.nout * d.nout;
    p.ks = ks();
    p.reps = 1;
    p.dzero = 0;
    return p;
  }

  int local2(Local2Params& p, int op, cpx<R>* f, cpx<R>* refl, cpx<R>* bulk) {
    p.op = op;
    const dim3 grid((unsigned)((L.HW + 127) / 128), (unsigned)d.nray);
    k_local2<R><<<grid, 128, 0, st>>>(p, g, f, refl, bulk);
    CKL("k_local2");
    return DTMM_OK;
  }

  // one interface call of the reference's _transfer_ray_2x2_2 on f (its
  // window's part): dd the signed sub-step thickness of the output layer
  // bo: the field array of the output layer jout (field_in, field_out or a
  // bulk slab) that the reference adds the layer's field to, or null
  // the interface step of chain2 (-1: the descriptor's reflection mode; 0:
  // none, for the 4x4 method's reference field)
  int chain_refl = -1;

  // one interface call of the reference's _transfer_ray_2x2_1 with reflection
  // 0 (dtmm/propagate_2x2.py:19-87, :193-284; its k-space field here in real
  // space, every step being linear) on f, its window's part: per sub-step
  // C . E(dd/2) per k, E P E^-1 of the output voxel over dd, E(dd/2) . C per k;
  // then the layer's E and H parts into bo
  int chain2k(Local2Params& p, int w, int nst, double dd, cpx<R>* f, cpx<R>* bo) {
    int rc;
    p.beta = wbeta() + w;
    p.phi = wphi() + w;
    p.bstride = L.nwin;
    const size_t ray4 = (size_t)d.nlam * L.HW * 4;
    const int pm = 2 * w + (p.mode < 0 ? 1 : 0);
    for (int s = 0; s < nst; ++s) {
      const cpx<R>* t1;
      const cpx<R>* t2;
      if ((rc = table(KT_2C1, dd / 2, t1, pm))) return rc;
      if ((rc = diffract(f, f, t1, ray4, 2))) return rc;
      if (dd != 0.0) {
        p.d = dd;
        p.reps = 1;
        if ((rc = local2(p, L2_HALF, f, nullptr, nullptr))) return rc;
      }
      if ((rc = table(KT_2C2, dd / 2, t2, pm))) return rc;
      if ((rc = diffract(f, f, t2, ray4, 2))) return rc;
    }
    if (p.mode > 0 && bo != nullptr) return local2(p, L2_BULK, f, nullptr, bo);
    return DTMM_OK;
  }

  int chain2(Local2Params& p, int w, int jout, int nst, double dd, cpx<R>* f, cpx<R>* r, cpx<R>* bo) {
    const int refl_mode = chain_refl >= 0 ? chain_refl : d.reflection;
    int rc;
    const bool tracked = r != nullptr;
    p.beta = wbeta() + w;
    p.phi = wphi() + w;
    p.bstride = L.nwin;
    p.d = dd / 2;
    const bool zero = dd == 0.0;
    const size_t ray4 = (size_t)d.nlam * L.HW * 4;
    for (int s = 0; s < nst; ++s) {
      if (s == 0 && refl_mode != 0) {
        p.dzero = zero ? 1 : 0;
        rc = local2(p, tracked ? L2_TR : L2_ETI, f, r, (tracked && p.mode < 0) ? bo : nullptr);
        p.dzero = 0;
        if (rc) return rc;
      } else if (!zero) {
        p.reps = d.diffraction == 0 ? 2 : 1;  // both halves at once without a diffraction step between
        rc = local2(p, L2_HALF, f, nullptr, nullptr);
        p.reps = 1;
        if (rc) return rc;
        if (d.diffraction == 0) continue;
      }
      if (d.diffraction > 0) {
        const cpx<R>* ce;
        if ((rc = table(KT_2CE, dd, ce, 2 * w + (p.mode < 0 ? 1 : 0)))) return rc;
        if ((rc = diffract(f, f, ce, ray4, 2))) return rc;
      }
      if (!zero && (rc = local2(p, L2_HALF, f, nullptr, nullptr))) return rc;
    }
    (void)jout;
    if (p.mode > 0 && bo != nullptr) return local2(p, L2_BULK, f, nullptr, bo);
    return DTMM_OK;
  }

  int run2_real() {
    int rc;
    cpx<R>* fin = (cpx<R>*)io.field_in;
    cpx<R>* fout = (cpx<R>*)io.field_out;
    cpx<R>* F2 = P(L.F);
    cpx<R>* G4 = P(L.X);
    const size_t bytes4 = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    const size_t bytes2 = bytes4 / 2;
    const size_t n2 = (size_t)NI * 2 * L.HW, n4 = 2 * n2;
    const int npass = d.npass;
    const int n = d.nlayers + 1;  // interfaces
    const bool tracked = npass > 1;
    cpx<R>* refl = tracked ? P(L.r2) : nullptr;
    if (tracked) CK(cudaMemsetAsync(refl, 0, bytes2 * (size_t)n, st));
    // the input's forward part: per k in the input medium, or for the beam
    // direction without diffraction (dtmm/transfer.py:1075-1078)
    if (d.diffraction > 0) {
      const cpx<R>* pin;
      if ((rc = table(KT_PROJ, 0.0, pin, 1, d.nin * d.nin))) return rc;
      if ((rc = diffract(G4, fin, pin))) return rc;
    } else {
      CK(cudaMemcpyAsync(G4, fin, bytes4, cudaMemcpyDeviceToDevice, st));
      k_project_beam<R><<<dim3((unsigned)((L.HW + 127) / 128), (unsigned)d.nray), 128, 0, st>>>(
          G4, rbeta(), rphi(), d.nin * d.nin, g);
      CKL("k_project_beam");
    }
    if (tracked) CK(cudaMemcpyAsync(fin, G4, bytes4, cudaMemcpyDeviceToDevice, st));
    k_epart<R><<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(G4, F2, g);
    CKL("k_epart");
    CK(cudaMemsetAsync(fout, 0, bytes4, st));
    // ret_bulk: slab k of the layer list (0 field_in, n field_out) collects
    // the fields of its layer; the block's slabs start at zero
    cpx<R>* bulk = (cpx<R>*)io.bulk;
    if (bulk) CK(cudaMemsetAsync(bulk + n4, 0, bytes4 * (size_t)d.nlayers, st));
    auto bslab = [&](int k) -> cpx<R>* {
      if (k == 0) return fin;
      if (k == n) return fout;
      return bulk ? bulk + (size_t)k * n4 : nullptr;
    };
    Local2Params p = local2_params();
    const bool win = L.nwin > 1;
    cpx<R>* P2 = win ? P(L.w2) : nullptr;
    cpx<R>* A2 = win ? P2 + n2 : nullptr;
    cpx<R>* RP = win ? A2 + n2 : nullptr;
    cpx<R>* RA = win ? RP + n2 : nullptr;
    const size_t ray4 = (size_t)d.nlam * L.HW * 4;
    for (int i = 0; i < npass; ++i) {
      const int dir = i % 2 == 0 ? 1 : -1;
      if (i > 0) CK(cudaMemsetAsync(F2, 0, bytes2, st));
      p.mode = dir;
      for (int q = 0; q < n; ++q) {
        const int j = dir > 0 ? q : n - 1 - q;
        const int jin = dir > 0 ? j : j + 1, jout = dir > 0 ? j + 1 : j;
        // layer list index -> layer of the block (-1 input medium, -2 output medium)
        auto lay = [&](int k) { return k == 0 ? -1 : (k == n ? -2 : k - 1); };
        p.lin = lay(jin);
        p.lout = lay(jout);
        const bool inner = p.lout >= 0;
        if (inner) cur_blk = blk_of(p.lout);  // boundary layers have no thickness: any block's medium
        const int nst = inner ? d.nstep[p.lout] : 1;
        const double dd = inner ? dir * d.thickness[p.lout] / d.nstep[p.lout] : 0.0;
        cpx<R>* Rj = tracked ? refl + (size_t)j * n2 : nullptr;
        cpx<R>* bo = bslab(jout);
        // reflection 0 with diffraction: the reference's k-space step
        const bool kstep = d.reflection == 0 && d.diffraction >= 1;
        if (!win) {
          if ((rc = kstep ? chain2k(p, 0, nst, dd, F2, bo) : chain2(p, 0, jout, nst, dd, F2, Rj, bo))) return rc;
          continue;
        }
        CK(cudaMemsetAsync(A2, 0, bytes2, st));
        if (tracked) CK(cudaMemsetAsync(RA, 0, bytes2, st));
        for (int w = 0; w < L.nwin; ++w) {
          const cpx<R>* wt;
          if ((rc = table(KT_2WIN, 0.0, wt, w))) return rc;
          if ((rc = diffract(P2, F2, wt, ray4, 2))) return rc;
          if (tracked && (rc = diffract(RP, Rj, wt, ray4, 2))) return rc;
          if ((rc = kstep ? chain2k(p, w, nst, dd, P2, bo) : chain2(p, w, jout, nst, dd, P2, tracked ? RP : nullptr, bo)))
            return rc;
          if ((rc = axpby(A2, A2, nullptr, 1.0, P2, nullptr, 1.0, 2))) return rc;
          if (tracked && (rc = axpby(RA, RA, nullptr, 1.0, RP, nullptr, 1.0, 2))) return rc;
        }
        CK(cudaMemcpyAsync(F2, A2, bytes2, cudaMemcpyDeviceToDevice, st));
        if (tracked) CK(cudaMemcpyAsync(Rj, RA, bytes2, cudaMemcpyDeviceToDevice, st));
      }
    }
    return DTMM_OK;
  }

  // mode amplitudes (FP64, in order of increasing beta) of the 2-component
  // field f into amp: the row DFT at the in-band columns, then the column DFT
  int full_amps2(const cpx<R>* f, cpx<double>* amp) {
    cpx<double>* Ab = A<cpx<double>>(L.fA);
    k_full_rowdft<R><<<dim3((unsigned)d.height, (unsigned)(NI * 2)), 128, 0, st>>>(fullp, g, f, Ab);
    CKL("k_full_rowdft");
    k_full_coldft<<<dim3((unsigned)((L.HW + 127) / 128), (unsigned)(NI * 2)), 128, 0, st>>>(fullp, g, Ab, amp);
    CKL("k_full_coldft");
    return DTMM_OK;
  }

  // 2x2 with diffraction = inf (dtmm/transfer.py:1009-1183 with
  // dtmm/propagate_2x2.py:379-464): the input's forward part per k in the
  // input medium, then per pass and interface (layer list n_in, the layers,
  // n_out) one modal step over the output layer's sub-step thickness d / nstep
  // (the reference takes one), through the interface with reflection 2; with
  // npass > 1 every interface keeps its reflected wave between passes.  The
  // field of each output layer is added to its slab (field_in, field_out or
  // the bulk output).
  int run2_full() {
    int rc;
    cpx<R>* fin = (cpx<R>*)io.field_in;
    cpx<R>* fout = (cpx<R>*)io.field_out;
    cpx<R>* F2 = P(L.F);
    cpx<R>* G4 = P(L.X);
    const size_t bytes4 = sizeof(cpx<R>) * (size_t)NI * 4 * L.HW;
    const size_t bytes2 = bytes4 / 2;
    const size_t n2 = (size_t)NI * 2 * L.HW, n4 = 2 * n2;
    const int n = d.nlayers + 1;  // interfaces
    const bool tracked = d.npass > 1;
    cpx<R>* refl = tracked ? P(L.r2) : nullptr;
    if (tracked) CK(cudaMemsetAsync(refl, 0, bytes2 * (size_t)n, st));
    const cpx<R>* pin;
    if ((rc = table(KT_PROJ, 0.0, pin, 1, d.nin * d.nin))) return rc;
    if ((rc = diffract(G4, fin, pin))) return rc;
    if (tracked) CK(cudaMemcpyAsync(fin, G4, bytes4, cudaMemcpyDeviceToDevice, st));
    k_epart<R><<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(G4, F2, g);
    CKL("k_epart");
    CK(cudaMemsetAsync(fout, 0, bytes4, st));
    cpx<R>* bulk = (cpx<R>*)io.bulk;
    if (bulk) CK(cudaMemsetAsync(bulk + n4, 0, bytes4 * (size_t)d.nlayers, st));
    auto bslab = [&](int k) -> cpx<R>* {
      if (k == 0) return fin;
      if (k == n) return fout;
      return bulk ? bulk + (size_t)k * n4 : nullptr;
    };
    if ((rc = full_prepare(fullp))) return rc;
    cpx<double>* amp = A<cpx<double>>(L.famp);
    cpx<double>* tamp = amp + n2;
    Local2Params p = local2_params();
    p.op = d.reflection != 0;
    const dim3 gk((unsigned)((L.HW + 127) / 128), (unsigned)d.nlam);
    for (int i = 0; i < d.npass; ++i) {
      const int dir = i % 2 == 0 ? 1 : -1;
      if (i > 0) CK(cudaMemsetAsync(F2, 0, bytes2, st));
      p.mode = dir;
      for (int q = 0; q < n; ++q) {
        const int j = dir > 0 ? q : n - 1 - q;
        const int jin = dir > 0 ? j : j + 1, jout = dir > 0 ? j + 1 : j;
        auto lay = [&](int k) { return k == 0 ? -1 : (k == n ? -2 : k - 1); };
        p.lin = lay(jin);
        p.lout = lay(jout);
        p.d = p.lout >= 0 ? dir * d.thickness[p.lout] / d.nstep[p.lout] : 0.0;
        cpx<R>* Rj = tracked ? refl + (size_t)j * n2 : nullptr;
        if ((rc = full_amps2(F2, amp))) return rc;
        if (tracked && (rc = full_amps2(Rj, tamp))) return rc;
        k_full2_apply<R><<<gk, 128, 0, st>>>(fullp, p, g, amp, tracked ? tamp : nullptr, F2, Rj, bslab(jout));
        CKL("k_full2_apply");
      }
    }
    return DTMM_OK;
  }
};

template <typename R>
int run_engine(const dtmm_transfer_desc* d, const dtmm_transfer_io* io, void* ws, const Layout& L, cudaStream_t st,
               Prof* prof, int* launches) {
  Engine<R> e(*d, *io, L, (unsigned char*)ws, st);
  e.prof = prof;
  e.g.H = d->height;
  e.g.W = d->width;
  e.NI = d->nray * d->npol * d->nlam;
  e.g.NI = e.NI;
  e.g.nlam = d->nlam;
  e.g.npol = d->npol;
  e.g.nray = d->nray;
  make_plan(d->height, e.pH, d->fft_schedule == 3);
  make_plan(d->width, e.pW, d->fft_schedule == 3);
  int rc;
  if (d->method == 4 && d->diffraction == 0 && d->npass == 1) {
    rc = e.run_local4();
  } else if (d->method == 4 && d->diffraction == DTMM_DIFFRACTION_FULL && d->npass == 1) {
    rc = e.run_full4();
  } else {
    rc = e.setup();
    if (rc == DTMM_OK) {
      if (d->method == 4)
        rc = e.run4();
      else if (d->diffraction == DTMM_DIFFRACTION_FULL)
        rc = e.run2_full();
      else
        rc = is_real2(d) ? e.run2_real() : e.run2();
    }
  }
  if (launches) *launches = e.launches;
  return rc;
}

// ---------------------------------------------------------------------------
// diffract (dtmm/diffract.py:254-299) in real space: fft2 -> per-k 4x4 matrix
// -> ifft2, with the transfer's own row and column kernels
// ---------------------------------------------------------------------------
struct DiffractLayout {
  size_t twH, permH, twW, permW, dmat, X, total;
};

DiffractLayout diffract_layout(int H, int W, int nimg, int nlam, int precision) {
  DiffractLayout L{};
  const size_t cplx = precision == DTMM_PRECISION_DOUBLE ? 16 : 8;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  L.twH = take(cplx * H);
  L.permH = take(sizeof(int) * H);
  L.twW = take(cplx * W);
  L.permW = take(sizeof(int) * W);
  L.dmat = precision == DTMM_PRECISION_DOUBLE ? 0 : take(cplx * 16 * (size_t)nlam * H * W);
  L.X = take(cplx * 4 * (size_t)nimg * H * W);
  L.total = off;
  return L;
}

int check_diffract(int H, int W, int nimg, int nlam, int precision) {
  if (H < 1 || W < 1 || nimg < 1 || nlam < 1) return fail(DTMM_EINVAL, "empty axis");
  if (nimg % nlam) return fail(DTMM_EINVAL, "image count must be a multiple of the wavelength count");
  if (nimg > 65535) return fail(DTMM_EINVAL, "too many images");
  if (precision != DTMM_PRECISION_MIXED && precision != DTMM_PRECISION_DOUBLE)
    return fail(DTMM_EINVAL, "invalid precision");
  FFTPlan p;
  if (!make_plan(H, p) || !make_plan(W, p))
    return fail(DTMM_ENOTSUP, "grid sides must factor into primes up to 31 (got %dx%d)", H, W);
  return DTMM_OK;
}

template <typename R>
int diffract_impl(int H, int W, int nimg, int nlam, const void* dmat, const void* in, void* out, unsigned char* ws,
                  const DiffractLayout& L, cudaStream_t st) {
  int launches = 0;
  FFTPlan pH, pW;
  make_plan(H, pH);
  make_plan(W, pW);
  cpx<R>* twH = (cpx<R>*)(ws + L.twH);
  cpx<R>* twW = (cpx<R>*)(ws + L.twW);
  int* permH = (int*)(ws + L.permH);
  int* permW = (int*)(ws + L.permW);
  k_fft_tables<R><<<(H + 255) / 256, 256, 0, st>>>(pH, twH, permH);
  CKL("k_fft_tables");
  k_fft_tables<R><<<(W + 255) / 256, 256, 0, st>>>(pW, twW, permW);
  CKL("k_fft_tables");
  const cpx<R>* tab = (const cpx<R>*)dmat;
  if (sizeof(R) == 4) {
    const size_t n = 16 * (size_t)nlam * H * W;
    k_convert<R, double><<<(unsigned)((n + 255) / 256), 256, 0, st>>>((cpx<R>*)(ws + L.dmat),
                                                                       (const cpx<double>*)dmat, n);
    CKL("k_convert");
    tab = (const cpx<R>*)(ws + L.dmat);
  }
  cpx<R>* X = (cpx<R>*)(ws + L.X);
  // rows forward (natural in and out), out of place into the workspace
  const int nlines = nimg * 4 * H;
  const bool rrows = sizeof(R) == 4 && reg_lanes(W) > 0;
  RegLaunch rl;
  if (rrows) {
    const int n1 = reg_lanes(W), rlpb = 256 / n1;
    rl.threads = rlpb * n1;
    rl.smem = (size_t)(W + rlpb * reg_row_stride(n1, W)) * sizeof(cpx<R>);
    rl.grid = dim3((unsigned)((nlines + rlpb - 1) / rlpb));
    rl.st = st;
  }
  int lpb = std::max(1, std::min(16, 4096 / W));
  size_t smem = (size_t)lpb * W * sizeof(cpx<R>) + W * (sizeof(cpx<R>) + sizeof(int));
  if (smem > 220 * 1024) return fail(DTMM_ENOTSUP, "row of %d pixels too large for one block", W);
  if (rrows) {
    const cudaError_t e = fft_rows_reg_dispatch(W, false, rl, in, X, nlines, twW, 1.0f);
    ++launches;
    if (e != cudaSuccess) return fail(DTMM_ECUDA, "launch k_fft_rows_reg: %s", cudaGetErrorString(e));
  } else {
    CK(cudaFuncSetAttribute(k_fft_rows<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_rows<R, false><<<(nlines + lpb - 1) / lpb, 256, smem, st>>>((const cpx<R>*)in, X, nlines, W, pW, twW,
                                                                      permW, 1.0, lpb);
    CKL("k_fft_rows");
  }
  // columns: forward transform, the per-k matrix, inverse transform (1/H)
  Grid g;
  g.H = H;
  g.W = W;
  g.NI = nimg;
  g.nlam = nlam;
  g.npol = 1;
  g.nray = nimg / nlam;
  ColParams p;
  memset(&p, 0, sizeof(p));
  p.cin = p.cout = 4;
  p.kop = KOP_MAT;
  p.ktab = tab;
  p.ktab_ray_stride = 0;
  p.ny = 1;
  p.cy = nullptr;
  p.j_only = -1;
  p.cy_rows = 1;
  p.do_fwd = 1;
  p.inverse_out = 1;
  p.out_scale = 1.0 / H;
  p.plan = pH;
  p.tw = twH;
  p.perm = permH;
  if (sizeof(R) == 4 && reg_lanes(H) > 0) {
    // register column transforms with the matrix exchanged through the tile
    const int n1 = reg_lanes(H);
    const size_t tiles = reg_col_tiles(H, 1);
    int tx = std::max(1, 256 / (4 * n1));
    if (tx > W) tx = W;
    while (tx > 1 && tiles * H * (4 * tx + 1) * sizeof(cpx<R>) > 100 * 1024) tx /= 2;
    p.tc = tx;
    RegLaunch cl;
    cl.smem = tiles * H * (4 * tx + 1) * sizeof(cpx<R>) + H * sizeof(cpx<R>);
    cl.threads = std::max(32, ((4 * tx * n1 + 31) / 32) * 32);
    cl.grid = dim3((W + tx - 1) / tx, nimg);
    cl.st = st;
    const cudaError_t e = col_reg_dispatch(H, 0, cl, p, g, X, out);
    ++launches;
    if (e != cudaSuccess) return fail(DTMM_ECUDA, "launch k_layer_col_reg: %s", cudaGetErrorString(e));
  } else {
    const size_t per = 4 * (size_t)H * sizeof(cpx<R>) * 2;
    int tc = 1;
    while (tc < 16 && per * (tc * 2) <= 72 * 1024) tc *= 2;
    if (tc > W) tc = W;
    p.tc = tc;
    smem = per * tc + H * (sizeof(cpx<R>) + sizeof(int));
    if (smem > 220 * 1024) return fail(DTMM_ENOTSUP, "column of %d pixels too large for one block", H);
    CK(cudaFuncSetAttribute(k_layer_col<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_layer_col<R><<<dim3((W + tc - 1) / tc, nimg), 256, smem, st>>>(p, g, X, (cpx<R>*)out);
    CKL("k_layer_col");
  }
  // rows inverse (1/W)
  if (rrows) {
    const cudaError_t e = fft_rows_reg_dispatch(W, true, rl, out, out, nlines, twW, (float)(1.0 / W));
    ++launches;
    if (e != cudaSuccess) return fail(DTMM_ECUDA, "launch k_fft_rows_reg: %s", cudaGetErrorString(e));
  } else {
    smem = (size_t)lpb * W * sizeof(cpx<R>) + W * (sizeof(cpx<R>) + sizeof(int));
    CK(cudaFuncSetAttribute(k_fft_rows<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_rows<R, true><<<(nlines + lpb - 1) / lpb, 256, smem, st>>>((cpx<R>*)out, (cpx<R>*)out, nlines, W, pW, twW,
                                                                     permW, 1.0 / W, lpb);
    CKL("k_fft_rows");
  }
  return DTMM_OK;
}

// plane-wave fills (k_planewave for FFT modes, k_wave_window for continuous
// wave vectors with an optional window): one block per kWaveRows rows of one
// image, the row and column phase factors in shared memory
int launch_wave(int H, int W, int nimg, const void* coef, const int* my, const int* mx, const double* kx,
                const double* ky, const double* window, int precision, void* field, void* stream) {
  if (H < 1 || W < 1) return fail(DTMM_EINVAL, "grid must be at least 1x1");
  if (nimg < 1 || nimg > 65535) return fail(DTMM_EINVAL, "image count %d outside 1..65535", nimg);
  if (!coef || !field || (kx == nullptr && (!my || !mx))) return fail(DTMM_EINVAL, "null pointer");
  if (precision != DTMM_PRECISION_MIXED && precision != DTMM_PRECISION_DOUBLE)
    return fail(DTMM_EINVAL, "invalid precision");
  const size_t csz = precision == DTMM_PRECISION_DOUBLE ? sizeof(cpx<double>) : sizeof(cpx<float>);
  const size_t smem = (size_t)(W + kWaveRows) * csz;
  if (smem > 220 * 1024) return fail(DTMM_ENOTSUP, "row of %d pixels too long for the plane-wave fill", W);
  dim3 grid((H + kWaveRows - 1) / kWaveRows, nimg);
  cudaStream_t st = (cudaStream_t)stream;
  const cpx<double>* c = (const cpx<double>*)coef;
  if (precision == DTMM_PRECISION_DOUBLE) {
    if (kx) {
      CK(cudaFuncSetAttribute(k_wave_window<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_wave_window<double><<<grid, 256, smem, st>>>((cpx<double>*)field, c, kx, ky, window, H, W);
    } else {
      CK(cudaFuncSetAttribute(k_planewave<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_planewave<double><<<grid, 256, smem, st>>>((cpx<double>*)field, c, my, mx, H, W);
    }
  } else {
    if (kx) {
      CK(cudaFuncSetAttribute(k_wave_window<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_wave_window<float><<<grid, 256, smem, st>>>((cpx<float>*)field, c, kx, ky, window, H, W);
    } else {
      CK(cudaFuncSetAttribute(k_planewave<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_planewave<float><<<grid, 256, smem, st>>>((cpx<float>*)field, c, my, mx, H, W);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DTMM_ECUDA, "plane-wave fill: %s", cudaGetErrorString(e));
  return DTMM_OK;
}

int transfer_impl(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* workspace, size_t workspace_bytes,
                  void* stream, Prof* prof, int* launches) {
  g_err.clear();
  int rc = check_desc(desc);
  if (rc) return rc;
  if (io == nullptr || io->field_in == nullptr || io->field_out == nullptr) return fail(DTMM_EINVAL, "null field buffer");
  // the 2x2 k-space sweep carries the sum over windows, whose E -> H conversion differs per window
  if (io->bulk != nullptr && desc->method == 2 && !is_real2(desc) && desc->diffraction > 1)
    return fail(DTMM_ENOTSUP, "2x2 bulk output in k-space is implemented without windows (diffraction <= 1)");
  Layout L = layout_of(desc);
  if (workspace == nullptr || workspace_bytes < L.total)
    return fail(DTMM_ENOSPACE, "workspace of %zu bytes, %zu needed", workspace_bytes, L.total);
  cudaStream_t st = (cudaStream_t)stream;
  if (desc->precision == DTMM_PRECISION_DOUBLE) return run_engine<double>(desc, io, workspace, L, st, prof, launches);
  return run_engine<float>(desc, io, workspace, L, st, prof, launches);
}

// ---------------------------------------------------------------------------
// Static device scratch for dtmm_transfer_noalloc.  In host code the name
// g_static_scratch is only a host-side stand-in for the device array, so the
// device address is resolved once per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_static_scratch[DTMM_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int static_scratch(void** out) {
  int dev = -1;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(DTMM_EINVAL, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return fail(DTMM_ECUDA, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return DTMM_OK;
}

}  // namespace

namespace dtmm {
std::string& last_error_slot() { return g_err; }
}

extern "C" {

int dtmm_abi_version(void) { return 7; }

const char* dtmm_last_error(void) { return g_err.c_str(); }

size_t dtmm_transfer_workspace_size(const dtmm_transfer_desc* desc) {
  if (check_desc(desc) != DTMM_OK) return 0;
  return layout_of(desc).total;
}

int dtmm_transfer(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* workspace, size_t workspace_bytes,
                  void* stream) {
  return transfer_impl(desc, io, workspace, workspace_bytes, stream, nullptr, nullptr);
}

int dtmm_transfer_noalloc(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* stream) {
  g_err.clear();
  int rc = check_desc(desc);
  if (rc) return rc;
  // npass > 1 caches every layer's operators when they fit the default limit;
  // when that layout is too large for the static scratch, the two alternating
  // operator buffers of the uncached schedule are tried (same results)
  dtmm_transfer_desc dd = *desc;
  Layout L = layout_of(&dd);
  if (L.total > DTMM_STATIC_SCRATCH_BYTES && L.cache_ops) {
    dd.op_cache_bytes = 1;
    L = layout_of(&dd);
  }
  if (L.total > DTMM_STATIC_SCRATCH_BYTES)
    return fail(DTMM_ENOSPACE, "transfer needs %zu bytes of scratch; the static scratch holds %zu", L.total,
                (size_t)DTMM_STATIC_SCRATCH_BYTES);
  void* ws = nullptr;
  if ((rc = static_scratch(&ws))) return rc;
  return transfer_impl(&dd, io, ws, DTMM_STATIC_SCRATCH_BYTES, stream, nullptr, nullptr);
}

int dtmm_transfer_timed(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* workspace,
                        size_t workspace_bytes, void* stream, dtmm_kernel_times* times) {
  Prof prof;
  int launches = 0;
  int rc = transfer_impl(desc, io, workspace, workspace_bytes, stream, &prof, &launches);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return fail(DTMM_ECUDA, "cudaStreamSynchronize: %s", cudaGetErrorString(e));
  if (times) {
    times->layer_row_ms = prof.total(PROF_ROW);
    times->layer_col_ms = prof.total(PROF_COL);
    times->voxel_op_ms = prof.total(PROF_OP);
    times->layer_row_launches = (int)prof.ev[PROF_ROW].size() / 2;
    times->layer_col_launches = (int)prof.ev[PROF_COL].size() / 2;
    times->voxel_op_launches = (int)prof.ev[PROF_OP].size() / 2;
    times->total_launches = launches;
  }
  return DTMM_OK;
}

int dtmm_planewave_field(int height, int width, int nimg, const void* coef, const int* my, const int* mx,
                         int precision, void* field, void* stream) {
  g_err.clear();
  return launch_wave(height, width, nimg, coef, my, mx, nullptr, nullptr, nullptr, precision, field, stream);
}

int dtmm_wave_field(int height, int width, int nimg, const void* coef, const double* kx, const double* ky,
                    const double* window, int precision, void* field, void* stream) {
  g_err.clear();
  if (!kx || !ky) return fail(DTMM_EINVAL, "null pointer");
  return launch_wave(height, width, nimg, coef, nullptr, nullptr, kx, ky, window, precision, field, stream);
}

int dtmm_field_diffraction_matrix(int height, int width, int nlam, const double* ks, double d, double eps_re,
                                  double eps_im, int mode, double betamax, void* dmat, void* stream) {
  g_err.clear();
  if (height < 1 || width < 1 || nlam < 1) return fail(DTMM_EINVAL, "empty grid or wavelength axis");
  if (!ks || !dmat) return fail(DTMM_EINVAL, "null pointer");
  if (mode < -1 || mode > 1) return fail(DTMM_EINVAL, "mode must be 0 (both), 1 (forward) or -1 (backward)");
  Grid g;
  memset(&g, 0, sizeof(g));
  g.H = height;
  g.W = width;
  g.nlam = nlam;
  cudaStream_t st = (cudaStream_t)stream;
  const long long hw = (long long)height * width;
  for (int l0 = 0; l0 < nlam; l0 += 64) {
    KsChunk kc;
    kc.n = std::min(64, nlam - l0);
    for (int i = 0; i < kc.n; ++i) kc.ks[i] = ks[l0 + i];
    const long long n = (long long)kc.n * hw;
    if (n > (long long)INT32_MAX) return fail(DTMM_EINVAL, "grid too large");
    k_field_dmat<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(kc, l0, g, mk<double>(eps_re, eps_im), d, mode, betamax,
                                                             (cpx<double>*)dmat);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DTMM_ECUDA, "k_field_dmat: %s", cudaGetErrorString(e));
  }
  return DTMM_OK;
}

int dtmm_field_intensity(int height, int width, int nimg, int precision, const void* field, double* sums,
                         void* stream) {
  g_err.clear();
  if (height < 1 || width < 1 || nimg < 1) return fail(DTMM_EINVAL, "empty field");
  if (nimg > INT32_MAX / 4) return fail(DTMM_EINVAL, "too many images");
  if (!field || !sums) return fail(DTMM_EINVAL, "null pointer");
  if (precision != DTMM_PRECISION_MIXED && precision != DTMM_PRECISION_DOUBLE)
    return fail(DTMM_EINVAL, "invalid precision");
  Grid g;
  memset(&g, 0, sizeof(g));
  g.H = height;
  g.W = width;
  g.NI = nimg;
  cudaStream_t st = (cudaStream_t)stream;
  // one chunk per image (the sums land in sums directly), at most 65535 images a launch
  const size_t per = 4 * (size_t)height * width;
  for (int o = 0; o < nimg; o += 65535) {
    const unsigned n = (unsigned)std::min(65535, nimg - o);
    if (precision == DTMM_PRECISION_DOUBLE)
      k_total_intensity<double><<<dim3(1, n), 256, 0, st>>>((const cpx<double>*)field + per * o, g, sums + o);
    else
      k_total_intensity<float><<<dim3(1, n), 256, 0, st>>>((const cpx<float>*)field + per * o, g, sums + o);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DTMM_ECUDA, "k_total_intensity: %s", cudaGetErrorString(e));
  return DTMM_OK;
}

int dtmm_scale_fields(int height, int width, int nimg, int precision, void* field, const double* base,
                      const double* num, const double* den, void* stream) {
  g_err.clear();
  if (height < 1 || width < 1 || nimg < 1 || nimg > 65535) return fail(DTMM_EINVAL, "image count outside 1..65535");
  if (!field) return fail(DTMM_EINVAL, "null pointer");
  if ((num == nullptr) != (den == nullptr)) return fail(DTMM_EINVAL, "num and den must be given together");
  if (precision != DTMM_PRECISION_MIXED && precision != DTMM_PRECISION_DOUBLE)
    return fail(DTMM_EINVAL, "invalid precision");
  const long long per = 4LL * height * width;
  dim3 grid((unsigned)std::min<long long>((per + 255) / 256, 304), nimg);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == DTMM_PRECISION_DOUBLE)
    k_scale_fields<double><<<grid, 256, 0, st>>>((cpx<double>*)field, per, base, num, den);
  else
    k_scale_fields<float><<<grid, 256, 0, st>>>((cpx<float>*)field, per, base, num, den);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DTMM_ECUDA, "k_scale_fields: %s", cudaGetErrorString(e));
  return DTMM_OK;
}

size_t dtmm_diffract_workspace_size(int height, int width, int nimg, int nlam, int precision) {
  g_err.clear();
  if (check_diffract(height, width, nimg, nlam, precision)) return 0;
  return diffract_layout(height, width, nimg, nlam, precision).total;
}

int dtmm_diffract(int height, int width, int nimg, int nlam, int precision, const void* dmat, const void* field_in,
                  void* field_out, void* workspace, size_t workspace_bytes, void* stream) {
  g_err.clear();
  int rc = check_diffract(height, width, nimg, nlam, precision);
  if (rc) return rc;
  if (!dmat || !field_in || !field_out || !workspace) return fail(DTMM_EINVAL, "null pointer");
  const DiffractLayout L = diffract_layout(height, width, nimg, nlam, precision);
  if (workspace_bytes < L.total) return fail(DTMM_ENOSPACE, "workspace too small (%zu < %zu)", workspace_bytes, L.total);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == DTMM_PRECISION_DOUBLE)
    return diffract_impl<double>(height, width, nimg, nlam, dmat, field_in, field_out, (unsigned char*)workspace, L,
                                 st);
  return diffract_impl<float>(height, width, nimg, nlam, dmat, field_in, field_out, (unsigned char*)workspace, L,
                              st);
}

}  // extern "C"
