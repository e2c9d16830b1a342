/*
 * dtmm_gb300 -- C ABI of the GB300 field-transfer engine.
 *
 * The reference (dtmm, pure Python + numba) has no FFI; its drop-in boundary
 * is the Python call
 *     dtmm.transfer_field(field_data, optical_data, beta, phi, nin, nout,
 *                         npass, nstep, diffraction, reflection, method, ...)
 * (dtmm/transfer.py:322-552) with the method drivers transfer_4x4
 * (dtmm/transfer.py:618-884) and transfer_2x2 (dtmm/transfer.py:1009-1183).
 * This ABI replaces the body of those drivers: option resolution, input
 * validation and the (field, wavelengths, pixelsize) / (thickness, eps,
 * angles) data model stay in the Python layer (dtmm_gb300/transfer.py), which
 * calls dtmm_transfer() once per transfer_field call.
 *
 * All pointers in dtmm_transfer_io and the material pointers in the
 * descriptor are device pointers; all other arrays in the descriptor are host
 * arrays read during the call.  Every function returns DTMM_OK (0) or a
 * negative status; dtmm_last_error() describes the last failure of the
 * calling thread.  No exception crosses the ABI.
 */
#ifndef DTMM_GB300_H
#define DTMM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DTMM_OK 0
#define DTMM_EINVAL (-1)      /* invalid argument (ValueError in the reference)         */
#define DTMM_ENOSPACE (-2)    /* workspace smaller than dtmm_transfer_workspace_size() */
#define DTMM_ECUDA (-3)       /* a CUDA call failed                                     */
#define DTMM_ENOTSUP (-4)     /* option combination outside this engine                 */

/* diffraction = inf: every eigenwave below betamax through the voxels exactly
   (dtmm/propagate_4x4.py:515-560); 4x4, any reflection mode, any npass */
#define DTMM_DIFFRACTION_FULL (-1)

#define DTMM_PRECISION_MIXED 0  /* complex64 bulk, FP64 eigen-solve and operator tables */
#define DTMM_PRECISION_DOUBLE 1 /* complex128 bulk (the reference's default precision)  */

typedef struct dtmm_transfer_desc {
  /* grid and images: images = nray * npol * nlam, in the reference's
     ([rays], [pols], wavelength) axis order */
  int height, width;
  int nlam, npol, nray;
  /* method and options (resolved by the caller as dtmm/transfer.py:433-465 does) */
  int method;        /* 4 = "4x4", 2 = "2x2"                                   */
  int diffraction;   /* >= 1: n > 1 groups modes into n x n windows; 0: no
                        diffraction (4x4 with reflection 2 or 4; 2x2);
                        DTMM_DIFFRACTION_FULL: inf                           */
  int reflection;    /* 4x4: 1 (diffraction >= 1), 2 and 4 (any diffraction),
                        3 (diffraction >= 1), any with DTMM_DIFFRACTION_FULL;
                        2x2: 0, 1 or 2 (1 without diffraction: npass 1; 0 or
                        2 with DTMM_DIFFRACTION_FULL)                        */
  int npass;         /* >= 1 (2x2 with npass > 1: reflection 1 or 2)            */
  int precision;     /* DTMM_PRECISION_*                                        */
  double betamax, nin, nout, smooth;
  /* layers of the (single) optical block */
  int nlayers;
  const double* thickness; /* host [nlayers], pixels                          */
  const int* nstep;        /* host [nlayers], sub-steps per layer (>= 1)      */
  /* material, device pointers; strides in elements of the (layer, y, x)
     axes, 0 for a broadcast axis; the last axis (3 values) is contiguous */
  const void* epsv;        /* float64 or complex128 eigenvalues                 */
  int eps_complex;
  long long epsv_strides[3];
  const double* epsa;      /* float64 Euler angles (psi, theta, phi)            */
  long long epsa_strides[3];
  /* beams, host arrays */
  const double* ks;        /* [nlam] 2*pi*pixelsize/wavelength                  */
  const double* beta;      /* [nray]                                            */
  const double* phi;       /* [nray]                                            */
  /* upper bound on the bytes of cached per-layer operators (npass > 1 reuses
     them across passes when they fit); 0 selects the default (48 GiB) */
  size_t op_cache_bytes;
  /* 1: the caller guarantees real eps whose every eigenvalue (and hence the
     effective medium) exceeds max(betamax, beta)^2; every radicand of the
     eigen-solve is then positive and the engine uses real FP64 arithmetic and
     half-size operator records.  Ignored for complex eps. */
  int real_path;
  /* tuning (0 = built-in choice; results do not depend on row_group and
     col_tile): wavelengths per row block, columns per column block, and the
     line transform schedule: 1 = two-step register transform where it
     applies (power-of-two sides 64..1024, complex64), 2 = shared-memory
     mixed radix with radix-4 passes first, 3 = the same with radix-8 first */
  int row_group;
  int col_tile;
  int fft_schedule;
  /* 1: some voxels are biaxial (eps[0] != eps[1]); their eigen-modes come
     from the general 4 x 4 eigen-solve and Poynting sort (dtmm/tmm.py:395-401)
     and real_path is ignored.  0: the caller guarantees eps[0] == eps[1] for
     every voxel (isotropic / uniaxial closed forms only). */
  int biaxial;
  /* 4x4 with npass > 1: 1 renormalises each image's total intensity after the
     output projection (the reference's norm = 0, "total",
     dtmm/transfer.py:140-155); 0 each k's intensity (DTMM_NORM_FFT,
     dtmm/transfer.py:78-90).  ABI 4. */
  int norm_total;
  /* host [nlayers] or null: the optical-data block of every layer (0, then
     each layer's block equal to or one above the previous layer's).  Each
     block has its own isotropic effective medium, the mean eps of its voxels
     (dtmm/transfer.py:926-1005 builds the layer list block by block; one
     block per layer with split_layers).  Null: one block.  2x2 reflection 0 /
     1 with several blocks: npass 1.  ABI 4. */
  const int* layer_block;
  /* 4x4 with npass > 1: 1 propagates a 2x2 reference field (the input's E
     part, then each backward pass's result) through the forward passes
     beside the transfer, 2x2 mode 2 without reflections, with its H part in
     the output medium (dtmm/transfer.py:637-645, :710-713, :770-806).  With
     norm_total 0 (the reference's DTMM_NORM_FFT | DTMM_NORM_REF) the
     intensities of the per-k normalisation come from it (the reference's
     projection there transforms fft2(ref) where the field was,
     dtmm/transfer.py:78-83, :830, and this does the same).  With
     norm_total 1 (the reference's DTMM_NORM_REF alone, "local",
     dtmm/transfer.py:103-136, :824-835) the projected field is split per
     pixel by the polarizer of its forward amplitudes at normal incidence in
     the output medium: the reference field's polarised part sets the
     intensity, its remainder is added.  Finite diffraction only.  ABI 5. */
  int norm_ref;
  /* host [nblocks] or null (every block isotropic): the symmetry of each
     block's effective medium (dtmm/data.py:1364-1419, dtmm/transfer.py:
     926-1005).  0: isotropic, the mean of the voxels' (e0 + e1 + e2) / 3;
     1: uniaxial, 2: biaxial, from the mean of the voxels' lab-frame tensors
     R diag(epsv) R^T: its eigenvalues ordered so that the third is the most
     distinct (the first two averaged for 1) and its eigen-frame as Euler
     angles.  The reference's per-layer symmetry is a block per layer.  With
     the 4x4 method a block of symmetry 1 or 2 takes the real-space chains of
     every reflection mode (mode 1: C E P F^-1 per k, E P E^-1 per voxel,
     F P E^-1 C per k) with the effective tensor's eigen-data in the k-space
     matrices (also for the reference field of norm_ref); the 2x2 method
     takes it on its real-space paths (reflection 2; reflection 0 with
     diffraction as the real-space chain C E(d/2) per k, E P E^-1 per
     voxel, E(d/2) C per k) and refuses reflection 1; diffraction 0 and inf
     do not use the effective medium.  The tensor's eigen-frame is found on the
     host: the call
     synchronises its stream once, and is refused inside a stream capture.
     ABI 6. */
  const int* block_sym;
  /* host [nblocks][9] or null: with block_sym 3 a block's effective medium
     is given (the reference's eff_data as an optical block, homogeneous in
     each layer, dtmm/transfer.py:941-948): epsv (re, im) x 3 and the Euler
     angles psi, theta, phi.  Three equal eigenvalues make it isotropic (the
     default path), otherwise it takes the real-space chains as block_sym 1
     and 2 do; no host synchronisation.  ABI 7. */
  const double* block_eff;
} dtmm_transfer_desc;

typedef struct dtmm_transfer_io {
  /* [images][4][height][width] complex (complex64 for MIXED, complex128 for
     DOUBLE).  field_in is rewritten in place with the reflected field when
     npass > 1 (dtmm/transfer.py:843-866), as the reference does. */
  void* field_in;
  void* field_out;
  int out_given;  /* 4x4: field_out holds the caller's out= array; its reflected
                     part is kept (dtmm/transfer.py:674); 2x2 zeroes it, as the
                     reference does (dtmm/transfer.py:1054) */
  /* optional: [(nlayers + 2)][images][4][H][W]; when set, receives the field
     after every layer (ret_bulk, dtmm/transfer.py:657-673, :1039-1062);
     field_in/field_out must then point at its first / last slab.  4x4: npass
     > 1 with reflection 1 only; 2x2: k-space (reflection 0 / 1) without
     windows (diffraction <= 1), real space any */
  void* bulk;
} dtmm_transfer_io;

/* Device-time accounting of one dtmm_transfer_timed call. */
typedef struct dtmm_kernel_times {
  double layer_row_ms;     /* fused row kernels (inverse row FFTs, per-voxel operators, forward row FFT) */
  double layer_col_ms;     /* fused column kernels (column FFTs, k-space operator, window split)        */
  double voxel_op_ms;      /* FP64 per-voxel layer-operator builds                                       */
  int layer_row_launches;
  int layer_col_launches;
  int voxel_op_launches;
  int total_launches;      /* every kernel launched by the call                                          */
} dtmm_kernel_times;

/* ABI version of this header (2: tuning fields in dtmm_transfer_desc, plane-wave inputs, POM image formation;
   3: the biaxial field of dtmm_transfer_desc; 4: norm_total, layer_block; 5: norm_ref; 6: block_sym; 7: block_eff). */
int dtmm_abi_version(void);

/* Message of the last failure on the calling thread ("" if none). */
const char* dtmm_last_error(void);

/* Device workspace (bytes) that dtmm_transfer needs for this descriptor;
   0 on an invalid descriptor (see dtmm_last_error). */
size_t dtmm_transfer_workspace_size(const dtmm_transfer_desc* desc);

/* Transfer the input field through the optical block: the work of
   transfer_4x4 / transfer_2x2 (dtmm/transfer.py:618, :1009) after option
   resolution.  4x4: the k-space split step (reflection 1,
   dtmm/propagate_4x4.py:376-444), the real-space reflection modes 2-4 with
   diffraction (dtmm/propagate_4x4.py:18-287, :447-512), the per-voxel
   transfer without diffraction (reflection 2 or 4) and the exact modal
   transfer (DTMM_DIFFRACTION_FULL, dtmm/propagate_4x4.py:515-560), each
   with any npass.  2x2: the k-space split step with reflection 0 or 1
   (dtmm/propagate_2x2.py:19-87, :193-284) and the real-space reflection
   mode 2 / no-diffraction transfer (dtmm/propagate_2x2.py:91-190, :286-377)
   and the exact modal transfer (DTMM_DIFFRACTION_FULL with reflection 0 or
   2, dtmm/propagate_2x2.py:379-464), any npass (the reflected waves kept per interface, backward passes adding
   into field_in, dtmm/transfer.py:1074-1183).  `stream` is a
   cudaStream_t (NULL = legacy default stream).  The call enqueues the work
   and returns; results are ready when the stream is.  The first call on a
   stream creates that stream's side stream (kept for the process), on
   which the per-layer operators run beside the transforms. */
int dtmm_transfer(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* workspace,
                  size_t workspace_bytes, void* stream);

/* dtmm_transfer plus device-time accounting: CUDA events are recorded on
   `stream` around every fused row / column kernel and operator build; the
   call synchronises the stream before it returns and fills *times.  Same
   computation and results as dtmm_transfer; no counterpart in the reference
   (which has no profiling hooks), used by the benchmark's roofline figures. */
int dtmm_transfer_timed(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* workspace,
                        size_t workspace_bytes, void* stream, dtmm_kernel_times* times);

/* Capacity of the library's static device scratch (64 MiB), see dtmm_transfer_noalloc. */
#define DTMM_STATIC_SCRATCH_BYTES ((size_t)64 << 20)

/* dtmm_transfer without any device allocation, for callers that cannot
   allocate device memory when they call: plugin hosts that hand the engine
   only their own input/output buffers and keep every other allocation to
   themselves, and latency-bound loops whose budget a cudaMalloc (which can
   synchronise or fail under memory pressure) would break.  The workspace is a
   file-scope device array of DTMM_STATIC_SCRATCH_BYTES that every GPU loading
   the library holds until the process exits; the caller still passes the
   input and output fields.  No counterpart in the reference (which allocates
   numpy temporaries freely).
   - The first call on a device resolves the array's device address
     (cudaGetSymbolAddress) with that device current; make that first call
     before any stream capture.
   - Transfers whose workspace (dtmm_transfer_workspace_size) exceeds the
     array are rejected with DTMM_ENOSPACE and a message giving both sizes;
     an npass > 1 transfer whose every-layer operator cache does not fit is
     first retried with two alternating operator buffers (same results).
   - The first call on a stream creates that stream's side stream, as
     dtmm_transfer does; later calls on it create nothing.
   - Every call shares the one array: calls that overlap on the GPU (other
     streams, other host threads) race and must be serialised by the caller.
     No part of the scratch has to start at zero: every buffer is written
     before it is read, so a call is unaffected by the previous call's
     leftovers.
   - Calls no cudaMalloc, cudaFree or allocating library routine. */
int dtmm_transfer_noalloc(const dtmm_transfer_desc* desc, const dtmm_transfer_io* io, void* stream);

/* Plane-wave input fields on the device: for every image i < nimg and
   component c < 4,
     field[i][c][y][x] = coef[i][c] * exp(2 pi i (my[i] y / height + mx[i] x / width))
   with the phase reduced exactly (integer arithmetic) before one FP64
   sincospi.  coef: device complex128 [nimg][4]; my, mx: device int [nimg]
   (taken modulo height / width); field: device complex64 (precision MIXED)
   or complex128 (DOUBLE) [nimg][4][height][width].  This is the grid-filling
   part of the reference's illumination_data (dtmm/field.py:586-713) for
   eigenmode input, whose waves are single FFT-grid modes (wave2eigenwave,
   dtmm/wave.py:432) and stay so through its diffraction filter
   (dtmm/diffract.py:301); the per-image vectors and modes come from the
   host (dtmm_gb300.illumination.illumination_modes). */
int dtmm_planewave_field(int height, int width, int nimg, const void* coef, const int* my, const int* mx,
                         int precision, void* field, void* stream);

/* ------------------------------------------------------------------------
   POM image formation on transferred fields (dtmm's field viewer pipeline).
   Fields are device arrays of complex64 (precision MIXED) or complex128
   (DOUBLE), [set][pol][lam][4][H][W] with npol == 2 (x / y inputs combined
   with the polarizer jones vector) or [set][lam][4][H][W] with npol == 1.
   ------------------------------------------------------------------------ */
typedef struct {
  int height, width;
  int nlam;              /* wavelengths */
  int nset;              /* leading image sets (e.g. rays), summed by the image */
  int npol;              /* 2: combine the x / y input axis with jvec; 1: no such axis */
  double jvec[4];        /* polarizer jones vector (re0, im0, re1, im1), npol == 2 */
  const void* pmat;      /* device complex128 4x4 analyzer matrix for every pixel, or null */
  const double* window;  /* device H x W real window, or null */
  int precision;         /* field type */
} dtmm_pom_desc;

/* calculate_pom_field (dtmm/field_viewer.py:70-143), real-space path
   without refocus: out[set][lam][4][H][W] = pmat . (window * (j0 Fx + j1 Fy)). */
int dtmm_pom_field(const dtmm_pom_desc* desc, const void* field, void* out, void* stream);

/* field2specter / field2spectersum (dtmm/field.py:784-847): normal Poynting
   component Re(f0 f1*) - Re(f2 f3*) of [set][lam][4][H][W] fields, written
   as spec[set][H][W][lam] (float64), or summed over the sets when sum_sets. */
int dtmm_field2specter(int height, int width, int nlam, int nset, int sum_sets, int precision, const void* field,
                       double* spec, void* stream);

/* specter2color (dtmm/color.py:133-224): spec[npix][nlam] (float64) times
   cmf[nlam][3] (float64) -> XYZ; norm_mode 0 = none, 1 = divide by
   norm_value, 2 = divide by the image maximum; sRGB (D65) or gray (Y);
   gamma 0 = none, < 0 = sRGB curve, > 0 = power 1/gamma; rgb[npix][3] float64. */
int dtmm_specter2color(long long npix, int nlam, const double* spec, const double* cmf, int norm_mode,
                       double norm_value, double gamma, int gray, double* rgb, void* stream);

/* The three steps fused, one pass over the field: rgb[H][W][3] float32 of
   the sets' summed specter (norm_mode, gamma, gray as above). */
int dtmm_pom_image(const dtmm_pom_desc* desc, const void* field, const double* cmf, int norm_mode,
                   double norm_value, double gamma, int gray, float* rgb, void* stream);

/* diffract (dtmm/diffract.py:254-299) in real space: fft2, a per-k 4x4
   matrix, ifft2.  field_in / field_out: device [nimg][4][H][W] (complex64
   for precision MIXED, complex128 for DOUBLE; image i uses wavelength
   i % nlam); dmat: device complex128 [nlam][H][W][4][4] (the reference's
   field_diffraction_matrix layout); workspace: caller-provided device
   memory of dtmm_diffract_workspace_size bytes. */
size_t dtmm_diffract_workspace_size(int height, int width, int nimg, int nlam, int precision);
int dtmm_diffract(int height, int width, int nimg, int nlam, int precision, const void* dmat, const void* field_in,
                  void* field_out, void* workspace, size_t workspace_bytes, void* stream);

/* Plane waves with continuous wave vectors (the windowed branch of
   illumination_data, dtmm/field.py:586-713; illumination_waves :459 and
   planewave, dtmm/wave.py:376): field[i][c][y][x] = coef[i][c] *
   exp(i (kx[i] x + ky[i] y)) * window[y][x].  coef: device complex128
   [nimg][4]; kx, ky: device float64 [nimg]; window: device float64 [H][W]
   or null; field: device complex64 (MIXED) or complex128 (DOUBLE). */
int dtmm_wave_field(int height, int width, int nimg, const void* coef, const double* kx, const double* ky,
                    const double* window, int precision, void* field, void* stream);

/* Field diffraction matrix of a homogeneous isotropic medium eps = eps_re + i
   eps_im over d pixels (field_diffraction_matrix, dtmm/diffract.py:125-138):
   dmat[lam][ky][kx][4][4] (device complex128) = F diag(exp(i alpha k_lam d))
   F^-1 on the FFT grid, keeping both directions (mode 0), the forward
   (mode 1) or the backward (mode -1) modes, zero where beta >= betamax.  ks:
   host float64 [nlam] (2 pi pixelsize / lambda).  The dmat argument of
   dtmm_diffract. */
int dtmm_field_diffraction_matrix(int height, int width, int nlam, const double* ks, double d, double eps_re,
                                  double eps_im, int mode, double betamax, void* dmat, void* stream);

/* Total intensity of each image: sums[i] = sum over pixels of the normal
   Poynting component (field2intensity, dtmm/field.py:780, summed over the
   grid).  field: device [nimg][4][H][W]; sums: device float64 [nimg]. */
int dtmm_field_intensity(int height, int width, int nimg, int precision, const void* field, double* sums,
                         void* stream);

/* field[i] *= base[i] * sqrt(num[i] / den[i]) (device float64 arrays; base
   null = 1; num and den both null = no ratio): the intensity rescale of
   illumination_data after its diffraction step. */
int dtmm_scale_fields(int height, int width, int nimg, int precision, void* field, const double* base,
                      const double* num, const double* den, void* stream);

/* director2data (dtmm/data.py:277-320) on the device: director[nvox][3]
   (float64, or float32 when director_double == 0) -> eps eigenvalues
   epsv[nvox][3] and Euler angles epsa[nvox][3] (float64).  The order
   parameter is sqrt(|director|) / scale_factor applied to (no^2, no^2, ne^2);
   voxels where mask[i] == 0 (uint8 [nvox], optional) get nhost^2. */
int dtmm_director2data(long long nvox, const void* director, int director_double, const void* mask, double no,
                       double ne, double nhost, double scale_factor, double* epsv, double* epsa, void* stream);

/* Q2data (dtmm/data.py:322-371) on the device: Q tensors qtensor[nvox][6]
   (float64: Q00, Q11, Q22, Q01, Q02, Q12) -> eps = (ne^2 - no^2) /
   scale_factor * Q + (2 no^2 + ne^2) / 3 * I, its eigenvalues epsv[nvox][3]
   sorted with the most distinct one last and the Euler angles epsa[nvox][3]
   of its eigenvector frame (float64).  Unless biaxial != 0 the eigenvalues
   are replaced by their uniaxial order 1; voxels where mask[i] == 0 (uint8
   [nvox], optional) get nhost^2. */
int dtmm_q2data(long long nvox, const double* qtensor, const void* mask, double no, double ne, double nhost,
                double scale_factor, int biaxial, double* epsv, double* epsa, void* stream);

/* Synthetic twisted-nematic Euler angles for benchmarks and serving tests
   (no reference counterpart; the seeded director of
   dtmm_gb300.samples.twisted_nematic): epsa[L][H][W][3] (device float64) =
   (0, pi/2 - (d_tilt + tilt), l twist / L + d_phi) with d_phi = amp_phi sum_i
   cos(ax_i x + ay_i y + c_i) over the first nmodes rows of `modes` and d_tilt
   = amp_tilt times the same sum over the next nmodes rows; modes: host
   float64 [2 nmodes][3] (ax, ay, c), nmodes <= 16. */
int dtmm_twisted_nematic_angles(int nlayers, int height, int width, const double* modes, int nmodes, double amp_phi,
                                double amp_tilt, double twist, double tilt, double* epsa, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DTMM_GB300_H */
