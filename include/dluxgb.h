/*
 * dluxgb.h -- C ABI of the GB300-native dLux diffraction hot path.
 *
 * Every entry point takes plain pointers to caller-owned device memory,
 * explicit sizes and a cudaStream_t (passed as void*; NULL is the legacy
 * default stream), enqueues its work on that stream and returns an int status
 * (DLX_OK or one of the DLX_ERR_* codes below). dlx_last_error() returns a
 * thread-local message for the most recent failure on the calling thread.
 *
 * Complex arrays are interleaved complex64 (float re, float im), row-major,
 * axis 0 = y and axis 1 = x, the same layout as a numpy/torch complex64 array.
 * Real arrays are float32, row-major.
 *
 * Citations are to dLux v0.16.0 (paths relative to the dLux project root).
 */
#ifndef DLUXGB_H
#define DLUXGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DLX_OK 0
#define DLX_ERR_ARG 1         /* invalid argument value (dLux raises ValueError) */
#define DLX_ERR_SHAPE 2       /* inconsistent sizes (dLux raises ValueError) */
#define DLX_ERR_NOMEM 3       /* device allocation failed */
#define DLX_ERR_CUDA 4        /* a CUDA runtime call failed */
#define DLX_ERR_TIMEOUT 5     /* a bounded device wait gave up */
#define DLX_ERR_UNSUPPORTED 6 /* device or configuration not supported */

/* ---- MFT arithmetic forms ---------------------------------------------- */
#define DLX_VARIANT_FP32 0       /* FP32 complex GEMM on the CUDA cores */
#define DLX_VARIANT_SPLIT_BF16 1 /* BF16 hi/lo three-product tcgen05 GEMM, FP32 accumulation */
#define DLX_VARIANT_RADIX 2      /* FFT plans only: radix-2 line FFTs in FP32 (pad * N a power of 2) */

/* Thread-local message of the last failing call ("" if none). */
const char* dlx_last_error(void);
/* ABI version (major * 10000 + minor * 100 + patch). */
int dlx_version(void);
/* Synchronises `stream`, then reports (and clears) the device status word that
 * the tensor-core kernels set when a bounded wait expires: *status is DLX_OK
 * or DLX_ERR_TIMEOUT. The status word is kept per device (the current one is
 * read). No dLux counterpart (dLux has no device-side waits). */
int dlx_device_status(void* stream, int* status);
/* Wall-clock limit of each wait inside the tensor-core GEMMs, in ns, read at
 * every launch (0 restores the default of 2 s). On expiry a GEMM sets the
 * device status word to DLX_ERR_TIMEOUT, lets the copies and MMAs it already
 * issued complete, frees its tensor memory and returns; its output is then
 * undefined. No dLux counterpart. */
int dlx_set_wait_limit_ns(unsigned long long limit_ns);
/* Test hook for the bounded waits: while enabled, the copy warp of the
 * loaded-operand tensor-core GEMM (single-CTA form) issues no copies, so its
 * consumers' waits run into the limit of dlx_set_wait_limit_ns with nothing in
 * flight. Results are undefined while it is on. No dLux counterpart. */
int dlx_test_gemm_withhold_copies(int enable);
/* Number of kernel launches the library has issued in this process. */
long long dlx_launch_count(void);
/* Brackets every complex-GEMM launch with CUDA events on its own stream until
 * dlx_gemm_timing_end, which waits for them and returns the summed kernel time
 * (ms), the number of launches and their algorithmic flops (8 M N K per
 * complex GEMM). Measurement aid for the roofline; not thread-safe. */
int dlx_gemm_timing_begin(void);
int dlx_gemm_timing_end(double* total_ms, int* launches, double* flops);

/* ---- a1: transfer matrix ------------------------------------------------
 * Replaces dLux utils/propagation.py:67-127 (transfer_matrix), batched over
 * wavelengths. out[b] is the [n_in][n_out] matrix
 *   exp(-+2 pi i in_vec (x) out_vec)
 * (or its [n_out][n_in] transpose when transpose != 0), with the phase
 * argument formed and range-reduced in FP64 on the device.
 * focal_length 0 means angular (dLux focal_length=None); a negative
 * focal_length is refused with DLX_ERR_ARG in every entry point (dLux's MFT
 * takes the log of the then negative fringe count and returns NaN).
 */
int dlx_transfer_matrix(const double* wavelengths_host, int batch, int n_in,
                        double pixel_scale_in, int n_out, double pixel_scale_out,
                        double shift, double focal_length, int inverse,
                        int transpose, void* out_c64, void* stream);

/* ---- a2/a3: batched MFT plan -------------------------------------------
 * Replaces dLux utils/propagation.py:178-256 (MFT) and its normalisation
 * utils/propagation.py:130-175,246-254, vmapped over a batch of wavelengths
 * (optical_systems.py:213-216). The plan caches the DFT matrices of every
 * wavelength on the device and owns its intermediate buffers.
 */
typedef struct dlx_mft_plan_s* dlx_mft_plan;
typedef struct {
  int batch;              /* number of fields (one wavelength each) */
  int n_in;               /* input side N */
  int n_out;              /* output side M */
  double pixel_scale_in;  /* input pixel scale (m/pixel) */
  double pixel_scale_out; /* output pixel scale (rad/pixel, or m/pixel with focal_length) */
  double focal_length;    /* 0: angular propagation; < 0 is refused */
  double shift_x;         /* output-plane shift in output pixels (dLux pixel=True) */
  double shift_y;
  int inverse;            /* dLux inverse=True */
  int variant;            /* DLX_VARIANT_* */
} dlx_mft_desc;

int dlx_mft_plan_create(const dlx_mft_desc* desc, const double* wavelengths_host,
                        dlx_mft_plan* plan);
int dlx_mft_plan_destroy(dlx_mft_plan plan);
/* out[b] = MFT(in[b]) : in [batch][n_in][n_in] c64 -> out [batch][n_out][n_out] c64. */
int dlx_mft_forward(dlx_mft_plan plan, const void* in_c64, void* out_c64, void* stream);
/* Adjoint (vector-Jacobian product) of dlx_mft_forward: gin = MFT^H(gout). */
int dlx_mft_adjoint(dlx_mft_plan plan, const void* gout_c64, void* gin_c64, void* stream);

/* The batched MFT of dlx_mft_forward (FP32 form) for callers that may not
 * allocate device memory -- e.g. a JAX/XLA custom call, where XLA has already
 * preallocated most of the GPU for its own pool, or a loop that forbids
 * allocation after start-up. No counterpart in the reference (dLux allocates
 * through XLA). Needs no plan: the DFT matrices and the intermediate field
 * live in a fixed 8 MiB device array inside the library, so
 * 3 * roundup(n_in * n_out * 8, 256) + 256 bytes must fit (n_in = n_out = 512
 * does); larger sizes return DLX_ERR_SHAPE. The caller passes input [batch][n_in][n_in] and
 * output [batch][n_out][n_out] complex64 device buffers. All calls share the
 * array: calls that can overlap on the GPU (unordered streams) race. The first
 * call on a device looks the array up (cudaGetSymbolAddress); make it before
 * any stream capture. */
int dlx_mft_forward_noalloc(const void* in_c64, int batch, int n_in, double pixel_scale_in,
                            int n_out, double pixel_scale_out, const double* wavelengths_host,
                            double focal_length, double shift_x, double shift_y, int inverse,
                            void* out_c64, void* stream);

/* ---- a4: FFT propagation -------------------------------------------------
 * Replaces dLux utils/propagation.py:8-64 (FFT) together with the optional
 * input/output phase ramps of wavefronts.py:654-727 (propagate_FFT) and
 * utils/fourier.py:48-78. The padded centred FFT is evaluated as a DFT-GEMM
 * pair (exact DFT, no radix restriction). ramp_shift_in/out are the ramp
 * shifts in output units (0 and 0 give dLux's spec_out=None behaviour).
 */
typedef struct dlx_fft_plan_s* dlx_fft_plan;
typedef struct {
  int batch;
  int n_in;               /* input side N */
  int pad;                /* output side is n_in * pad */
  double pixel_scale_in;
  double focal_length;    /* 0: angular; < 0 is refused */
  int inverse;
  int apply_ramps;        /* 0: no ramps (spec_out None); 1: ramps from centers below */
  double center_in;       /* input grid centre (m) */
  double center_out;      /* requested output centre (CoordSpec.c) */
  int variant;
} dlx_fft_desc;
int dlx_fft_plan_create(const dlx_fft_desc* desc, const double* wavelengths_host,
                        dlx_fft_plan* plan);
int dlx_fft_plan_destroy(dlx_fft_plan plan);
int dlx_fft_forward(dlx_fft_plan plan, const void* in_c64, void* out_c64, void* stream);
int dlx_fft_adjoint(dlx_fft_plan plan, const void* gout_c64, void* gin_c64, void* stream);

/* ---- a5-a11: phasor build ----------------------------------------------
 * Replaces the elementwise wavefront updates of wavefronts.py:70-122
 * (1/N^2 initial field), :332-368 (add_phase / add_opd), :370-395 (tilt),
 * layers/optical_layers.py:181-186 and layers/optics.py:77-96 (transmission),
 * fused into one pass:
 *   out[b][y][x] = (in ? in[b][y][x] : 1) * scale_b * amp[y][x]
 *                  * exp(i (2 pi (opd[y][x] + tx*X + ty*Y) / lambda_b + phase[y][x]))
 * scale_b = (amp_scale ? *amp_scale : 1) * (weights ? sqrt(weights[b]) : 1) * const_scale.
 * X, Y are the wavefront pixel centres (pixel_scale, centre 0). amp, opd,
 * phase, in, amp_scale and weights may be NULL. The phase is reduced in
 * cycles in FP64 before sincos. in/out may alias.
 */
int dlx_phasor(const void* in_c64, const float* amp, const float* opd, const float* phase,
               const float* amp_scale, const float* weights, double const_scale,
               const double* wavelengths_host, int batch, int n, double pixel_scale,
               double tilt_x, double tilt_y, void* out_c64, void* stream);
/* Reverse pass of dlx_phasor as the layer-by-layer path calls it (no tilt,
 * amp_scale, weights or const_scale): for out_b = in_b * amp * u_b with
 * u_b = exp(i (2 pi opd / lambda_b + phase)),
 *   g_in_b = g_b conj(amp u_b),   g_amp = sum_b Re(conj(in_b u_b) g_b),
 *   g_phase = sum_b Im(conj(out_b) g_b),   g_opd = sum_b (2 pi / lambda_b) Im(...).
 * Replaces JAX's reverse mode of Wavefront.add_opd / add_phase
 * (wavefronts.py:332-368) and of the real multiply (wavefronts.py:834-906).
 * u_b is rebuilt with the forward's own reduction, bit for bit. in, amp, opd,
 * phase and every output may be NULL (in NULL: a field of ones). */
int dlx_phasor_backward(const void* in_c64, const float* amp, const float* opd,
                        const float* phase, const double* wavelengths_host, int batch, int n,
                        const void* g_c64, void* g_in_c64, float* g_amp, float* g_opd,
                        float* g_phase, void* stream);

/* ---- a8: power and normalisation ----------------------------------------
 * Wavefront.normalise (wavefronts.py:397-424), mode "power":
 * out_scale[b] = sqrt(value / sum |in[b]|^2). Deterministic two-level reduction.
 */
int dlx_power_scale(const void* in_c64, int batch, int n, double value,
                    float* out_scale, void* stream);
/* Wavefront.normalise (wavefronts.py:397-424) on each plane of a batch:
 * out[b] = in[b] * s_b with s_b = sqrt(value / P_b), P_b = sum |in[b]|^2
 * (mode 0, "power") or max |in[b]|^2 (mode 1, "peak"); out_scale[b] = s_b
 * (NULL: not written). Another mode is refused with dLux's message. */
int dlx_normalise(const void* in_c64, int batch, long long npix, int mode, double value,
                  void* out_c64, float* out_scale, void* stream);
/* Its reverse pass: g_in = s g - in s D / P with D = sum Re(conj(g) in), on
 * every pixel (power) or on the pixels at the peak, shared equally among ties
 * (peak), as JAX's reverse mode of max shares it. */
int dlx_normalise_backward(const void* in_c64, int batch, long long npix, int mode,
                           double value, const void* g_c64, void* g_in_c64, void* stream);
/* Same for a real amplitude: out_scale = sqrt(value / sum amp^2). */
int dlx_amp_norm(const float* amp, int n, double value, float* out_scale, void* stream);
/* Reverse of a_eff = amp * sqrt(value / sum amp^2): g_amp from g_eff. */
int dlx_amp_norm_backward(const float* amp, const float* g_eff, int n, double value,
                          float* g_amp, void* stream);

/* ---- a9 / a21: basis contraction and its reverse ------------------------
 * eval_basis (utils/math.py:177-196): out[p] = base[p] + sum_k coeffs[k] basis[k][p].
 * coeffs is a device pointer; base may be NULL.
 */
int dlx_basis_eval(const float* basis, const float* coeffs, const float* base,
                   int nterms, long long npix, float* out, void* stream);
/* g_coeffs[k] = sum_p basis[k][p] g[p] (deterministic, fixed order). */
int dlx_basis_grad(const float* basis, const float* g, int nterms, long long npix,
                   float* g_coeffs, void* stream);

/* ---- a16/a13: intensity ------------------------------------------------
 * Wavefront.psf (wavefronts.py:269-279) summed over the batch
 * (optical_systems.py:222-223): psf[p] = sum_b |in[b][p]|^2.
 */
int dlx_psf_sum(const void* in_c64, int batch, long long npix, float* psf, void* stream);
/* The PSF of OpticalSystem.propagate (optical_systems.py:211-223) from the
 * unweighted focal fields: psf[p] = sum_b w_b |in[b][p]|^2 (weights NULL: 1),
 * i.e. the field times sqrt(w_b) in dLux's vmap body, then the sum of |E|^2. */
int dlx_psf_sum_weighted(const void* in_c64, const float* weights, int batch, long long npix,
                         float* psf, void* stream);
/* Its reverse pass: g_in[b][p] = 2 w_b g[p] in[b][p] and
 * g_weights[b] = sum_p g[p] |in[b][p]|^2 (each output may be NULL). */
int dlx_psf_sum_weighted_backward(const void* in_c64, const float* weights, int batch,
                                  long long npix, const float* g, void* g_in_c64,
                                  float* g_weights, void* stream);

/* ---- a17/a18: detector ---------------------------------------------------
 * downsample(mean=False) (utils/array_ops.py:124-162, psfs.py:74-91) fused
 * with ApplyPixelResponse (layers/detector_layers.py:100-131):
 * out[a][c] = (flat ? flat[a][c] : 1) * sum_{i,j<k} in[a k + i][c k + j].
 * k = 1 gives the pixel response alone. mean != 0 divides by k*k.
 */
int dlx_downsample(const float* in, int n_in, int k, int mean, const float* flat,
                   float* out, void* stream);
/* Reverse: g_in[y][x] = g_out[y/k][x/k] * flat(...) (/k^2 if mean);
 * g_flat[a][c] = g_out[a][c] * downsample(in) (g_flat may be NULL). */
int dlx_downsample_backward(const float* in, const float* g_out, int n_in, int k, int mean,
                            const float* flat, float* g_in, float* g_flat, void* stream);

/* ---- fused polychromatic PSF plan ----------------------------------------
 * The whole of OpticalSystem.propagate (optical_systems.py:147-223) for a
 * layered system whose layers reduce to a wavelength-independent amplitude,
 * OPD and phase (Transmissive/Basis/Aberrated/Optic/BasisOptic/Tilt/
 * Normalise layers) followed by AngularOpticalSystem.to_focus
 * (optical_systems.py:659-680) or CartesianOpticalSystem.to_focus
 * (:754-775):
 *   psf = sum_l |MFT_l( sqrt(w_l) amp exp(i (2 pi (opd + tilt)/lambda_l + phase)) )|^2
 * and its reverse-mode gradient, which recomputes every focal field instead
 * of storing it.
 */
typedef struct dlx_poly_plan_s* dlx_poly_plan;
typedef struct {
  int n_wavelengths;      /* L */
  int n_in;               /* pupil side N */
  int n_out;              /* focal side M (psf_npixels * oversample) */
  double pixel_scale_in;  /* diameter / N */
  double pixel_scale_out; /* rad/pixel (angular) or m/pixel */
  double focal_length;    /* 0: angular; < 0 is refused */
  int variant;            /* DLX_VARIANT_* */
  int operand_mode;       /* split form only: 0 = cached DFT matrices streamed by TMA,
                             1 = DFT operand generated inside the GEMM (no cached matrices) */
} dlx_poly_desc;

int dlx_poly_plan_create(const dlx_poly_desc* desc, const double* wavelengths_host,
                         dlx_poly_plan* plan);

/* One independent object of a batched evaluation: a request of the serving
 * loop, or one point source of PointSources.model (sources.py:392-411, which
 * vmaps optics.propagate over positions). All pointers are device pointers;
 * any may be NULL where the matching quantity is absent or not wanted.
 * weights [L] carry the source's spectral weights times its flux. */
typedef struct {
  const float* amp;        /* [N][N] pupil amplitude (NULL: 1) */
  const float* amp_scale;  /* device scalar multiplying amp (e.g. from dlx_amp_norm) */
  const float* opd;        /* [N][N] OPD in metres */
  const float* phase;      /* [N][N] phase in radians */
  const float* weights;    /* [L] */
  double tilt_x, tilt_y;   /* source offset in radians (the initial wavefront tilt) */
  float* psf;              /* [M][M] output of dlx_poly_forward (NULL: only summed) */
  const float* g_psf;      /* [M][M] cotangent for dlx_poly_backward */
  float* g_amp;            /* [N][N] d/d effective amplitude */
  float* g_opd;            /* [N][N] */
  float* g_phase;          /* [N][N] */
  float* g_w;              /* [L] */
  float* g_tilt;           /* [2] d/d (tilt_x, tilt_y) */
} dlx_poly_object;

/* Plan for up to max_objects (<= 32) objects per launch; the per-wavelength
 * DFT operands are shared by all objects of a batch, so the GEMMs run over
 * L x objects fields in one launch. */
int dlx_poly_plan_create_batched(const dlx_poly_desc* desc, const double* wavelengths_host,
                                 int max_objects, dlx_poly_plan* plan);
/* A plan that owns only its cached per-wavelength state (DFT operands,
 * scales); the per-call buffers come from caller workspace attached with
 * dlx_poly_attach_workspace before each use. Lets many resident plans (e.g.
 * one per serving bucket) share a few workspaces, one per stream in use.
 * dlx_poly_workspace_bytes gives the size a plan of this description needs. */
int dlx_poly_plan_create_shared(const dlx_poly_desc* desc, const double* wavelengths_host,
                                int max_objects, dlx_poly_plan* plan);
int dlx_poly_workspace_bytes(const dlx_poly_desc* desc, int max_objects, size_t* bytes);
/* workspace: 256-byte aligned device memory of at least the size above. The
 * plan uses it until another workspace is attached; the caller keeps it alive
 * and must not use it for anything else while the plan's work is in flight. */
int dlx_poly_attach_workspace(dlx_poly_plan plan, void* workspace, size_t bytes);
/* PSFs of n_objects objects (any count; runs in chunks of the plan's capacity):
 * per-object PSFs into objs[r].psf and/or their sum into psf_sum (added to its
 * contents when accumulate != 0). The sum over objects is the PointSources
 * image (sources.py:409-411). */
int dlx_poly_forward(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                     float* psf_sum, int accumulate, void* stream);
/* Reverse pass for every object with its own cotangent objs[r].g_psf. */
int dlx_poly_backward(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                      void* stream);
/* Forward-to-backward reuse, the counterpart of the residuals a jax.custom_vjp
 * forward hands to its backward (here they stay in the plan's fixed
 * workspace, so no memory is added). After a dlx_poly_forward of at most
 * max_objects objects, the workspace holds that forward's pupil field, its
 * first-stage product D1 and the path pairs until the next call on the plan.
 * dlx_poly_forward_token returns a token for that state (0 if none is intact).
 * dlx_poly_reuse_forward(token) lets the next dlx_poly_backward /
 * dlx_poly_psf_grad start from it: it skips the phasor rebuild and the first
 * MFT stage, and recomputes the per-wavelength focal field from D1 unless
 * that forward kept it (dlx_poly_keep_focal).
 * The request covers one backward call. It is ignored, and the backward
 * recomputes everything, if another call used the plan in between or the
 * objects' inputs (amp, amp_scale, opd, phase, weights, tilt pointers and
 * values) differ. The caller orders the backward after the forward on the
 * device, as for any two calls on one plan. */
int dlx_poly_forward_token(dlx_poly_plan plan, unsigned long long* token);
/* Split K for the tensor-core GEMMs of poly plans created after the call
 * with their own workspace (default on): a GEMM whose output tiles over the
 * plan's capacity (wavelengths x max_objects) would leave most SMs idle runs
 * each tile as up to 8 K ranges in parallel and sums the FP32 partials in a
 * fixed order. The choice is made per plan, so an object's result is the
 * same alone and in a batch of that plan. Plans on a shared workspace
 * (dlx_poly_plan_create_shared) do not split. No dLux counterpart. */
int dlx_set_split_k(int enable);
/* Paired form of the loaded-operand tensor-core GEMM (default off; also
 * DLX_GEMM_PAIR=1 in the environment): a GEMM with an even number of
 * 128-column output tiles and no split K runs in clusters of two CTAs that
 * issue 256-row MMAs (cta_group::2), each CTA loading half of the A tile.
 * Results are bitwise the single-CTA form's. Read at every launch (CUDA
 * graphs keep the form they were captured with). No dLux counterpart. */
int dlx_set_gemm_pair(int enable);
/* Two-CTA clusters of the paired GEMM that fit on the device at once (0: the
 * paired form is unavailable). No dLux counterpart. */
int dlx_gemm_pair_clusters(int* clusters);
/* Launch form of one poly plan's tensor-core GEMMs, for the autotuner:
 * pair_mode 0 follows dlx_set_gemm_pair, 1 never pairs, 2 pairs wherever the
 * shape allows (an even number of 128-column tiles and no split K);
 * split_k 0 keeps every GEMM whole, 1 uses the K split the plan chose at
 * creation (if any). Applies to the plan's later calls (CUDA graphs keep the
 * form they were captured with); each choice is fixed per plan, so an
 * object's result stays the same alone and in a batch. No dLux counterpart. */
int dlx_poly_plan_set_gemm_form(dlx_poly_plan plan, int pair_mode, int split_k);
int dlx_poly_reuse_forward(dlx_poly_plan plan, unsigned long long token);
/* Focal fields kept for the reverse pass, the residual a jax.custom_vjp
 * forward of MFT -> |.|^2 would save (JAX keeps the focal field F for the
 * backward of optical_systems.py:211-223). With keep != 0 the next
 * dlx_poly_forward (or dlx_poly_psf) of at most max_objects objects also
 * writes F = alpha D of every wavelength into the plan's workspace (8 bytes
 * per focal pixel and wavelength, already part of the workspace size). A
 * backward that reuses that forward (dlx_poly_reuse_forward) then forms
 * F-bar = 2 G F elementwise instead of repeating the y-contraction GEMM. The
 * request covers one forward call; without a reusing backward the kept fields
 * are simply overwritten later. */
int dlx_poly_keep_focal(dlx_poly_plan plan, int keep);
/* PSF and reverse pass in one sweep for objects whose cotangent objs[r].g_psf
 * is known before the forward pass (a serving request, a linear functional):
 * writes objs[r].psf (optional) and the gradient outputs like
 * dlx_poly_backward, without recomputing the forward fields (4 instead of 6
 * GEMMs). No dLux counterpart: JAX's reverse mode always runs after its
 * forward pass. */
int dlx_poly_forward_backward(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                              void* stream);
/* Same, for objects that share one pupil (the sources of one scene): the
 * pupil-pixel gradients are summed over all objects into g_amp / g_opd /
 * g_phase ([N][N], any may be NULL; overwritten), while g_w and g_tilt stay
 * per object (source fluxes and positions). */
int dlx_poly_backward_sum(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                          float* g_amp, float* g_opd, float* g_phase, void* stream);
int dlx_poly_plan_destroy(dlx_poly_plan plan);
/* Device bytes the plan owns: cached DFT matrices, plus its intermediates
 * unless it was made with dlx_poly_plan_create_shared. */
int dlx_poly_plan_footprint(dlx_poly_plan plan, size_t* bytes);
/* Shape of a plan; any output pointer may be NULL. */
int dlx_poly_plan_info(dlx_poly_plan plan, int* n_wavelengths, int* n_in, int* n_out,
                       int* max_objects);

/* ---- f4: ABCD propagators -------------------------------------------------
 * Device side of dLux's MFTPropagator, FFTPropagator and ASMPropagator
 * (layers/abcd_propagators.py:245-459). The reference takes their arithmetic
 * from the abcdLux package (lct.lct_prop, lct.lct_prop_fft, asm.asm_prop;
 * pyproject.toml:21 "abcdLux>=0.0.2", not vendored), restated here from the
 * published linear canonical transform and angular-spectrum method.
 *
 * Separable transform: out[b] = A_y[b] in[b] A_x[b]^T with generated
 * matrices, element (j, i) of an axis being
 *   scale * exp(2 pi i [sigma x_i u_j + q_in x_i^2 + q_out u_j^2 + phase]),
 *   x_i = a_in i + b_in,  u_j = a_out j + b_out      (all FP64 at creation).
 * The LCT of an ABCD system (Collins integral) per axis is sigma = -1/(lambda B),
 * q_in = A/(2 lambda B), q_out = D/(2 lambda B), phase = -sign(B)/8 and
 * scale = dx/sqrt(lambda |B|). Same forms and split-BF16 tensor-core GEMMs as
 * the MFT plan. */
typedef struct {
  double a_in, b_in;    /* input coordinate x_i = a_in * i + b_in */
  double a_out, b_out;  /* output coordinate u_j = a_out * j + b_out */
  double sigma;         /* cycles per x * u */
  double q_in, q_out;   /* cycles per x^2 and per u^2 */
  double phase;         /* constant phase, cycles */
  double scale;         /* real factor */
} dlx_xform_axis;
typedef struct {
  int batch, n_in, n_out;
  int variant;          /* DLX_VARIANT_FP32 or DLX_VARIANT_SPLIT_BF16 */
} dlx_xform_desc;
typedef struct dlx_xform_plan_s* dlx_xform_plan;
/* ax_x, ax_y: host arrays of batch axes each. */
int dlx_xform_plan_create(const dlx_xform_desc* desc, const dlx_xform_axis* ax_x,
                          const dlx_xform_axis* ax_y, dlx_xform_plan* plan);
int dlx_xform_plan_destroy(dlx_xform_plan plan);
/* in [batch][n_in][n_in] c64 -> out [batch][n_out][n_out] c64, and its adjoint. */
int dlx_xform_forward(dlx_xform_plan plan, const void* in_c64, void* out_c64, void* stream);
int dlx_xform_adjoint(dlx_xform_plan plan, const void* gout_c64, void* gin_c64, void* stream);

/* Angular-spectrum propagation over `distance` (asm.asm_prop, called at
 * layers/abcd_propagators.py:442-449): the field is zero-padded (centred) from
 * n_in to n_pad pixels, transformed by a centred DFT, multiplied by
 * exp(2 pi i z sqrt(1/lambda^2 - fx^2 - fy^2)) (evanescent components decay
 * as exp(-2 pi z sqrt(f^2 - 1/lambda^2))) and transformed back; the output
 * keeps the pixel scale. The phase is formed in FP64 on the device. */
typedef struct {
  int batch, n_in, n_pad;
  double pixel_scale;   /* m */
  double distance;      /* m */
  int variant;
} dlx_asm_desc;
typedef struct dlx_asm_plan_s* dlx_asm_plan;
int dlx_asm_plan_create(const dlx_asm_desc* desc, const double* wavelengths_host,
                        dlx_asm_plan* plan);
int dlx_asm_plan_destroy(dlx_asm_plan plan);
/* in [batch][n_in][n_in] c64 -> out [batch][n_pad][n_pad] c64, and its adjoint. */
int dlx_asm_forward(dlx_asm_plan plan, const void* in_c64, void* out_c64, void* stream);
int dlx_asm_adjoint(dlx_asm_plan plan, const void* gout_c64, void* gin_c64, void* stream);

/* ---- a12: dynamic aberrated apertures --------------------------------------
 * Replaces AberratedAperture over a CircularAperture, SquareAperture,
 * RectangularAperture or RegPolyAperture (layers/apertures.py:240-555,
 * 643-800): the soft-edged transmission (utils/geometry.py:49-91, 229-351,
 * 402-579) and OPD = sum_j coeffs[j] Z_noll[j] (polynomials.py:20-51,
 * utils/zernikes.py:122-294) at the coordinates divided by the aperture's
 * extent -- for the polygonal shapes the polygon-stretched Zernikes of
 * utils/zernikes.py:318-419 with the shape's side count (4 for squares and
 * rectangles) -- evaluated per pixel on the device after dLux's
 * CoordTransform (coordinates.py:240-320: translate, shear, compress,
 * rotate). No basis array is read or stored. Up to 64 terms, radial order
 * <= 16 (both outputs may be NULL). dlx_aberrated_aperture_grad returns
 * d<g_opd, opd>/d coeffs. dlx_zernike_table is host-only: the (n, m) of each
 * Noll index and its radial coefficients (9 per term, highest power of
 * rho^2 first).
 */
#define DLX_APERTURE_CIRCLE 0    /* radius */
#define DLX_APERTURE_SQUARE 1    /* width */
#define DLX_APERTURE_RECTANGLE 2 /* width (x) and height (y) */
#define DLX_APERTURE_POLYGON 3   /* nsides (3..32) and radius = rmax */
typedef struct {
  int npixels;             /* wavefront side N */
  double pixel_scale;      /* m per pixel */
  double translation[2];   /* m */
  double rotation;         /* rad, clockwise */
  double compression[2];
  double shear[2];
  double radius;           /* m: circle radius, or polygon circumradius (rmax) */
  double softening;        /* soft edge width in pixels (> 0) */
  int occulting;
  int shape;               /* DLX_APERTURE_* */
  double width;            /* m: square side, rectangle x side */
  double height;           /* m: rectangle y side */
  int nsides;              /* regular polygon sides */
} dlx_aperture_desc;
int dlx_zernike_table(const int* noll, int n_terms, int* n_out, int* m_out, float* coeffs_out);
int dlx_aberrated_aperture(const dlx_aperture_desc* desc, const int* noll_host, int n_terms,
                           const float* coeffs, float* transmission, float* opd, void* stream);
int dlx_aberrated_aperture_grad(const dlx_aperture_desc* desc, const int* noll_host, int n_terms,
                                const float* g_opd, float* g_coeffs, void* stream);

/* ---- PSF convolution, mode "same" ---------------------------------------
 * Replaces jax.scipy.signal.convolve(psf, kernel, mode="same") of
 * PSF.convolve (psfs.py:93-110), ResolvedSource / PointResolvedSource
 * (sources.py:490-521, 711-748) and ApplyJitter
 * (layers/detector_layers.py:134-199): out[i][j] = sum_{a,b}
 * in[i + (K0-1)/2 - a][j + (K1-1)/2 - b] kernel[a][b], zero outside `in`, for a
 * batch of [H][W] images and one [K0][K1] kernel (sides <= 128). The backward
 * gives d/d in and d/d kernel (summed over the batch); either may be NULL.
 */
int dlx_conv2d_same(const float* in, int batch, int height, int width, const float* kernel,
                    int k0, int k1, float* out, void* stream);
int dlx_conv2d_same_backward(const float* in, int batch, int height, int width,
                             const float* kernel, int k0, int k1, const float* g_out,
                             float* g_in, float* g_kernel, void* stream);

/* ---- a20/a21: many point sources through one pupil ---------------------
 * Replaces PointSources.model (sources.py:392-411) for a pupil that does not
 * need gradients: image [M][M] = sum_s sum_l weights[s][l] PSF_l(position_s),
 * with the source tilt (wavefronts.py:370-395) folded into per-source DFT
 * matrices (an output-coordinate shift) instead of a tilted pupil field per
 * source. positions: device double [S][2] (rad, x then y); weights: device
 * float [S][L] (spectrum x flux). amp/amp_scale/opd/phase as dlx_poly_psf.
 * The reverse pass gives d/d(position) (float [S][2]) and d/d(weights)
 * (float [S][L]); either output may be NULL. Sources are processed
 * max_sources (<= 32) at a time.
 */
typedef struct dlx_scene_plan_s* dlx_scene_plan;
typedef struct {
  int n_wavelengths;
  int n_in;                /* pupil side N */
  int n_out;               /* PSF side M */
  double pixel_scale_in;   /* pupil pixel (m) */
  double pixel_scale_out;  /* PSF pixel (rad, or m with focal_length) */
  double focal_length;     /* 0: angular; < 0 is refused */
  int variant;             /* DLX_VARIANT_* */
  int max_sources;         /* sources per launch, 1..32 */
} dlx_scene_desc;
int dlx_scene_plan_create(const dlx_scene_desc* desc, const double* wavelengths_host,
                          dlx_scene_plan* plan);
int dlx_scene_plan_destroy(dlx_scene_plan plan);
int dlx_scene_plan_footprint(dlx_scene_plan plan, size_t* bytes);
int dlx_scene_forward(dlx_scene_plan plan, const float* amp, const float* amp_scale,
                      const float* opd, const float* phase, const double* positions,
                      const float* weights, int n_sources, float* image, int accumulate,
                      void* stream);
int dlx_scene_backward(dlx_scene_plan plan, const float* amp, const float* amp_scale,
                       const float* opd, const float* phase, const double* positions,
                       const float* weights, int n_sources, const float* g_image, float* g_pos,
                       float* g_weights, void* stream);
/* Forward-to-backward retention, as for poly plans. A dlx_scene_forward
 * whose retained fields fit the plan's limit (default 48 GiB; 0 disables)
 * keeps every source chunk's half-transformed fields D1 and Y.D1, i.e.
 * 2 x n_sources x n_wavelengths x n_out x n_in complex values. The buffer is
 * allocated outside stream capture only. dlx_scene_forward_token returns a
 * token for that state (0 if none). After dlx_scene_reuse_forward(token),
 * the next dlx_scene_backward with the same input pointers starts from
 * those fields instead of repeating the first GEMM, and still recomputes the
 * focal fields. Otherwise it recomputes everything. */
int dlx_scene_forward_token(dlx_scene_plan plan, unsigned long long* token);
int dlx_scene_reuse_forward(dlx_scene_plan plan, unsigned long long token);
int dlx_scene_set_retain_limit(dlx_scene_plan plan, size_t bytes);

/* ---- Serving batch ----
 * No counterpart in dLux, which has no serving loop. One batch of requests
 * that share a plan (same N, M and wavelengths), each with its own Zernike
 * coefficients and spectral weights; the first n_grad requests also want
 * d<g_psf, PSF>/d coefficients. Everything is stream-ordered on `stream`:
 * host->device copies of the inputs, OPD = basis . coefficients per request,
 * the fused forward (and reverse) pass, the coefficient gradient and the
 * device->host copies of PSFs and gradients. The call allocates nothing and
 * synchronises nothing, so a batch can be captured in a CUDA graph once
 * the plan's workspace is attached and replayed while the buffers stay put.
 * Host buffers must be pinned for the copies to be asynchronous. */
typedef struct dlx_serve_batch {
  int n_objects;           /* R, 1..max_objects of the plan */
  int n_grad;              /* 0..R: requests 0..n_grad-1 want gradients */
  int n_coeffs;            /* K: basis terms (coefficients zero-padded to K) */
  const float* basis;      /* device [K][N][N] */
  const float* amp;        /* device [N][N] aperture transmission */
  const float* amp_scale;  /* device scalar multiplying amp, or NULL for 1 */
  const float* h_coeffs;   /* host [R][K] */
  const float* h_weights;  /* host [R][L] */
  const float* h_g_psf;    /* host [n_grad][M][M] cotangents (NULL if n_grad == 0) */
  float* h_psf;            /* host [R][M][M] result */
  float* h_grad;           /* host [n_grad][K] result (NULL if n_grad == 0) */
  void* d_work;            /* device scratch of dlx_serve_workspace_bytes, 256-B aligned */
  size_t d_work_bytes;
} dlx_serve_batch;
int dlx_serve_workspace_bytes(int max_objects, int n_coeffs, int n_in, int n_out,
                              int n_wavelengths, size_t* bytes);
int dlx_serve_run(dlx_poly_plan plan, const dlx_serve_batch* batch, void* stream);
/* psf_out [M][M] = polychromatic PSF. amp, amp_scale (device scalar that
 * multiplies amp, e.g. from dlx_amp_norm), opd, phase and weights ([L]) are
 * device pointers and may be NULL (1, 1, 0, 0, 1). tilt is the source offset
 * in radians (initialise_wavefront, optical_systems.py:363-389). */
int dlx_poly_psf(dlx_poly_plan plan, const float* amp, const float* amp_scale, const float* opd,
                 const float* phase, const float* weights, double tilt_x, double tilt_y,
                 float* psf_out, void* stream);
/* Gradient of <g_psf, psf> w.r.t. the effective amplitude (amp * amp_scale),
 * opd, phase ([N][N]) and weights ([L]). Any output pointer may be NULL (not
 * computed). The focal fields are recomputed, not stored. */
int dlx_poly_psf_grad(dlx_poly_plan plan, const float* amp, const float* amp_scale,
                      const float* opd, const float* phase, const float* weights, double tilt_x,
                      double tilt_y, const float* g_psf, float* g_amp, float* g_opd,
                      float* g_phase, float* g_w, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DLUXGB_H */
