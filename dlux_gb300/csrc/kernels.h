// kernels.h -- host launchers shared between the translation units.
#pragma once

#include "common.cuh"

namespace dlx {

// focal_length of the C ABI: 0 selects the angular form (dLux's
// focal_length=None), a positive value the Cartesian form. A negative value is
// refused: dLux's own MFT takes log(nfringes), which is NaN for it.
int check_focal(double focal_length, const char* who);

// Per-batch double scalars passed by value (chunks of up to kMaxBatchArg).
constexpr int kMaxBatchArg = 256;
struct BatchD {
  double v[kMaxBatchArg];
};
// Per-batch (hi, lo) float pairs, e.g. 1 / lambda for the FP32 phase reduction.
struct BatchFF {
  float2 v[kMaxBatchArg];
};

// --- elementwise.cu --------------------------------------------------------
// Angular-spectrum transfer function: tabulated once per plan into H
// [batch][P][P] (complex64), then applied in place to centred spectra
// (conj != 0: its conjugate, the adjoint).
int launch_asm_table(float2* H, int batch, int P, double df, const double* zl,
                     const double* lam2, cudaStream_t s);
int launch_asm_apply(float2* spec, const float2* H, int batch, int P, int conj, cudaStream_t s);
int launch_dft_gen(const DftAxis* axes_dev, int batch, int rows, int cols, bool rows_are_out,
                   float2* out_c64, long long out_batch_stride, __nv_bfloat16* out_split,
                   cudaStream_t s);

// Independent objects (requests, sources) evaluated in one batch: batch index
// b = l * n + r for wavelength l and object r, so the per-wavelength DFT
// operand is shared by all objects (A index = b / n). Passed by value.
constexpr int kMaxObj = 32;
struct ObjDesc {
  const float* amp;        // nullable [N][N]
  const float* amp_scale;  // nullable device scalar
  const float* opd;        // nullable [N][N]
  const float* phase;      // nullable [N][N]
  const float* weights;    // nullable [L]
  const float* G;          // [M][M] cotangent (reverse pass)
  double tilt_x, tilt_y;
};
struct ObjTable {
  int n;                   // 0: not used (single-object fields of the enclosing struct)
  ObjDesc o[kMaxObj];
};
struct ObjOut {
  float* psf;              // [M][M] per-object PSF, nullable
  float* g_amp;            // [N][N], nullable
  float* g_opd;
  float* g_phase;
  float* g_w;              // [L]
  float* g_tilt;           // [2]
};
struct OutTable {
  int n;
  ObjOut o[kMaxObj];
};

struct PhasorArgs {
  ObjTable objs;           // when objs.n > 0 the per-object fields replace the ones below
  const float2* in;        // nullable [b][n][n]
  const float* amp;        // nullable [n][n]
  const float* opd;        // nullable [n][n]
  const float* phase;      // nullable [n][n]
  const float* amp_scale;  // nullable device scalar
  const float* weights;    // nullable [b]
  const float2* inv_lambda_ff;   // [b] (hi, lo) of 1/lambda (device), or nullptr -> by value
  double const_scale;
  int batch, n;
  double pixel_scale, tilt_x, tilt_y;
  float2* out_c64;             // one of the two outputs
  __nv_bfloat16* out_split;    // [b][4][n][n]
  // nullable [object][n][n]: (path hi, path lo, phase hi, phase lo) per pixel, the
  // wavelength-independent inputs of cis_ff, for the reverse pass's epilogue
  float4* out_path;
};
int launch_phasor(const PhasorArgs& a, const BatchFF* inv_lambda_arg, cudaStream_t s);

int launch_c64_to_split_batched(const float2* in, int rows, int cols, int batch,
                                __nv_bfloat16* out_split, cudaStream_t s);
// F-bar = 2 G_r F from kept focal fields F [batch][M][M] (complex64, b = l R +
// r): split planes [batch][4][M][split_ld(M)] into out_split, or complex64
// into out_c64 (which may be f itself).
int launch_focal_gradf(const float2* f, const ObjTable& objs, int batch, int M,
                       __nv_bfloat16* out_split, float2* out_c64, cudaStream_t s);
int launch_psf_sum(const float2* in, int batch, long long npix, float* psf, cudaStream_t s);
int launch_power_scale(const float2* in, int batch, long long npix, double value, float* out,
                       cudaStream_t s);
int launch_amp_norm(const float* amp, long long npix, double value, float* out_scale,
                    double* partial_ws, int nparts, cudaStream_t s);
int launch_amp_norm_backward(const float* amp, const float* g_eff, long long npix, double value,
                             float* g_amp, double* partial_ws, int nparts, cudaStream_t s);
int launch_basis_eval(const float* basis, const float* coeffs, const float* base, int nterms,
                      long long npix, float* out, cudaStream_t s);
int basis_grad_parts(int nterms, long long npix, int sms);
int launch_basis_grad(const float* basis, const float* g, int nterms, long long npix,
                      float* g_coeffs, double* partial_ws, int nparts, cudaStream_t s);
int launch_downsample(const float* in, int n_in, int k, int mean, const float* flat, float* out,
                      cudaStream_t s);
int launch_downsample_backward(const float* in, const float* g_out, int n_in, int k, int mean,
                               const float* flat, float* g_in, float* g_flat, cudaStream_t s);

// Per-object reductions of a batched plan (b = l * R + r).
struct ObjReduceArgs {
  ObjTable objs;
  OutTable outs;
  int L;                     // wavelengths
  long long npix;            // pixels per plane
  const float* planes;       // intensity planes [L*R][npix]
  const float2* fields;      // or (when set) kept focal fields F = alpha D [L*R][npix]:
                             // the wavelength sum forms |F|^2 itself
  float* psf_sum;            // nullable: sum over objects (and wavelengths)
  int accumulate;            // add into psf_sum instead of overwriting it
  const float* pre;          // pupil planes [L*R][npix]
  const float* pim;
  const double* k_dev;       // [L] 2 pi / lambda
  int n_side;                // pupil side (tilt gradients)
  double pixel_scale;
  double* partial_ws;        // >= R * nparts * (L + 2) doubles
  int nparts;
  // Pixel gradients summed over all objects into these (objects share one
  // pupil); when set, outs.o[r].g_amp/g_opd/g_phase are ignored.
  float* sum_g_amp;
  float* sum_g_opd;
  float* sum_g_phase;
  int sum_pixels;
  int accumulate_sum;        // add into the sums instead of overwriting them
  // Fused form (launch_obj_pupil_fused): the reverse pass's pupil field
  // Ebar [L*R][npix] (alpha applied) and the phasor kernel's (path, phase)
  // pairs [R][npix] replace the pre/pim planes.
  const float2* ebar;
  const float4* path;
  const float2* inv_lambda_ff;  // [L]
  float* pix_scratch;        // [R][3][npix] per-object pixel sums (sum_pixels only)
  int split_form;            // the plan's split-BF16 form: phasors by cis_ff_split
};
int launch_obj_psf_reduce(const ObjReduceArgs& a, cudaStream_t s);
int launch_obj_pupil_reduce(const ObjReduceArgs& a, cudaStream_t s);
// Largest wavelength count the fused pupil reduction accepts.
constexpr int kFusedPupilMaxL = 2048;
int launch_obj_pupil_fused(const ObjReduceArgs& a, cudaStream_t s);


// --- zernike.cu: dynamic aperture + Zernike aberrations ----------------------
constexpr int kMaxZern = 64;       // terms per call
constexpr int kMaxZernCoeff = 9;   // radial coefficients per term ((n - |m|)/2 + 1)
struct ZernTable {                 // passed by value
  int K;
  int n[kMaxZern], m[kMaxZern], nc[kMaxZern];
  float norm[kMaxZern];
  float c[kMaxZern][kMaxZernCoeff];  // highest power of rho^2 first
};
constexpr int kMaxPolySides = 32;  // sides of a regular-polygon aperture
enum ApertureShape { AP_CIRCLE = 0, AP_SQUARE = 1, AP_RECTANGLE = 2, AP_POLYGON = 3 };
struct ZernAperture {
  int n;                  // pixels per side
  float pixel_scale;      // m
  float translation[2], shear[2], compression[2];
  float rot_c, rot_s;     // cos(-rotation), sin(-rotation)
  int shape;              // ApertureShape
  float radius;           // circle radius / polygon circumradius, m
  float half_w, half_h;   // square and rectangle half widths, m
  float extent;           // m: the Zernikes are evaluated at coordinates / extent
  int nsides;             // 0: Zernikes; >= 3: polygon-stretched Zernikes with that many sides
  int n_edges;            // polygon edges: signed distance a x + b y + c, the largest wins
  float edge_a[kMaxPolySides], edge_b[kMaxPolySides], edge_c[kMaxPolySides];
  float clip;             // soft-edge half width, m
  int occulting;
};
int launch_aperture_eval(const ZernAperture& a, const ZernTable& z, const float* coeffs,
                         unsigned* minmax_ws, float* trans, float* opd, cudaStream_t s);
int launch_zernike_grad(const ZernAperture& a, const ZernTable& z, const float* g, double* partial,
                        int nparts, float* g_coeffs, cudaStream_t s);

// --- fft.cu: radix-2 form of the padded centred FFT --------------------------
struct LineRamp;
struct RadixFft {
  int batch = 0, N = 0, P = 0, log2p = 0, npad = 0, c = 0;
  float sign = -1.0f;           // forward transform direction
  LineRamp* ramps_x = nullptr;  // device [batch]: forward x, forward y (with the
  LineRamp* ramps_y = nullptr;  // normalisation), adjoint x, adjoint y
  LineRamp* ramps_ax = nullptr;
  LineRamp* ramps_ay = nullptr;
  float2* tmp = nullptr;        // device [batch][N][P]
  float2* tw = nullptr;         // device [P - 1]: butterfly twiddles, stage by stage
};
int radix_fft_create(RadixFft* f, int batch, int N, int pad, bool inverse, const DftAxis* axes,
                     const float* alphas);
void radix_fft_release(RadixFft* f);
int radix_fft_forward(const RadixFft& f, const float2* in, float2* out, cudaStream_t s);
int radix_fft_adjoint(const RadixFft& f, const float2* gout, float2* gin, cudaStream_t s);

// --- gemm_fp32.cu / gemm_tc.cu ---------------------------------------------
// Complex GEMM D[b][m][n] = sum_k opA(A[b][m][k]) * B[b][n][k], opA = conj if conj_a.
// Epilogue kinds shared by both arithmetic forms.
enum EpiKind {
  EPI_C64 = 0,       // out_c64[b][m][n] = alpha_b * D
  EPI_SPLIT = 1,     // out_split[b][4][m][n] = split(alpha_b * D)   (tensor-core form only)
  EPI_INTENSITY = 2, // out_f32[b][m][n] = alpha_b^2 |D|^2
  EPI_GRADF = 3,     // out[b][m][n] = 2 alpha_b G[m][n] D    (c64 or split)
  EPI_PUPIL = 4,     // pupil-gradient planes from D = Ebar_unscaled[b][y=m][x=n]
  EPI_PSF_GRADF = 5, // both EPI_INTENSITY (out_f32) and EPI_GRADF (out_split / out_c64);
                     // with no cotangent (G null) the second output is F = alpha D
  EPI_SPLIT2 = 6,    // EPI_SPLIT / EPI_C64, plus the same values times colw[n] into out_*2
  EPI_DOT = 7,       // out_f32 = k_l alpha_l (Fb.im D.re - Fb.re D.im), Fb read from in_*
  EPI_PARTIAL = 8,   // split K: raw FP32 partial sums [split][b][m][n] (tensor-core form,
                     // internal: a reduction kernel then applies the GEMM's own epilogue)
};

struct EpiArgs {
  int kind;
  ObjTable objs;             // objects of a batched plan (objs.n == 0: single object below)
  const float* alpha;        // [wavelength] device
  float2* out_c64;
  __nv_bfloat16* out_split;
  float* out_f32;            // intensity planes, or pre planes for EPI_PUPIL
  float* out_f32b;           // pim planes for EPI_PUPIL
  const float* G;            // [m][n] for EPI_GRADF (null: store F = alpha D instead)
  // EPI_PUPIL recompute of the unit phasor
  const float* amp;          // nullable
  const float* amp_scale;    // nullable device scalar multiplying amp
  const float* opd;          // nullable
  const float* phase;        // nullable
  const float* weights;      // [b] nullable (1)
  const float2* inv_lambda_ff;  // [b] (hi, lo) of 1/lambda
  double pixel_scale, tilt_x, tilt_y;
  const float4* path;        // nullable [object][n][n] from PhasorArgs::out_path
  // many-source scenes
  const float* bweight;      // nullable [b]: extra factor of the EPI_GRADF cotangent
  const float* colw;         // [n] weights of EPI_SPLIT2's second output
  __nv_bfloat16* out_split2; // EPI_SPLIT2 second output (tensor-core form)
  float2* out_c642;          // EPI_SPLIT2 second output (FP32 form)
  const __nv_bfloat16* in_split;  // EPI_DOT: F-bar [b][4][m][n] (tensor-core form)
  const float2* in_c64;      // EPI_DOT: F-bar [b][m][n] (FP32 form)
  const float* kf;           // EPI_DOT: [wavelength] 2 pi / lambda
  float2* partial;           // EPI_PARTIAL: [split][b][m][n] FP32 partial sums
  const float2* coltilt;     // nullable [b][n]: phasor multiplying column n of the
                             // EPI_C64 / EPI_SPLIT / EPI_SPLIT2 outputs of batch element b
};

struct GemmArgs {
  int batch, M, N, K;
  const float2* A;          // c64 form
  long long a_bs;           // batch stride in elements (0: shared)
  const float2* B;
  long long b_bs;
  const __nv_bfloat16* As;  // split form [b][4][M][K]
  const __nv_bfloat16* Bs;  // split form [b][4][N][K]
  int a_batch_div;          // A batch index = b / a_batch_div (split form)
  int b_batch_div;          // B batch index = b / b_batch_div (0 or 1: B per batch element)
  bool conj_a;
  // Tensor-core form only: when a_axes is set, A is not read from memory but
  // generated in the CTA as the DFT matrix of a_axes[b / a_batch_div]; rows
  // are output indices (a_rows_are_out) or input indices.
  const DftAxis* a_axes;
  bool a_rows_are_out;
  EpiArgs epi;
  // Split K (tensor-core form, loaded operands): `splits` > 1 CTAs share each
  // output tile, each over a contiguous range of K, writing FP32 partials
  // into split_ws [splits][batch][M][N]; a reduction kernel sums them in split
  // order and applies `epi`. The caller fixes `splits` from the shape alone
  // (split_k_count), so a result does not depend on what else is in the batch.
  int splits;
  float2* split_ws;
  // Paired (cta_group::2) form of the loaded-operand tensor-core GEMM:
  // 0 follows the process-wide switch (dlx_set_gemm_pair), 1 never, 2 where
  // the shape allows it (an even number of 128-column tiles, no split K).
  int pair_mode;
};

// Splits for a GEMM with `tiles` output tiles (over the largest batch the
// caller will run) and inner size K: > 1 only when the tiles leave most SMs
// idle. 1 on devices without the tensor-core form.
int split_k_count(long long tiles, int K);
// Whether plans created now may split K (dlx_set_split_k).
bool split_k_enabled();
// Bytes of split_ws for that GEMM (0 when not split).
size_t split_k_bytes(int splits, long long batch, int M, int N);

int launch_gemm_fp32(const GemmArgs& g, cudaStream_t s);
// Either form by variant, bracketed by CUDA events while dlx_gemm_timing is on.
int run_gemm_timed(int variant, const GemmArgs& g, cudaStream_t s);
int launch_gemm_tc(const GemmArgs& g, cudaStream_t s);
bool tc_supported();

}  // namespace dlx
