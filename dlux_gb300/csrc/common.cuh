// common.cuh -- shared device helpers and host-side error plumbing.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string>

#include "../../include/dluxgb.h"

namespace dlx {

// ---------------------------------------------------------------------------
// Host-side error reporting (thread-local message, integer status).
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);

#define DLX_TRY_CUDA(expr)                                        \
  do {                                                            \
    cudaError_t _e = (expr);                                      \
    if (_e != cudaSuccess) return ::dlx::check_cuda(_e, #expr);   \
  } while (0)

#define DLX_TRY(expr)                 \
  do {                                \
    int _s = (expr);                  \
    if (_s != DLX_OK) return _s;      \
  } while (0)

// Counts every kernel launch of the library (dlx_launch_count).
void note_launch();

// Host-side state that depends on the device (kernel attributes, SM counts,
// status words) is kept once per device: a process may drive several
// devices, making each current in turn. Device indices are below kMaxDevices.
constexpr int kMaxDevices = 64;
// Writes the current device's index; DLX_ERR_CUDA / DLX_ERR_UNSUPPORTED otherwise.
int current_device(int* dev);
// Multiprocessor count of the current device (looked up once per device).
int device_sm_count(int* sms);

#define DLX_LAUNCH_CHECK(what)                                          \
  do {                                                                  \
    cudaError_t _e = cudaGetLastError();                                \
    if (_e != cudaSuccess) return ::dlx::check_cuda(_e, what);          \
    ::dlx::note_launch();                                               \
  } while (0)

// ---------------------------------------------------------------------------
// Programmatic dependent launch (PDL) for the kernels of the PSF + gradient
// step, which run as a chain of dependent launches. A kernel launched with
// launch_pdl may be scheduled before its predecessor in the stream has
// finished; it calls pdl_enter() before touching global memory, which waits
// for the predecessor to complete (its writes visible) and then lets the next
// kernel of the stream be launched early. Both instructions are no-ops for
// a kernel launched without the attribute.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t s, Args&&... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

#define DLX_PDL_LAUNCH(what, kernel, grid, block, smem, stream, ...)                      \
  do {                                                                                     \
    cudaError_t _e = ::dlx::launch_pdl(kernel, grid, block, smem, stream, __VA_ARGS__);    \
    if (_e != cudaSuccess) return ::dlx::check_cuda(_e, what);                             \
    ::dlx::note_launch();                                                                  \
  } while (0)

// ---------------------------------------------------------------------------
// DFT-type axis description. Element (i_in, j_out) of a generated matrix is
//   exp(2 pi i * [ sigma * x_i * u_j + g_in * i + d_in + g_out * j + d_out
//                  + q_in * x_i^2 + q_out * u_j^2 ])
// with x_i = a_in * i + b_in and u_j = a_out * j + b_out, all in FP64 cycles.
// This covers the MFT transfer matrices (no ramps), the padded centred FFT
// with its separable input/output phase ramps, and the linear canonical
// transform kernel of an ABCD system (the quadratic chirps q_in, q_out).
// `scale` multiplies the result.
// ---------------------------------------------------------------------------
struct DftAxis {
  double a_in, b_in, a_out, b_out;
  double g_in, d_in, g_out, d_out;
  double sigma;
  double scale;
  double q_in, q_out;
};

// Round-to-nearest FP64 cycle reduction followed by the FP32 sincospi of the
// reduced argument: returns (cos 2 pi t, sin 2 pi t).
__device__ __forceinline__ float2 cis_cycles(double t) {
  double r = t - rint(t);  // |r| <= 0.5, exact in FP64
  float s, c;
  sincospif(2.0f * (float)r, &s, &c);
  return make_float2(c, s);
}

// Per-(pixel, wavelength) phase in cycles, reduced with FP64 accuracy using
// FP32 instructions only (GB300's FP64 rate is ~1/64 of its FP32 rate, and
// this runs once per pixel per wavelength). The path length and the inverse
// wavelength arrive as unevaluated float pairs (hi + lo, |lo| <= ulp(hi)/2)
// formed once in FP64; Dekker's error-free product hi*hi = p + e (one FMA)
// gives the leading term exactly, p - rint(p) is exact for |p| < 2^22, and
// the remaining terms are below 2^-24 of |p|. The result has the absolute
// error of an FP64 reduction followed by rounding to FP32 (~3e-8 cycles).
struct FF {
  float hi, lo;
};

__host__ __device__ __forceinline__ FF ff_from_double(double v) {
  FF r;
  r.hi = (float)v;
  r.lo = (float)(v - (double)r.hi);
  return r;
}

// Float-pair arithmetic in FP32 alone (FP64 issues at a small fraction of
// the FP32 rate on this GPU): TwoSum (Knuth), Fast2Sum (Dekker, |a| >= |b|)
// and Dekker's product through one FMA. Results are normalised pairs within a
// few units of 2^-46 of the exact value, relative.
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bv = s - a;
  return FF{s, (a - (s - bv)) + (b - bv)};
}
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return FF{s, b - (s - a)};
}
// v * c for a float v and a float pair c
__device__ __forceinline__ FF ff_mul(float v, FF c) {
  const float p = v * c.hi;
  const float e = fmaf(v, c.hi, -p);
  return ff_fast_two_sum(p, fmaf(v, c.lo, e));
}
// a + b for float pairs
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
// 1 / (2 pi) as a float pair
__device__ __forceinline__ FF ff_inv_two_pi() { return FF{0x1.45f306p-3f, 0x1.b93910p-28f}; }

// Per-pixel inputs of cis_ff, formed once per pixel and object: the optical
// path opd + tx X + ty Y (m) with X = (x - c) dx, Y = (y - c) dx and
// c = (n - 1) / 2, from the float pairs t = (tx dx, ty dx); and the phase
// (radians) in cycles. xc = x - c and yc = y - c are exact in FP32. With no
// tilt the path is (opd, 0) exactly.
__device__ __forceinline__ FF pupil_path(float opd, float xc, float yc, float4 t) {
  FF path{opd, 0.f};
  if (t.x != 0.f || t.z != 0.f) {
    path = ff_add(path, ff_mul(xc, FF{t.x, t.y}));
    path = ff_add(path, ff_mul(yc, FF{t.z, t.w}));
  }
  return path;
}
__device__ __forceinline__ FF phase_cycles(float phase) { return ff_mul(phase, ff_inv_two_pi()); }
// (tx dx, ty dx) as float pairs; FP64 once per object
__host__ __device__ __forceinline__ float4 tilt_pairs(double tx, double ty, double dx) {
  const FF a = ff_from_double(tx * dx), b = ff_from_double(ty * dx);
  return make_float4(a.hi, a.lo, b.hi, b.lo);
}

__device__ __forceinline__ float2 cis_ff(FF path, FF inv_lambda, FF phase_cycles) {
  const float p = path.hi * inv_lambda.hi;
  const float e = fmaf(path.hi, inv_lambda.hi, -p);  // exact residual of the product
  const float small = e + fmaf(path.hi, inv_lambda.lo, path.lo * inv_lambda.hi);
  float r = (p - rintf(p)) + phase_cycles.hi;
  r = r + (small + phase_cycles.lo);
  r = r - rintf(r);
  float s, c;
  sincospif(2.0f * r, &s, &c);
  return make_float2(c, s);
}

// cis_ff for the split-BF16 form: the same exact reduction to r in [-1/2, 1/2]
// cycles, then the hardware sine/cosine of 2 pi r (absolute error below 1e-6
// on [-pi, pi]), which is below the ~7.6e-6 resolution of the hi/lo bf16
// operands that the result feeds. The FP32 form keeps cis_ff.
__device__ __forceinline__ float2 cis_ff_split(FF path, FF inv_lambda, FF phase_cycles) {
  const float p = path.hi * inv_lambda.hi;
  const float e = fmaf(path.hi, inv_lambda.hi, -p);
  const float small = e + fmaf(path.hi, inv_lambda.lo, path.lo * inv_lambda.hi);
  float r = (p - rintf(p)) + phase_cycles.hi;
  r = r + (small + phase_cycles.lo);
  r = r - rintf(r);
  float s, c;
  __sincosf(6.28318530717958647692f * r, &s, &c);
  return make_float2(c, s);
}

// |F|^2 of F = (fx, fy), with no FMA contraction: the same bits wherever it
// is formed (the GEMM epilogues from alpha D, and the wavelength sum over kept
// focal fields F = alpha D stored by a forward).
__device__ __forceinline__ float intensity_rn(float fx, float fy) {
  return __fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// hi/lo bf16 split of an FP32 value: hi = rn(x), lo = rn(x - hi).
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// split_bf16 of two values with one packed conversion (cvt.rn.bf16x2.f32)
// for both hi parts and one for both lo parts: the same bits as two
// split_bf16 calls, half the conversion instructions.
__device__ __forceinline__ void split_bf16x2(float x0, float x1, __nv_bfloat16& h0,
                                             __nv_bfloat16& h1, __nv_bfloat16& l0,
                                             __nv_bfloat16& l1) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
  h0 = h.x;
  h1 = h.y;
  l0 = l.x;
  l1 = l.y;
}

// Block sum of per-thread float pairs (hi, lo): the warps reduce in FP32
// float pairs (TwoSum at each shuffle level), and only the BLOCK / 32 warp
// totals are added in FP64, by warp 0. A fixed order, like block_sum, at a
// fraction of its FP64 work (FP64 issues at a small fraction of the FP32 rate
// on this GPU). Valid in thread 0.
template <int BLOCK>
__device__ __forceinline__ double block_sum_ff(float hi, float lo, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, hi, o);
    const float ol = __shfl_down_sync(0xffffffffu, lo, o);
    const float t = hi + oh;
    const float bv = t - hi;
    lo += ((hi - (t - bv)) + (oh - bv)) + ol;
    hi = t;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = (double)hi + (double)lo;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = (lane < BLOCK / 32) ? smem[lane] : 0.0;
#pragma unroll
    for (int o = (BLOCK / 32) / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Split operand layout: [batch][4][rows][split_ld(cols)] bf16, planes = re_hi,
// re_lo, im_hi, im_lo. TMA needs row pitches that are multiples of 16 bytes,
// so a row of `cols` elements is padded to a multiple of 8. The padding is
// never written and never read: the tensor maps declare `cols` as the extent
// along K and fill the columns past it with zeros. For sides that are
// multiples of 8 the layout is dense.
__host__ __device__ __forceinline__ int split_ld(int cols) { return (cols + 7) & ~7; }
__host__ __device__ __forceinline__ long long split_plane(int rows, int cols) {
  return (long long)rows * split_ld(cols);
}
// Bytes of `batch` split operands of rows x cols.
inline size_t split_bytes(long long batch, int rows, int cols) {
  return (size_t)batch * 4 * (size_t)split_plane(rows, cols) * 2;
}

}  // namespace dlx
