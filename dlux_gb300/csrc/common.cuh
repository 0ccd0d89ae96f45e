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

#define DLX_LAUNCH_CHECK(what)                                          \
  do {                                                                  \
    cudaError_t _e = cudaGetLastError();                                \
    if (_e != cudaSuccess) return ::dlx::check_cuda(_e, what);          \
    ::dlx::note_launch();                                               \
  } while (0)

// ---------------------------------------------------------------------------
// Affine-phase DFT description. Element (i_in, j_out) of a generated matrix is
//   exp(2 pi i * [ sigma * x_i * u_j + g_in * i + d_in + g_out * j + d_out ])
// with x_i = a_in * i + b_in and u_j = a_out * j + b_out, all in FP64 cycles.
// This covers the MFT transfer matrices (no ramps) and the padded centred FFT
// with its separable input/output phase ramps. `scale` multiplies the result.
// ---------------------------------------------------------------------------
struct DftAxis {
  double a_in, b_in, a_out, b_out;
  double g_in, d_in, g_out, d_out;
  double sigma;
  double scale;
};

// Round-to-nearest FP64 cycle reduction followed by the FP32 sincospi of the
// reduced argument: returns (cos 2 pi t, sin 2 pi t).
__device__ __forceinline__ float2 cis_cycles(double t) {
  double r = t - rint(t);  // |r| <= 0.5, exact in FP64
  float s, c;
  sincospif(2.0f * (float)r, &s, &c);
  return make_float2(c, s);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// hi/lo bf16 split of an FP32 value: hi = rn(x), lo = rn(x - hi).
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Split operand layout: [batch][4][rows][cols] bf16, planes = re_hi, re_lo, im_hi, im_lo.
struct SplitView {
  __nv_bfloat16* p;
  int rows, cols;
  __host__ __device__ long long plane() const { return (long long)rows * cols; }
  __host__ __device__ long long batch_stride() const { return 4LL * rows * cols; }
};

}  // namespace dlx
