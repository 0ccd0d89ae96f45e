// layers.cu -- kernels of the layer-by-layer path: the reverse pass of the
// phasor multiply, the weighted sum of focal intensities and its reverse
// pass, and Wavefront.normalise with its reverse pass.
//
// The fused system path (capi.cu dlx_poly_*) covers systems whose layers fold
// into one pupil. Any other layer list runs layer by layer: each optical layer
// multiplies the field by amp * exp(i (k opd + phase)) (dlx_phasor forward),
// the propagators run the MFT/FFT plans, and the PSF is the weighted sum of
// the focal intensities. These kernels give that path its hand-written
// reverse passes:
//
//   phasor_bwd_kernel   out_b = f_b A u_b, u_b = exp(i (2 pi opd / l_b + phase))
//                       g_f_b = g_b conj(A u_b);  g_A = sum_b Re(conj(f_b u_b) g_b);
//                       g_phase = sum_b Im(conj(out_b) g_b);  g_opd = sum_b k_b (same)
//                       (JAX's reverse mode of wavefronts.py:332-368 and of the
//                       real multiply of wavefronts.py:834-906). u_b is rebuilt
//                       with the forward's own error-free reduction (cis_ff, the
//                       same float pairs), so forward and reverse phasors are
//                       bit-identical.
//   psf_wsum_kernel     psf = sum_b w_b |f_b|^2 (optical_systems.py:211-223: the
//                       field times sqrt(w) in the vmap body, then the sum of
//                       |E|^2); reverse g_f_b = 2 w_b g f_b and
//                       g_w_b = sum_p g |f_b|^2.
//   plane_stats_kernel  per plane: sum |f|^2, max |f|^2 and its tie count, and
//   norm_*              for the reverse pass D = sum Re(conj(g) f). normalise
//                       (wavefronts.py:397-424) scales by s = sqrt(value / P) with
//                       P the power or the peak; its reverse pass is
//                       g_f = s g - f s D / P on every pixel (power) or on the
//                       pixels at the peak, shared among ties (peak), as JAX's
//                       max rule shares it.
//
// Every sum over pixels is a fixed-order block reduction in FP64, and every
// sum over wavelengths runs in a fixed order inside one thread, so results do
// not depend on the launch.
#include <math_constants.h>

#include <cmath>
#include <string>

#include "kernels.h"

namespace dlx {
namespace {

constexpr int kBlock = 256;
constexpr int kStatBlock = 1024;

// |v|^2 rounded the same way at every call site (no FMA contraction), so that
// the peak test below sees exactly the values the maximum was taken over.
__device__ __forceinline__ float abs2_rn(float2 v) {
  return __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
}

template <int BLOCK>
__device__ __forceinline__ double block_sum_d(double v, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = (lane < BLOCK / 32) ? smem[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) smem[0] = t;
  }
  __syncthreads();
  t = smem[0];
  __syncthreads();
  return t;  // every thread
}

template <int BLOCK>
__device__ __forceinline__ float block_max_f(float v, float* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  float t = 0.f;
  if (warp == 0) {
    t = (lane < BLOCK / 32) ? smem[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_down_sync(0xffffffffu, t, o));
    if (lane == 0) smem[0] = t;
  }
  __syncthreads();
  t = smem[0];
  __syncthreads();
  return t;
}

struct PhasorBwdArgs {
  const float2* in;   // nullable [b][p]: the multiplied field (1 when absent)
  const float* amp;   // nullable [p]
  const float* opd;   // nullable [p]
  const float* phase; // nullable [p]
  const float2* g;    // [b][p]
  float2* g_in;       // nullable [b][p]
  float* g_amp;       // nullable [p]
  float* g_opd;       // nullable [p]
  float* g_phase;     // nullable [p]
  int batch;          // planes of this launch (at most kMaxBatchArg)
  long long npix;
  int accumulate;     // add the sums into g_amp / g_opd / g_phase (later chunks)
};

__global__ void phasor_bwd_kernel(PhasorBwdArgs a, BatchFF il, BatchD kb) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  // The forward's float pairs (dlx_phasor with no tilt): path in metres, phase in cycles.
  const FF path = ff_from_double(a.opd ? (double)a.opd[p] : 0.0);
  const FF ph_cyc = ff_from_double(a.phase ? (double)a.phase[p] * (0.5 / CUDART_PI) : 0.0);
  const float amp = a.amp ? a.amp[p] : 1.0f;
  double s_amp = 0.0, s_ph = 0.0, s_opd = 0.0;
  for (int b = 0; b < a.batch; ++b) {
    const float2 u = cis_ff(path, FF{il.v[b].x, il.v[b].y}, ph_cyc);
    const long long o = (long long)b * a.npix + p;
    const float2 g = a.g[o];
    const float2 f = a.in ? a.in[o] : make_float2(1.f, 0.f);
    const float2 fu = cmul(f, u);                         // f u
    const float2 out = make_float2(fu.x * amp, fu.y * amp);
    if (a.g_in) {
      const float2 fac = make_float2(u.x * amp, u.y * amp);
      a.g_in[o] = make_float2(g.x * fac.x + g.y * fac.y, g.y * fac.x - g.x * fac.y);  // g conj(fac)
    }
    s_amp += (double)(fu.x * g.x + fu.y * g.y);            // Re(conj(f u) g)
    const double im = (double)(out.x * g.y - out.y * g.x);  // Im(conj(out) g)
    s_ph += im;
    s_opd += kb.v[b] * im;
  }
  if (a.accumulate) {
    if (a.g_amp) a.g_amp[p] = (float)(s_amp + (double)a.g_amp[p]);
    if (a.g_phase) a.g_phase[p] = (float)(s_ph + (double)a.g_phase[p]);
    if (a.g_opd) a.g_opd[p] = (float)(s_opd + (double)a.g_opd[p]);
  } else {
    if (a.g_amp) a.g_amp[p] = (float)s_amp;
    if (a.g_phase) a.g_phase[p] = (float)s_ph;
    if (a.g_opd) a.g_opd[p] = (float)s_opd;
  }
}

__global__ void psf_wsum_kernel(const float2* __restrict__ in, const float* __restrict__ w,
                                int batch, long long npix, float* __restrict__ psf) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  float acc = 0.f;
  for (int b = 0; b < batch; ++b) {
    const float2 v = in[(long long)b * npix + p];
    const float i2 = v.x * v.x + v.y * v.y;
    acc += w ? w[b] * i2 : i2;
  }
  psf[p] = acc;
}

__global__ void psf_wsum_bwd_field_kernel(const float2* __restrict__ in,
                                          const float* __restrict__ w, int batch,
                                          long long npix, const float* __restrict__ g,
                                          float2* __restrict__ g_in) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)batch * npix) return;
  const int b = (int)(i / npix);
  const long long p = i - (long long)b * npix;
  const float s = 2.0f * g[p] * (w ? w[b] : 1.0f);
  const float2 v = in[i];
  g_in[i] = make_float2(s * v.x, s * v.y);
}

// g_w[b] = sum_p g[p] |f_b[p]|^2, one block per plane.
__global__ void psf_wsum_bwd_weight_kernel(const float2* __restrict__ in, long long npix,
                                           const float* __restrict__ g,
                                           float* __restrict__ g_w) {
  __shared__ double smem[32];
  const int b = blockIdx.x;
  const float2* f = in + (long long)b * npix;
  double acc = 0.0;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    const float2 v = f[p];
    acc += (double)g[p] * ((double)v.x * v.x + (double)v.y * v.y);
  }
  const double t = block_sum_d<kStatBlock>(acc, smem);
  if (threadIdx.x == 0) g_w[b] = (float)t;
}

// Per plane: sum |f|^2, max |f|^2, pixels at the max, and sum Re(conj(g) f)
// (the last only when g is given: the reverse pass).
struct PlaneStats {
  double power, peak, ties, dot;
};

__global__ void plane_stats_kernel(const float2* __restrict__ in, long long npix,
                                   const float2* __restrict__ g, PlaneStats* __restrict__ stats) {
  __shared__ double dsm[32];
  __shared__ float fsm[32];
  const int b = blockIdx.x;
  const float2* f = in + (long long)b * npix;
  const float2* gb = g ? g + (long long)b * npix : nullptr;
  double pw = 0.0, dd = 0.0;
  float mx = 0.f;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    const float2 v = f[p];
    pw += (double)v.x * v.x + (double)v.y * v.y;
    mx = fmaxf(mx, abs2_rn(v));
    if (gb) {
      const float2 q = gb[p];
      dd += (double)q.x * v.x + (double)q.y * v.y;
    }
  }
  pw = block_sum_d<kStatBlock>(pw, dsm);
  dd = block_sum_d<kStatBlock>(dd, dsm);
  mx = block_max_f<kStatBlock>(mx, fsm);
  double ties = 0.0;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x)
    ties += abs2_rn(f[p]) == mx ? 1.0 : 0.0;
  ties = block_sum_d<kStatBlock>(ties, dsm);
  if (threadIdx.x == 0) stats[b] = PlaneStats{pw, (double)mx, ties, dd};
}

// mode 0: power, 1: peak.
__device__ __forceinline__ double norm_base(const PlaneStats& st, int mode) {
  return mode == 0 ? st.power : st.peak;
}

__global__ void norm_fwd_kernel(const float2* __restrict__ in, int batch, long long npix,
                                int mode, double value, const PlaneStats* __restrict__ stats,
                                float2* __restrict__ out, float* __restrict__ scale_out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)batch * npix) return;
  const int b = (int)(i / npix);
  const float s = (float)sqrt(value / norm_base(stats[b], mode));
  const float2 v = in[i];
  out[i] = make_float2(v.x * s, v.y * s);
  if (scale_out && i == (long long)b * npix) scale_out[b] = s;
}

__global__ void norm_bwd_kernel(const float2* __restrict__ in, int batch, long long npix,
                                int mode, double value, const PlaneStats* __restrict__ stats,
                                const float2* __restrict__ g, float2* __restrict__ g_in) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)batch * npix) return;
  const int b = (int)(i / npix);
  const PlaneStats st = stats[b];
  const double P = norm_base(st, mode);
  const double s = sqrt(value / P);
  const float2 v = in[i];
  const float2 q = g[i];
  double c = 0.0;  // coefficient of f: s D / P, over the pixels the scale depends on
  if (mode == 0)
    c = s * st.dot / P;
  else if (abs2_rn(v) == (float)st.peak)
    c = s * st.dot / (P * st.ties);
  g_in[i] = make_float2((float)(s * q.x - c * v.x), (float)(s * q.y - c * v.y));
}

int check_stats_args(int batch, long long npix, const char* who) {
  if (batch < 0 || npix < 0) return fail(DLX_ERR_SHAPE, std::string(who) + ": negative size");
  return DLX_OK;
}

}  // namespace
}  // namespace dlx

using namespace dlx;

extern "C" {

int dlx_phasor_backward(const void* in, const float* amp, const float* opd, const float* phase,
                        const double* wavelengths_host, int batch, int n, const void* g,
                        void* g_in, float* g_amp, float* g_opd, float* g_phase, void* stream) {
  if (batch < 0 || n < 0) return fail(DLX_ERR_SHAPE, "phasor_backward: negative size");
  const long long npix = (long long)n * n;
  if (npix == 0) return DLX_OK;
  if (!wavelengths_host || (batch > 0 && !g))
    return fail(DLX_ERR_ARG, "phasor_backward: null pointer");
  for (int b = 0; b < batch; ++b)
    if (!(wavelengths_host[b] > 0))
      return fail(DLX_ERR_ARG, "phasor_backward: wavelengths must be positive");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (batch == 0) {
    // no planes: the sums over the batch are zero
    for (float* o : {g_amp, g_opd, g_phase})
      if (o) DLX_TRY_CUDA(cudaMemsetAsync(o, 0, sizeof(float) * npix, s));
    return DLX_OK;
  }
  // Chunks of kMaxBatchArg planes in order; later chunks add into the sums.
  for (int b0 = 0; b0 < batch; b0 += kMaxBatchArg) {
    const int nb = (batch - b0) < kMaxBatchArg ? (batch - b0) : kMaxBatchArg;
    BatchFF il;
    BatchD kb;
    for (int i = 0; i < kMaxBatchArg; ++i) {
      il.v[i] = make_float2(0.f, 0.f);
      kb.v[i] = 0.0;
    }
    for (int i = 0; i < nb; ++i) {
      const double w = wavelengths_host[b0 + i];
      const FF f = ff_from_double(1.0 / w);
      il.v[i] = make_float2(f.hi, f.lo);
      kb.v[i] = 2.0 * CUDART_PI / w;
    }
    const long long off = (long long)b0 * npix;
    PhasorBwdArgs a{};
    a.in = in ? reinterpret_cast<const float2*>(in) + off : nullptr;
    a.amp = amp; a.opd = opd; a.phase = phase;
    a.g = reinterpret_cast<const float2*>(g) + off;
    a.g_in = g_in ? reinterpret_cast<float2*>(g_in) + off : nullptr;
    a.g_amp = g_amp; a.g_opd = g_opd; a.g_phase = g_phase;
    a.batch = nb;
    a.npix = npix;
    a.accumulate = b0 > 0 ? 1 : 0;
    phasor_bwd_kernel<<<ceil_div(npix, kBlock), kBlock, 0, s>>>(a, il, kb);
    DLX_LAUNCH_CHECK("phasor_bwd_kernel");
  }
  return DLX_OK;
}

int dlx_psf_sum_weighted(const void* in, const float* weights, int batch, long long npix,
                         float* psf, void* stream) {
  DLX_TRY(check_stats_args(batch, npix, "psf_sum_weighted"));
  if (npix == 0) return DLX_OK;
  if (!psf || (batch > 0 && !in)) return fail(DLX_ERR_ARG, "psf_sum_weighted: null pointer");
  psf_wsum_kernel<<<ceil_div(npix, kBlock), kBlock, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(in), weights, batch, npix, psf);
  DLX_LAUNCH_CHECK("psf_wsum_kernel");
  return DLX_OK;
}

int dlx_psf_sum_weighted_backward(const void* in, const float* weights, int batch,
                                  long long npix, const float* g, void* g_in, float* g_weights,
                                  void* stream) {
  DLX_TRY(check_stats_args(batch, npix, "psf_sum_weighted_backward"));
  if (batch == 0) return DLX_OK;
  if (!in || !g) return fail(DLX_ERR_ARG, "psf_sum_weighted_backward: null pointer");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* f = reinterpret_cast<const float2*>(in);
  if (g_in && npix > 0) {
    psf_wsum_bwd_field_kernel<<<ceil_div((long long)batch * npix, kBlock), kBlock, 0, s>>>(
        f, weights, batch, npix, g, reinterpret_cast<float2*>(g_in));
    DLX_LAUNCH_CHECK("psf_wsum_bwd_field_kernel");
  }
  if (g_weights) {
    psf_wsum_bwd_weight_kernel<<<batch, kStatBlock, 0, s>>>(f, npix, g, g_weights);
    DLX_LAUNCH_CHECK("psf_wsum_bwd_weight_kernel");
  }
  return DLX_OK;
}

int dlx_normalise(const void* in, int batch, long long npix, int mode, double value, void* out,
                  float* scale_out, void* stream) {
  DLX_TRY(check_stats_args(batch, npix, "normalise"));
  if (mode != 0 && mode != 1) return fail(DLX_ERR_ARG, "mode must be 'power' or 'peak'");
  if (batch == 0 || npix == 0) return DLX_OK;
  if (!in || !out) return fail(DLX_ERR_ARG, "normalise: null pointer");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  PlaneStats* stats = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&stats, sizeof(PlaneStats) * batch, s));
  const float2* f = reinterpret_cast<const float2*>(in);
  plane_stats_kernel<<<batch, kStatBlock, 0, s>>>(f, npix, nullptr, stats);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    note_launch();
    norm_fwd_kernel<<<ceil_div((long long)batch * npix, kBlock), kBlock, 0, s>>>(
        f, batch, npix, mode, value, stats, reinterpret_cast<float2*>(out), scale_out);
    e = cudaGetLastError();
    if (e == cudaSuccess) note_launch();
  }
  cudaFreeAsync(stats, s);
  if (e != cudaSuccess) return check_cuda(e, "normalise");
  return DLX_OK;
}

int dlx_normalise_backward(const void* in, int batch, long long npix, int mode, double value,
                           const void* g, void* g_in, void* stream) {
  DLX_TRY(check_stats_args(batch, npix, "normalise_backward"));
  if (mode != 0 && mode != 1) return fail(DLX_ERR_ARG, "mode must be 'power' or 'peak'");
  if (batch == 0 || npix == 0) return DLX_OK;
  if (!in || !g || !g_in) return fail(DLX_ERR_ARG, "normalise_backward: null pointer");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  PlaneStats* stats = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&stats, sizeof(PlaneStats) * batch, s));
  const float2* f = reinterpret_cast<const float2*>(in);
  const float2* gg = reinterpret_cast<const float2*>(g);
  plane_stats_kernel<<<batch, kStatBlock, 0, s>>>(f, npix, gg, stats);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    note_launch();
    norm_bwd_kernel<<<ceil_div((long long)batch * npix, kBlock), kBlock, 0, s>>>(
        f, batch, npix, mode, value, stats, gg, reinterpret_cast<float2*>(g_in));
    e = cudaGetLastError();
    if (e == cudaSuccess) note_launch();
  }
  cudaFreeAsync(stats, s);
  if (e != cudaSuccess) return check_cuda(e, "normalise_backward");
  return DLX_OK;
}

}  // extern "C"
