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
//   stats_*_kernel      per plane: sum |f|^2, max |f|^2 and its tie count, and
//   norm_*              for the reverse pass D = sum Re(conj(g) f). normalise
//                       (wavefronts.py:397-424) scales by s = sqrt(value / P) with
//                       P the power or the peak; its reverse pass is
//                       g_f = s g - f s D / P on every pixel (power) or on the
//                       pixels at the peak, shared among ties (peak), as JAX's
//                       max rule shares it.
//
// Every sum over pixels runs in a fixed order: per-thread float pairs (exact
// products by FMA, Knuth's TwoSum), per-block FP64 sums of those, and one warp
// per plane that adds the blocks' partials; every sum over wavelengths runs in
// a fixed order inside one thread in float pairs. FP64 issues at a small
// fraction of the FP32 rate on this GPU, so no per-element work is in FP64.
// Results do not depend on the launch.
#include <math_constants.h>

#include <cmath>
#include <string>

#include "kernels.h"

namespace dlx {
namespace {

constexpr int kBlock = 256;

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

// Float-pair running sum: TwoSum of each addend into (hi, lo).
struct FFSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = hi + x;
    const float bv = t - hi;
    lo += (hi - (t - bv)) + (x - bv);
    hi = t;
  }
  __device__ __forceinline__ void add(FF x) {
    add(x.hi);
    lo += x.lo;
  }
  // x * y with its exact rounding error (FMA)
  __device__ __forceinline__ void add_prod(float x, float y) {
    const float p = x * y;
    add(p);
    lo += fmaf(x, y, -p);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Pixel chunks of the per-plane sums: about 8192 pixels (32 per thread) each,
// at most kMaxParts per plane.
constexpr int kMaxParts = 64;
inline int plane_parts(long long npix) {
  const long long p = (npix + 8191) / 8192;
  return (int)(p < 1 ? 1 : (p > kMaxParts ? kMaxParts : p));
}

// One warp per plane b: the sum of parts[b * nparts + i] over i, lanes taking
// every 32nd partial, then a shuffle tree (a fixed order).
__device__ __forceinline__ double warp_sum_parts(const double* __restrict__ parts, int b,
                                                 int nparts, int stride, int field) {
  double t = 0.0;
  for (int i = threadIdx.x; i < nparts; i += 32)
    t += parts[((long long)b * nparts + i) * stride + field];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  return t;  // lane 0
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

__global__ void phasor_bwd_kernel(PhasorBwdArgs a, BatchFF il, BatchFF kf) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  // The forward's float pairs (dlx_phasor with no tilt): path in metres, phase in cycles.
  const FF path{a.opd ? a.opd[p] : 0.f, 0.f};
  const FF ph_cyc = a.phase ? phase_cycles(a.phase[p]) : FF{0.f, 0.f};
  const float amp = a.amp ? a.amp[p] : 1.0f;
  FFSum s_amp, s_ph, s_opd;
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
    s_amp.add(fu.x * g.x + fu.y * g.y);                   // Re(conj(f u) g)
    const float im = out.x * g.y - out.y * g.x;           // Im(conj(out) g)
    s_ph.add(im);
    s_opd.add(ff_mul(im, FF{kf.v[b].x, kf.v[b].y}));      // k_b im
  }
  if (a.accumulate) {
    if (a.g_amp) s_amp.add(a.g_amp[p]);
    if (a.g_phase) s_ph.add(a.g_phase[p]);
    if (a.g_opd) s_opd.add(a.g_opd[p]);
  }
  if (a.g_amp) a.g_amp[p] = (float)s_amp.value();
  if (a.g_phase) a.g_phase[p] = (float)s_ph.value();
  if (a.g_opd) a.g_opd[p] = (float)s_opd.value();
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

// g_w[b] = sum_p g[p] |f_b[p]|^2: grid (parts, planes), one FP64 partial per
// block, then one warp per plane.
__global__ void psf_wsum_bwd_weight_partial_kernel(const float2* __restrict__ in,
                                                   long long npix, int nparts,
                                                   const float* __restrict__ g,
                                                   double* __restrict__ parts) {
  __shared__ double smem[32];
  const int b = blockIdx.y;
  const float2* f = in + (long long)b * npix;
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  FFSum acc;
  for (long long p = lo + threadIdx.x; p < hi; p += blockDim.x) {
    const float2 v = __ldg(f + p);
    const float gp = __ldg(g + p);
    acc.add_prod(gp, __fmul_rn(v.x, v.x));
    acc.add_prod(gp, __fmul_rn(v.y, v.y));
    // the squares' own rounding errors, weighted
    acc.lo += gp * (fmaf(v.x, v.x, -__fmul_rn(v.x, v.x)) + fmaf(v.y, v.y, -__fmul_rn(v.y, v.y)));
  }
  const double t = block_sum_ff<kBlock>(acc.hi, acc.lo, smem);
  if (threadIdx.x == 0) parts[(long long)b * nparts + blockIdx.x] = t;
}

__global__ void psf_wsum_bwd_weight_finish_kernel(const double* __restrict__ parts, int nparts,
                                                  float* __restrict__ g_w) {
  const double t = warp_sum_parts(parts, blockIdx.x, nparts, 1, 0);
  if (threadIdx.x == 0) g_w[blockIdx.x] = (float)t;
}

// Per plane: sum |f|^2, max |f|^2, pixels at the max, and sum Re(conj(g) f)
// (the last only when g is given: the reverse pass).
struct PlaneStats {
  double power, peak, ties, dot;
};

// Grid (parts, planes): per block the partial power and dot (FP64 sums of
// float-pair thread sums) and the partial max, as [plane][part][3] doubles.
__global__ void stats_partial_kernel(const float2* __restrict__ in, long long npix, int nparts,
                                     const float2* __restrict__ g, double* __restrict__ parts) {
  __shared__ double dsm[32];
  __shared__ float fsm[32];
  const int b = blockIdx.y;
  const float2* f = in + (long long)b * npix;
  const float2* gb = g ? g + (long long)b * npix : nullptr;
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  FFSum pw, dd;
  float mx = 0.f;
  for (long long p = lo + threadIdx.x; p < hi; p += blockDim.x) {
    const float2 v = __ldg(f + p);
    pw.add_prod(v.x, v.x);
    pw.add_prod(v.y, v.y);
    mx = fmaxf(mx, abs2_rn(v));
    if (gb) {
      const float2 q = __ldg(gb + p);
      dd.add_prod(q.x, v.x);
      dd.add_prod(q.y, v.y);
    }
  }
  const double tp = block_sum_ff<kBlock>(pw.hi, pw.lo, dsm);
  const double td = block_sum_ff<kBlock>(dd.hi, dd.lo, dsm);
  const float tm = block_max_f<kBlock>(mx, fsm);
  if (threadIdx.x == 0) {
    double* o = parts + ((long long)b * nparts + blockIdx.x) * 3;
    o[0] = tp;
    o[1] = td;
    o[2] = (double)tm;
  }
}

// One warp per plane: power, dot and peak from the partials; ties zeroed
// (counted next, when the peak is needed).
__global__ void stats_finish_kernel(const double* __restrict__ parts, int nparts,
                                    PlaneStats* __restrict__ stats) {
  const int b = blockIdx.x;
  const double pw = warp_sum_parts(parts, b, nparts, 3, 0);
  const double dd = warp_sum_parts(parts, b, nparts, 3, 1);
  float mx = 0.f;
  for (int i = threadIdx.x; i < nparts; i += 32)
    mx = fmaxf(mx, (float)parts[((long long)b * nparts + i) * 3 + 2]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if (threadIdx.x == 0) stats[b] = PlaneStats{pw, (double)mx, 0.0, dd};
}

// Pixels at the peak, per block, then added per plane (integer counts: any
// order gives the same sum).
__global__ void stats_ties_kernel(const float2* __restrict__ in, long long npix, int nparts,
                                  PlaneStats* __restrict__ stats,
                                  unsigned long long* __restrict__ ties) {
  __shared__ unsigned int cnt;
  const int b = blockIdx.y;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const float2* f = in + (long long)b * npix;
  const float mx = (float)stats[b].peak;
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  unsigned int c = 0;
  for (long long p = lo + threadIdx.x; p < hi; p += blockDim.x)
    c += abs2_rn(__ldg(f + p)) == mx ? 1u : 0u;
  atomicAdd(&cnt, c);
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(ties + b, (unsigned long long)cnt);
}

__global__ void stats_ties_finish_kernel(const unsigned long long* __restrict__ ties,
                                         PlaneStats* __restrict__ stats, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) stats[b].ties = (double)ties[b];
}

// mode 0: power, 1: peak.
__device__ __forceinline__ double norm_base(const PlaneStats& st, int mode) {
  return mode == 0 ? st.power : st.peak;
}

// Grid (pixel blocks, planes): the scale s = sqrt(value / P) once per block.
__global__ void norm_fwd_kernel(const float2* __restrict__ in, long long npix, int mode,
                                double value, const PlaneStats* __restrict__ stats,
                                float2* __restrict__ out, float* __restrict__ scale_out) {
  __shared__ float sh;
  const int b = blockIdx.y;
  if (threadIdx.x == 0) sh = (float)sqrt(value / norm_base(stats[b], mode));
  __syncthreads();
  const float s = sh;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const long long i = (long long)b * npix + p;
  const float2 v = in[i];
  out[i] = make_float2(v.x * s, v.y * s);
  if (scale_out && p == 0) scale_out[b] = s;
}

// g_f = s g - c f with c = s D / P (power: every pixel; peak: the pixels at
// the peak, D / P shared among the ties), in float pairs; s and c are formed
// once per block in FP64.
__global__ void norm_bwd_kernel(const float2* __restrict__ in, long long npix, int mode,
                                double value, const PlaneStats* __restrict__ stats,
                                const float2* __restrict__ g, float2* __restrict__ g_in) {
  __shared__ float4 sc;  // (s, c) as float pairs
  __shared__ float peak;
  const int b = blockIdx.y;
  if (threadIdx.x == 0) {
    const PlaneStats st = stats[b];
    const double P = norm_base(st, mode);
    const double s = sqrt(value / P);
    const double c = mode == 0 ? s * st.dot / P : s * st.dot / (P * st.ties);
    const FF sf = ff_from_double(s), cf = ff_from_double(c);
    sc = make_float4(sf.hi, sf.lo, cf.hi, cf.lo);
    peak = (float)st.peak;
  }
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const long long i = (long long)b * npix + p;
  const float2 v = in[i];
  const float2 q = g[i];
  const FF s{sc.x, sc.y};
  const bool at = mode == 0 || abs2_rn(v) == peak;
  const FF c = at ? FF{sc.z, sc.w} : FF{0.f, 0.f};
  const FF x = ff_add(ff_mul(q.x, s), ff_mul(-v.x, c));
  const FF y = ff_add(ff_mul(q.y, s), ff_mul(-v.y, c));
  g_in[i] = make_float2(x.hi, y.hi);
}

// Stats of `batch` planes into stats (device), with the tie counts when
// `ties_needed`. ws: [batch][plane_parts][3] doubles then [batch] counters.
int plane_stats(const float2* f, const float2* g, int batch, long long npix, bool ties_needed,
                PlaneStats* stats, double* ws, cudaStream_t s) {
  const int np = plane_parts(npix);
  stats_partial_kernel<<<dim3(np, batch), kBlock, 0, s>>>(f, npix, np, g, ws);
  DLX_LAUNCH_CHECK("stats_partial_kernel");
  stats_finish_kernel<<<batch, 32, 0, s>>>(ws, np, stats);
  DLX_LAUNCH_CHECK("stats_finish_kernel");
  if (ties_needed) {
    auto* ties = reinterpret_cast<unsigned long long*>(ws + (size_t)batch * np * 3);
    DLX_TRY_CUDA(cudaMemsetAsync(ties, 0, sizeof(unsigned long long) * batch, s));
    stats_ties_kernel<<<dim3(np, batch), kBlock, 0, s>>>(f, npix, np, stats, ties);
    DLX_LAUNCH_CHECK("stats_ties_kernel");
    stats_ties_finish_kernel<<<ceil_div(batch, 256), 256, 0, s>>>(ties, stats, batch);
    DLX_LAUNCH_CHECK("stats_ties_finish_kernel");
  }
  return DLX_OK;
}

size_t plane_stats_ws_bytes(int batch, long long npix) {
  return sizeof(double) * (size_t)batch * plane_parts(npix) * 3 +
         sizeof(unsigned long long) * (size_t)batch;
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
    BatchFF il, kf;
    for (int i = 0; i < kMaxBatchArg; ++i) {
      il.v[i] = make_float2(0.f, 0.f);
      kf.v[i] = make_float2(0.f, 0.f);
    }
    for (int i = 0; i < nb; ++i) {
      const double w = wavelengths_host[b0 + i];
      const FF f = ff_from_double(1.0 / w);
      il.v[i] = make_float2(f.hi, f.lo);
      const FF k = ff_from_double(2.0 * CUDART_PI / w);
      kf.v[i] = make_float2(k.hi, k.lo);
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
    phasor_bwd_kernel<<<ceil_div(npix, kBlock), kBlock, 0, s>>>(a, il, kf);
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
    const int np = plane_parts(npix);
    double* parts = nullptr;
    DLX_TRY_CUDA(cudaMallocAsync((void**)&parts, sizeof(double) * (size_t)batch * np, s));
    psf_wsum_bwd_weight_partial_kernel<<<dim3(np, batch), kBlock, 0, s>>>(f, npix, np, g, parts);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
      note_launch();
      psf_wsum_bwd_weight_finish_kernel<<<batch, 32, 0, s>>>(parts, np, g_weights);
      e = cudaGetLastError();
      if (e == cudaSuccess) note_launch();
    }
    cudaFreeAsync(parts, s);
    if (e != cudaSuccess) return check_cuda(e, "psf_sum_weighted_backward");
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
  double* ws = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&stats, sizeof(PlaneStats) * batch, s));
  const cudaError_t ea = cudaMallocAsync((void**)&ws, plane_stats_ws_bytes(batch, npix), s);
  if (ea != cudaSuccess) {
    cudaFreeAsync(stats, s);
    return check_cuda(ea, "normalise");
  }
  const float2* f = reinterpret_cast<const float2*>(in);
  int st = plane_stats(f, nullptr, batch, npix, false, stats, ws, s);
  if (st == DLX_OK) {
    norm_fwd_kernel<<<dim3(ceil_div(npix, kBlock), batch), kBlock, 0, s>>>(
        f, npix, mode, value, stats, reinterpret_cast<float2*>(out), scale_out);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launch();
    else st = check_cuda(e, "normalise");
  }
  cudaFreeAsync(ws, s);
  cudaFreeAsync(stats, s);
  return st;
}

int dlx_normalise_backward(const void* in, int batch, long long npix, int mode, double value,
                           const void* g, void* g_in, void* stream) {
  DLX_TRY(check_stats_args(batch, npix, "normalise_backward"));
  if (mode != 0 && mode != 1) return fail(DLX_ERR_ARG, "mode must be 'power' or 'peak'");
  if (batch == 0 || npix == 0) return DLX_OK;
  if (!in || !g || !g_in) return fail(DLX_ERR_ARG, "normalise_backward: null pointer");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  PlaneStats* stats = nullptr;
  double* ws = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&stats, sizeof(PlaneStats) * batch, s));
  const cudaError_t ea = cudaMallocAsync((void**)&ws, plane_stats_ws_bytes(batch, npix), s);
  if (ea != cudaSuccess) {
    cudaFreeAsync(stats, s);
    return check_cuda(ea, "normalise_backward");
  }
  const float2* f = reinterpret_cast<const float2*>(in);
  const float2* gg = reinterpret_cast<const float2*>(g);
  int st = plane_stats(f, gg, batch, npix, mode == 1, stats, ws, s);
  if (st == DLX_OK) {
    norm_bwd_kernel<<<dim3(ceil_div(npix, kBlock), batch), kBlock, 0, s>>>(
        f, npix, mode, value, stats, gg, reinterpret_cast<float2*>(g_in));
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launch();
    else st = check_cuda(e, "normalise_backward");
  }
  cudaFreeAsync(ws, s);
  cudaFreeAsync(stats, s);
  return st;
}

}  // extern "C"
