// elementwise.cu -- DFT-matrix generation, phasor build, reductions, basis
// contraction and detector kernels. All of these are HBM- or latency-bound;
// each is written for coalesced access with one pixel per thread and a
// wavelength loop inside the thread where the inputs are shared across the
// batch.
#include <algorithm>
#include <atomic>

#include "kernels.h"

#include <math_constants.h>

namespace dlx {

// ---------------------------------------------------------------------------
// DFT / transfer-matrix generation (dLux utils/propagation.py:67-127 for the
// MFT, utils/propagation.py:8-64 + utils/fourier.py:48-78 for the FFT).
// ---------------------------------------------------------------------------
__global__ void dft_gen_kernel(const DftAxis* __restrict__ axes, int rows, int cols,
                               bool rows_are_out, float2* __restrict__ out_c64,
                               long long out_bs, __nv_bfloat16* __restrict__ out_split) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y * blockDim.y + threadIdx.y;
  const int b = blockIdx.z;
  if (r >= rows || c >= cols) return;
  const DftAxis ax = axes[b];
  const int i_in = rows_are_out ? c : r;
  const int j_out = rows_are_out ? r : c;
  const double x = ax.a_in * (double)i_in + ax.b_in;
  const double u = ax.a_out * (double)j_out + ax.b_out;
  const double t = ax.sigma * x * u + (ax.g_in * (double)i_in + ax.d_in) +
                   (ax.g_out * (double)j_out + ax.d_out) + ax.q_in * x * x + ax.q_out * u * u;
  float2 v = cis_cycles(t);
  v.x *= (float)ax.scale;
  v.y *= (float)ax.scale;
  const long long idx = (long long)r * cols + c;
  if (out_c64) out_c64[(long long)b * out_bs + idx] = v;
  if (out_split) {
    const long long plane = split_plane(rows, cols);
    __nv_bfloat16* base = out_split + (long long)b * 4 * plane + (long long)r * split_ld(cols) + c;
    __nv_bfloat16 h, l;
    split_bf16(v.x, h, l);
    base[0] = h;
    base[plane] = l;
    split_bf16(v.y, h, l);
    base[2 * plane] = h;
    base[3 * plane] = l;
  }
}

int launch_dft_gen(const DftAxis* axes_dev, int batch, int rows, int cols, bool rows_are_out,
                   float2* out_c64, long long out_batch_stride, __nv_bfloat16* out_split,
                   cudaStream_t s) {
  if (batch <= 0 || rows <= 0 || cols <= 0) return DLX_OK;
  dim3 block(32, 8);
  dim3 grid(ceil_div(cols, 32), ceil_div(rows, 8), batch);
  dft_gen_kernel<<<grid, block, 0, s>>>(axes_dev, rows, cols, rows_are_out, out_c64,
                                        out_batch_stride, out_split);
  DLX_LAUNCH_CHECK("dft_gen_kernel");
  return DLX_OK;
}

// ---------------------------------------------------------------------------
// Phasor build (wavefronts.py:70-122, :332-395; optical_layers.py:181-186,
// 319-327; optics.py:77-96; optical_systems.py:213-215).
// One thread per pixel; the wavelength loop reuses amp/opd/phase.
// ---------------------------------------------------------------------------
// kSplit: the output is the split-BF16 operand only (cis_ff_split).
template <bool kSplit>
__global__ void phasor_kernel(PhasorArgs a, BatchFF inv_lambda_arg, int cached) {
  // cached: per-wavelength 1/lambda pairs and per-(object, wavelength)
  // sqrt(weight) staged once per block in shared memory
  extern __shared__ float psm[];
  __shared__ float4 s_tilt[kMaxObj];
  const long long npix = (long long)a.n * a.n;
  const int R = a.objs.n > 0 ? a.objs.n : 1;
  const int L = a.batch / R;
  float2* c_il = reinterpret_cast<float2*>(psm);
  float* c_sw = psm + 2 * L;
  if (cached) {
    for (int i = threadIdx.x; i < L; i += blockDim.x)
      c_il[i] = a.inv_lambda_ff ? a.inv_lambda_ff[i] : inv_lambda_arg.v[i];
    for (int i = threadIdx.x; i < R * L; i += blockDim.x) {
      const int r = i / L, wl = i - (i / L) * L;
      const float* o_w = a.objs.n > 0 ? a.objs.o[r].weights : a.weights;
      c_sw[i] = o_w ? sqrtf(o_w[wl]) : 1.0f;
    }
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x)
    s_tilt[r] = a.objs.n > 0 ? tilt_pairs(a.objs.o[r].tilt_x, a.objs.o[r].tilt_y, a.pixel_scale)
                             : tilt_pairs(a.tilt_x, a.tilt_y, a.pixel_scale);
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int y = (int)(p / a.n);
  const int x = (int)(p - (long long)y * a.n);
  const float half = 0.5f * (float)(a.n - 1);
  const float xc = (float)x - half, yc = (float)y - half;
  const float cs = (float)a.const_scale;
  // Objects r of a batched plan (b = l * R + r), or one object described by
  // the plain fields of PhasorArgs.
  for (int r = 0; r < R; ++r) {
    const bool obj = a.objs.n > 0;
    const float* o_amp = obj ? a.objs.o[r].amp : a.amp;
    const float* o_scale = obj ? a.objs.o[r].amp_scale : a.amp_scale;
    const float* o_opd = obj ? a.objs.o[r].opd : a.opd;
    const float* o_phase = obj ? a.objs.o[r].phase : a.phase;
    const float* o_w = obj ? a.objs.o[r].weights : a.weights;
    // Per pixel and object, once: optical path (m) and phase (cycles) as float pairs.
    const FF path = pupil_path(o_opd ? o_opd[p] : 0.f, xc, yc, s_tilt[r]);
    const FF ph_cyc = o_phase ? phase_cycles(o_phase[p]) : FF{0.f, 0.f};
    if (a.out_path) a.out_path[(long long)r * npix + p] = make_float4(path.hi, path.lo, ph_cyc.hi, ph_cyc.lo);
    float amp = o_amp ? o_amp[p] : 1.0f;
    if (o_scale) amp *= *o_scale;
    amp *= cs;
    for (int wl = 0; wl < L; ++wl) {
      const int b = wl * R + r;
      const float2 il2 = cached ? c_il[wl]
                                : (a.inv_lambda_ff ? a.inv_lambda_ff[wl] : inv_lambda_arg.v[wl]);
      float2 u = kSplit ? cis_ff_split(path, FF{il2.x, il2.y}, ph_cyc)
                        : cis_ff(path, FF{il2.x, il2.y}, ph_cyc);
      float sc = amp;
      if (cached) sc *= c_sw[r * L + wl];
      else if (o_w) sc *= sqrtf(o_w[wl]);
      float2 v = make_float2(u.x * sc, u.y * sc);
      const long long o = (long long)b * npix + p;
      if (a.in) v = cmul(a.in[o], v);
      if (a.out_c64) a.out_c64[o] = v;
      if (a.out_split) {
        // padded rows (split_ld)
        const long long splane = split_plane(a.n, a.n);
        __nv_bfloat16* base =
            a.out_split + (long long)b * 4 * splane + (long long)y * split_ld(a.n) + x;
        __nv_bfloat16 h, lo;
        split_bf16(v.x, h, lo);
        base[0] = h;
        base[splane] = lo;
        split_bf16(v.y, h, lo);
        base[2 * splane] = h;
        base[3 * splane] = lo;
      }
    }
  }
}

template <int V>
struct alignas(2 * V) Bf16Vec {
  __nv_bfloat16 v[V];
};

// Split-BF16 output only, V adjacent pixels of one row per thread (n % V ==
// 0, so that with rows padded to split_ld(n) every store is aligned): each of
// the four planes gets one 2V-byte store per thread and
// wavelength, and the per-pixel FP64 path set-up is amortised over a
// wavelength group (blockIdx.y: wavelengths [y * lg, (y + 1) * lg)). Same
// arithmetic per pixel as phasor_kernel.
template <int V>
__global__ void phasor_splitv_kernel(PhasorArgs a, BatchFF inv_lambda_arg, int cached, int lg) {
  pdl_enter();
  extern __shared__ float psm[];
  __shared__ float4 s_tilt[kMaxObj];
  const long long npix = (long long)a.n * a.n;
  const int R = a.objs.n > 0 ? a.objs.n : 1;
  const int L = a.batch / R;
  float2* c_il = reinterpret_cast<float2*>(psm);
  float* c_sw = psm + 2 * L;
  if (cached) {
    for (int i = threadIdx.x; i < L; i += blockDim.x)
      c_il[i] = a.inv_lambda_ff ? a.inv_lambda_ff[i] : inv_lambda_arg.v[i];
    for (int i = threadIdx.x; i < R * L; i += blockDim.x) {
      const int r = i / L, wl = i - (i / L) * L;
      const float* o_w = a.objs.n > 0 ? a.objs.o[r].weights : a.weights;
      c_sw[i] = o_w ? sqrtf(o_w[wl]) : 1.0f;
    }
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x)
    s_tilt[r] = a.objs.n > 0 ? tilt_pairs(a.objs.o[r].tilt_x, a.objs.o[r].tilt_y, a.pixel_scale)
                             : tilt_pairs(a.tilt_x, a.tilt_y, a.pixel_scale);
  __syncthreads();
  const long long p0 = V * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (p0 >= npix) return;
  const int y = (int)(p0 / a.n);
  const int x0 = (int)(p0 - (long long)y * a.n);
  const float half = 0.5f * (float)(a.n - 1);
  const float yc = (float)y - half;
  const float cs = (float)a.const_scale;
  for (int r = 0; r < R; ++r) {
    const bool obj = a.objs.n > 0;
    const float* o_amp = obj ? a.objs.o[r].amp : a.amp;
    const float* o_scale = obj ? a.objs.o[r].amp_scale : a.amp_scale;
    const float* o_opd = obj ? a.objs.o[r].opd : a.opd;
    const float* o_phase = obj ? a.objs.o[r].phase : a.phase;
    const float* o_w = obj ? a.objs.o[r].weights : a.weights;
    const float scale = (o_scale ? *o_scale : 1.0f);
    const float4 t = s_tilt[r];
    FF path[V], ph[V];
    float amp[V];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const long long p = p0 + k;
      path[k] = pupil_path(o_opd ? o_opd[p] : 0.f, (float)(x0 + k) - half, yc, t);
      ph[k] = o_phase ? phase_cycles(o_phase[p]) : FF{0.f, 0.f};
      if (a.out_path && blockIdx.y == 0)
        a.out_path[(long long)r * npix + p] =
            make_float4(path[k].hi, path[k].lo, ph[k].hi, ph[k].lo);
      float am = o_amp ? o_amp[p] : 1.0f;
      if (o_scale) am *= scale;
      amp[k] = am * cs;
    }
    const int wl1 = min(L, (int)(blockIdx.y + 1) * lg);
    // (unrolling this loop by 2 or 4 measured 31.5 / 31.7 against 30.9 us)
    for (int wl = blockIdx.y * lg; wl < wl1; ++wl) {
      const int b = wl * R + r;
      const float2 il2 = cached ? c_il[wl]
                                : (a.inv_lambda_ff ? a.inv_lambda_ff[wl] : inv_lambda_arg.v[wl]);
      float sw = 1.0f;
      if (cached) sw = c_sw[r * L + wl];
      else if (o_w) sw = sqrtf(o_w[wl]);
      Bf16Vec<V> q[4];
      float re[V], im[V];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const float2 u = cis_ff_split(path[k], FF{il2.x, il2.y}, ph[k]);
        const float sc = amp[k] * sw;
        re[k] = u.x * sc;
        im[k] = u.y * sc;
      }
      // adjacent pixels' splits share packed conversions
      static_assert(V % 2 == 0, "pixels are split in pairs");
#pragma unroll
      for (int k = 0; k < V; k += 2) {
        split_bf16x2(re[k], re[k + 1], q[0].v[k], q[0].v[k + 1], q[1].v[k], q[1].v[k + 1]);
        split_bf16x2(im[k], im[k + 1], q[2].v[k], q[2].v[k + 1], q[3].v[k], q[3].v[k + 1]);
      }
      const long long splane = split_plane(a.n, a.n);
      __nv_bfloat16* base =
          a.out_split + (long long)b * 4 * splane + (long long)y * split_ld(a.n) + x0;
#pragma unroll
      for (int c = 0; c < 4; ++c) *reinterpret_cast<Bf16Vec<V>*>(base + c * splane) = q[c];
    }
  }
}

int launch_phasor(const PhasorArgs& a, const BatchFF* inv_lambda_arg, cudaStream_t s) {
  const long long npix = (long long)a.n * a.n;
  if (npix == 0 || a.batch == 0) return DLX_OK;
  BatchFF dummy;
  if (!inv_lambda_arg) {
    for (int i = 0; i < kMaxBatchArg; ++i) dummy.v[i] = make_float2(0.f, 0.f);
    inv_lambda_arg = &dummy;
  }
  const int R = a.objs.n > 0 ? a.objs.n : 1;
  const int L = a.batch / R;
  // stage the per-wavelength factors in shared memory when they fit in 32 KB
  const size_t smem = sizeof(float) * (size_t)(2 * L + R * L);
  const int cached = smem <= 32 * 1024 ? 1 : 0;
  // Four pixels per thread pays with many wavelengths; with a few, one pixel
  // per thread gives four times the threads and a quarter of the per-thread
  // FP64 set-up.
  if (a.out_split && !a.out_c64 && !a.in && a.n % 4 == 0 && L >= 8) {
    // One wavelength group: spreading the wavelengths over more blocks
    // measured slower at 512^2 x 64 (42.9 vs 38.3 us) with the FP64 path
    // set-up repeated per group, and no faster (35.9 us plus 12.9 us for a
    // separate FP64 pass over the pixels) with the set-up done once: the
    // per-element phase reduction and sincos bound the kernel.
    // 4 pixels per thread (2 measured the same at 512^2 x 64, 8 slower: 42.0
    // vs 37.0 us)
    // With the path set-up in FP32 float pairs, 2, 4, 8, 16 and 32 wavelength
    // groups measured 30.5, 30.3, 30.5, 35.7 and 47.7 us against 30.7 us for
    // one.
    constexpr int V = 4;
    constexpr int kPhasorGroups = 1;
    const int lg = (L + kPhasorGroups - 1) / kPhasorGroups;
    const int gy = (L + lg - 1) / lg;
    constexpr int kPhasorBlock = 256;  // 64 and 128 measured 30.5 and 30.1 against 29.0 us
    DLX_PDL_LAUNCH("phasor_splitv_kernel", phasor_splitv_kernel<V>,
                   dim3(ceil_div(npix / V, kPhasorBlock), gy), dim3(kPhasorBlock),
                   cached ? smem : 0, s, a, *inv_lambda_arg, cached, lg);
    return DLX_OK;
  } else if (a.out_split && !a.out_c64 && !a.in)
    phasor_kernel<true><<<ceil_div(npix, 256), 256, cached ? smem : 0, s>>>(a, *inv_lambda_arg,
                                                                             cached);
  else
    phasor_kernel<false><<<ceil_div(npix, 256), 256, cached ? smem : 0, s>>>(a, *inv_lambda_arg,
                                                                              cached);
  DLX_LAUNCH_CHECK("phasor_kernel");
  return DLX_OK;
}

// c64 [b][rows][cols] -> split [b][4][rows][split_ld(cols)], one element
// per thread over a plane, the batch looped inside the thread.
__global__ void c64_to_split_kernel(const float2* __restrict__ in, int rows, int cols, int batch,
                                    __nv_bfloat16* __restrict__ out) {
  const long long plane = (long long)rows * cols;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const long long splane = split_plane(rows, cols);
  const int r = (int)(p / cols);
  const long long sp = (long long)r * split_ld(cols) + (p - (long long)r * cols);
  for (int b = 0; b < batch; ++b) {
    __nv_bfloat16* base = out + (long long)b * 4 * splane;
    float2 v = in[(long long)b * plane + p];
    __nv_bfloat16 h, l;
    split_bf16(v.x, h, l);
    base[sp] = h;
    base[splane + sp] = l;
    split_bf16(v.y, h, l);
    base[2 * splane + sp] = h;
    base[3 * splane + sp] = l;
  }
}

int launch_c64_to_split_batched(const float2* in, int rows, int cols, int batch,
                                __nv_bfloat16* out_split, cudaStream_t s) {
  const long long plane = (long long)rows * cols;
  if (plane == 0 || batch == 0) return DLX_OK;
  c64_to_split_kernel<<<ceil_div(plane, 256), 256, 0, s>>>(in, rows, cols, batch, out_split);
  DLX_LAUNCH_CHECK("c64_to_split_kernel");
  return DLX_OK;
}

// F-bar of the poly reverse pass from the focal fields a forward kept (the
// cotangent of sum G |F|^2 is 2 G F): V adjacent pixels of one row per thread
// (M % V == 0, so that with rows padded to split_ld(M) each split plane gets
// one 2V-byte store), the objects looped inside and their wavelengths
// [blockIdx.y lg, (blockIdx.y + 1) lg) as well, so each G value is read once
// per wavelength group. Wavelength groups give the pass enough threads to
// keep HBM busy (measured at 64 x 512^2: 62 us in one group, 47 us in 8).
// out_c64 may be f itself (every element is read and written by the same
// thread).
template <int V>
__global__ void focal_gradf_kernel(const float2* f, ObjTable objs, int batch, int M, int lg,
                                   __nv_bfloat16* __restrict__ out_split, float2* out_c64) {
  pdl_enter();
  const long long npix = (long long)M * M;
  const long long p0 = V * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (p0 >= npix) return;
  const int R = objs.n > 0 ? objs.n : 1;
  const int y = (int)(p0 / M);
  const long long splane = split_plane(M, M);
  const long long sp = (long long)y * split_ld(M) + (p0 - (long long)y * M);
  const int l0 = blockIdx.y * lg;
  const int l1 = min(batch / R, l0 + lg);
  for (int r = 0; r < R; ++r) {
    float g[V];
#pragma unroll
    for (int k = 0; k < V; ++k) g[k] = 2.0f * objs.o[r].G[p0 + k];
    for (int l = l0; l < l1; ++l) {
      const long long b = (long long)l * R + r;
      float2 o[V];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const float2 v = f[b * npix + p0 + k];
        o[k] = make_float2(g[k] * v.x, g[k] * v.y);
      }
      if (out_split) {
        Bf16Vec<V> q[4];
        if constexpr (V % 2 == 0) {
#pragma unroll
          for (int k = 0; k < V; k += 2) {
            split_bf16x2(o[k].x, o[k + 1].x, q[0].v[k], q[0].v[k + 1], q[1].v[k], q[1].v[k + 1]);
            split_bf16x2(o[k].y, o[k + 1].y, q[2].v[k], q[2].v[k + 1], q[3].v[k], q[3].v[k + 1]);
          }
        } else {
#pragma unroll
          for (int k = 0; k < V; ++k) {
            split_bf16(o[k].x, q[0].v[k], q[1].v[k]);
            split_bf16(o[k].y, q[2].v[k], q[3].v[k]);
          }
        }
        __nv_bfloat16* base = out_split + b * 4 * splane + sp;
#pragma unroll
        for (int c = 0; c < 4; ++c) *reinterpret_cast<Bf16Vec<V>*>(base + c * splane) = q[c];
      } else {
#pragma unroll
        for (int k = 0; k < V; ++k) out_c64[b * npix + p0 + k] = o[k];
      }
    }
  }
}

int launch_focal_gradf(const float2* f, const ObjTable& objs, int batch, int M,
                       __nv_bfloat16* out_split, float2* out_c64, cudaStream_t s) {
  const long long npix = (long long)M * M;
  if (npix == 0 || batch == 0) return DLX_OK;
  for (int r = 0; r < (objs.n > 0 ? objs.n : 1); ++r)
    if (!objs.o[r].G) return fail(DLX_ERR_ARG, "focal_gradf: every object needs g_psf");
  // up to 8 wavelength groups
  const int L = batch / (objs.n > 0 ? objs.n : 1);
  const int lg = (L + 7) / 8;
  const int groups = (L + lg - 1) / lg;
  if (M % 4 == 0)
    DLX_PDL_LAUNCH("focal_gradf_kernel", focal_gradf_kernel<4>,
                   dim3(ceil_div(npix / 4, 256), groups), dim3(256), 0, s, f, objs, batch, M, lg,
                   out_split, out_c64);
  else
    DLX_PDL_LAUNCH("focal_gradf_kernel", focal_gradf_kernel<1>,
                   dim3(ceil_div(npix, 256), groups), dim3(256), 0, s, f, objs, batch, M, lg,
                   out_split, out_c64);
  return DLX_OK;
}

// ---------------------------------------------------------------------------
// Block-level double reduction helper (fixed order -> deterministic).
// ---------------------------------------------------------------------------
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double* smem) {
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
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// psf[p] = sum_b |in[b][p]|^2 (wavefronts.py:279 summed as optical_systems.py:223)
__global__ void psf_sum_kernel(const float2* __restrict__ in, int batch, long long npix,
                               float* __restrict__ psf) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  float acc = 0.f;
  for (int b = 0; b < batch; ++b) {
    float2 v = in[(long long)b * npix + p];
    acc += v.x * v.x + v.y * v.y;
  }
  psf[p] = acc;
}

int launch_psf_sum(const float2* in, int batch, long long npix, float* psf, cudaStream_t s) {
  if (npix == 0) return DLX_OK;
  psf_sum_kernel<<<ceil_div(npix, 256), 256, 0, s>>>(in, batch, npix, psf);
  DLX_LAUNCH_CHECK("psf_sum_kernel");
  return DLX_OK;
}

// out[b] = sqrt(value / sum_p |in[b][p]|^2): one block per batch element.
__global__ void power_scale_kernel(const float2* __restrict__ in, long long npix, double value,
                                   float* __restrict__ out) {
  __shared__ double smem[32];
  const int b = blockIdx.x;
  const float2* src = in + (long long)b * npix;
  double acc = 0.0;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    float2 v = src[p];
    acc += (double)v.x * v.x + (double)v.y * v.y;
  }
  double t = block_sum<1024>(acc, smem);
  if (threadIdx.x == 0) out[b] = (float)sqrt(value / t);
}

int launch_power_scale(const float2* in, int batch, long long npix, double value, float* out,
                       cudaStream_t s) {
  if (batch == 0) return DLX_OK;
  power_scale_kernel<<<batch, 1024, 0, s>>>(in, npix, value, out);
  DLX_LAUNCH_CHECK("power_scale_kernel");
  return DLX_OK;
}

// Two-level deterministic sum of amp^2 (partials then one block).
__global__ void sumsq_partial_kernel(const float* __restrict__ x, long long npix, int nparts,
                                     double* __restrict__ partial) {
  pdl_enter();
  __shared__ double smem[32];
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  // exact squares (FMA) summed in float pairs, eight loads in flight before
  // the adds, which keep the element order
  float h = 0.f, l = 0.f;
  auto add = [&](float v) {
    const float pr = v * v;
    const float t = h + pr;
    const float bv = t - h;
    l += ((h - (t - bv)) + (pr - bv)) + fmaf(v, v, -pr);
    h = t;
  };
  const long long step = blockDim.x;
  long long p = lo + threadIdx.x;
  for (; p + 7 * step < hi; p += 8 * step) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldg(x + p + u * step);
#pragma unroll
    for (int u = 0; u < 8; ++u) add(v[u]);
  }
  for (; p < hi; p += step) add(__ldg(x + p));
  const double t = block_sum_ff<256>(h, l, smem);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void norm_finish_kernel(const double* __restrict__ partial, int nparts, double value,
                                   float* __restrict__ out_scale) {
  pdl_enter();
  __shared__ double smem[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partial[i];
  double t = block_sum<256>(acc, smem);
  if (threadIdx.x == 0) out_scale[0] = (float)sqrt(value / t);
}

int launch_amp_norm(const float* amp, long long npix, double value, float* out_scale,
                    double* partial_ws, int nparts, cudaStream_t s) {
  DLX_PDL_LAUNCH("sumsq_partial_kernel", sumsq_partial_kernel, dim3(nparts), dim3(256), 0, s,
                 amp, npix, nparts, partial_ws);
  DLX_PDL_LAUNCH("norm_finish_kernel", norm_finish_kernel, dim3(1), dim3(256), 0, s,
                 partial_ws, nparts, value, out_scale);
  return DLX_OK;
}

// Reverse of a_eff = a * n, n = sqrt(value / S), S = sum a^2:
// g_a[j] = n g_eff[j] - a_j n^3 / value * sum_i a_i g_eff[i].
// Three launches: per-chunk partials of S and D = sum a g (float-pair sums,
// as in the coefficient gradient), one warp that reduces them in a fixed
// order and forms n and c = n^3 D / value once in FP64, and the per-pixel
// n g - a c in FP32 float pairs. (Every block forming n and c for itself in
// FP64 made the last kernel 20 us at 512^2: FP64 division and square root run
// at a small fraction of the FP32 rate on this GPU.)
__global__ void dot_sumsq_partial_kernel(const float* __restrict__ a, const float* __restrict__ g,
                                         long long npix, int nparts,
                                         double* __restrict__ partial) {
  pdl_enter();
  __shared__ double smem[32];
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  // exact products (FMA) summed in float pairs (Knuth's TwoSum), widened once
  float s2h = 0.f, s2l = 0.f, sgh = 0.f, sgl = 0.f;
  auto add = [](float x, float y, float& h, float& l) {
    const float pr = x * y;
    const float pe = fmaf(x, y, -pr);
    const float t = h + pr;
    const float bv = t - h;
    l += ((h - (t - bv)) + (pr - bv)) + pe;
    h = t;
  };
  const long long step = blockDim.x;
  long long p = lo + threadIdx.x;
  for (; p + 7 * step < hi; p += 8 * step) {
    float av[8], gv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      av[u] = __ldg(a + p + u * step);
      gv[u] = __ldg(g + p + u * step);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      add(av[u], av[u], s2h, s2l);
      add(av[u], gv[u], sgh, sgl);
    }
  }
  for (; p < hi; p += step) {
    const float av = __ldg(a + p), gv = __ldg(g + p);
    add(av, av, s2h, s2l);
    add(av, gv, sgh, sgl);
  }
  const double t2 = block_sum_ff<256>(s2h, s2l, smem);
  const double tg = block_sum_ff<256>(sgh, sgl, smem);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = t2;
    partial[2 * blockIdx.x + 1] = tg;
  }
}

// One warp: lanes take every 32nd partial, then a shuffle tree (fixed order).
// nc = (n, c) as float pairs.
__global__ void amp_norm_bwd_finish_kernel(const double* __restrict__ partial, int nparts,
                                           double value, float4* __restrict__ nc) {
  pdl_enter();
  double s2 = 0.0, sg = 0.0;
  for (int i = threadIdx.x; i < nparts; i += 32) {
    s2 += partial[2 * i];
    sg += partial[2 * i + 1];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    sg += __shfl_down_sync(0xffffffffu, sg, o);
  }
  if (threadIdx.x == 0) {
    const double n = sqrt(value / s2);
    const double c = n * n * n / value * sg;
    const FF nf = ff_from_double(n), cf = ff_from_double(c);
    *nc = make_float4(nf.hi, nf.lo, cf.hi, cf.lo);
  }
}

__global__ void amp_norm_bwd_kernel(const float* __restrict__ a, const float* __restrict__ g,
                                    long long npix, const float4* __restrict__ nc,
                                    float* __restrict__ g_a) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const float4 q = *nc;
  const FF t1 = ff_mul(__ldg(g + p), FF{q.x, q.y});
  const FF t2 = ff_mul(__ldg(a + p), FF{q.z, q.w});
  const FF d = ff_add(t1, FF{-t2.hi, -t2.lo});
  g_a[p] = d.hi;
}

int launch_amp_norm_backward(const float* amp, const float* g_eff, long long npix, double value,
                             float* g_amp, double* partial_ws, int nparts, cudaStream_t s) {
  // partial_ws: 2 * nparts doubles of partials, then (n, c) as float pairs
  float4* nc = reinterpret_cast<float4*>(partial_ws + 2 * (size_t)nparts);
  DLX_PDL_LAUNCH("dot_sumsq_partial_kernel", dot_sumsq_partial_kernel, dim3(nparts), dim3(256),
                 0, s, amp, g_eff, npix, nparts, partial_ws);
  DLX_PDL_LAUNCH("amp_norm_bwd_finish_kernel", amp_norm_bwd_finish_kernel, dim3(1), dim3(32), 0,
                 s, partial_ws, nparts, value, nc);
  DLX_PDL_LAUNCH("amp_norm_bwd_kernel", amp_norm_bwd_kernel, dim3(ceil_div(npix, 256)),
                 dim3(256), 0, s, amp, g_eff, npix, nc, g_amp);
  return DLX_OK;
}

// ---------------------------------------------------------------------------
// Basis contraction (utils/math.py:177-196) and its reverse.
// ---------------------------------------------------------------------------
// acc + sum_{u < C} c[k + u] B[k + u][p] in term order, the C loads issued first
template <int C>
__device__ __forceinline__ float basis_terms(const float* __restrict__ basis, const float* sc,
                                             int k, long long npix, long long p, float acc) {
  float v[C];
#pragma unroll
  for (int u = 0; u < C; ++u) v[u] = __ldg(basis + (long long)(k + u) * npix + p);
#pragma unroll
  for (int u = 0; u < C; ++u) acc = fmaf(sc[k + u], v[u], acc);
  return acc;
}

// basis_terms<rem> for a run-time rem in [0, C]
template <int C>
__device__ __forceinline__ float basis_tail(const float* __restrict__ basis, const float* sc,
                                            int k, int rem, long long npix, long long p,
                                            float acc) {
  if constexpr (C == 0) {
    return acc;
  } else {
    if (rem == C) return basis_terms<C>(basis, sc, k, npix, p, acc);
    return basis_tail<C - 1>(basis, sc, k, rem, npix, p, acc);
  }
}

__global__ void basis_eval_kernel(const float* __restrict__ basis,
                                  const float* __restrict__ coeffs,
                                  const float* __restrict__ base, int nterms, long long npix,
                                  float* __restrict__ out) {
  pdl_enter();
  extern __shared__ float sc[];
  for (int k = threadIdx.x; k < nterms; k += blockDim.x) sc[k] = coeffs[k];
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  float acc = base ? base[p] : 0.f;
  // kEvalBatch terms' loads issued before their FMAs (which keep the term
  // order), so that the loads' latencies overlap; the remainder is one batch
  // too: 8.8 us at 512^2 x 21 terms (8.6 with 16, 9.0 with 4; a serial
  // remainder 9.4; sixteen with the last group masked 24.8).
  constexpr int kEvalBatch = 8;
  int k = 0;
  for (; k + kEvalBatch <= nterms; k += kEvalBatch)
    acc = basis_terms<kEvalBatch>(basis, sc, k, npix, p, acc);
  // the last nterms % kEvalBatch terms as one batch as well
  acc = basis_tail<kEvalBatch - 1>(basis, sc, k, nterms - k, npix, p, acc);
  out[p] = acc;
}

int launch_basis_eval(const float* basis, const float* coeffs, const float* base, int nterms,
                      long long npix, float* out, cudaStream_t s) {
  if (npix == 0) return DLX_OK;
  DLX_PDL_LAUNCH("basis_eval_kernel", basis_eval_kernel, dim3(ceil_div(npix, 256)), dim3(256),
                 sizeof(float) * (nterms > 0 ? nterms : 1), s, basis, coeffs, base, nterms, npix,
                 out);
  return DLX_OK;
}

__global__ void basis_grad_partial_kernel(const float* __restrict__ basis,
                                          const float* __restrict__ g, long long npix,
                                          int nparts, double* __restrict__ partial) {
  pdl_enter();
  __shared__ double smem[32];
  const int k = blockIdx.y;
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  const float* row = basis + (long long)k * npix;
  // Error-free FP32 accumulation (FP64 arithmetic is slow on this GPU): each
  // product is split exactly into p + e (fmaf), the running sum is kept as a
  // float pair with Knuth's TwoSum, and only the per-thread pair is widened.
  float hi_s = 0.f, lo_s = 0.f;
  auto add = [&](float x, float y) {
    const float pr = x * y;
    const float pe = fmaf(x, y, -pr);
    const float t = hi_s + pr;
    const float bv = t - hi_s;
    const float err = (hi_s - (t - bv)) + (pr - bv);
    hi_s = t;
    lo_s += err + pe;
  };
  const long long step = blockDim.x;
  long long p = lo + threadIdx.x;
  // kGradBatch pixels' loads in flight before the (ordered) float-pair sums
  // (12.3-12.5 us at 512^2 x 21 terms with 8, 13.8 with 16 or 32)
  constexpr int kGradBatch = 8;
  for (; p + (kGradBatch - 1) * step < hi; p += kGradBatch * step) {
    float xv[kGradBatch], yv[kGradBatch];
#pragma unroll
    for (int u = 0; u < kGradBatch; ++u) {
      xv[u] = __ldg(row + p + u * step);
      yv[u] = __ldg(g + p + u * step);
    }
#pragma unroll
    for (int u = 0; u < kGradBatch; ++u) add(xv[u], yv[u]);
  }
  for (; p < hi; p += step) add(__ldg(row + p), __ldg(g + p));
  const double t = block_sum_ff<256>(hi_s, lo_s, smem);
  if (threadIdx.x == 0) partial[(long long)k * nparts + blockIdx.x] = t;
}

__global__ void basis_grad_finish_kernel(const double* __restrict__ partial, int nparts,
                                         float* __restrict__ g_coeffs) {
  pdl_enter();
  __shared__ double smem[32];
  const int k = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partial[(long long)k * nparts + i];
  double t = block_sum<256>(acc, smem);
  if (threadIdx.x == 0) g_coeffs[k] = (float)t;
}

// Pixel chunks of the coefficient-gradient partials: nterms x nparts blocks of
// 256 threads, kBlocksPerSM per SM when there are enough pixels, with chunks
// of at least 2048 pixels (8 per thread). At 512^2 x 21 terms: 11.2 us with
// 4 per SM, 11.7 with 3, 12.9 with 2, 13.0 with 8 and 15.9 with 16 (12.3 with
// the earlier fixed 64 chunks).
int basis_grad_parts(int nterms, long long npix, int sms) {
  constexpr int kBlocksPerSM = 4;
  const long long wave = (long long)kBlocksPerSM * sms / std::max(1, nterms);
  const long long by_pixels = (npix + 2047) / 2048;
  return (int)std::max(1LL, std::min(wave, by_pixels));
}

int launch_basis_grad(const float* basis, const float* g, int nterms, long long npix,
                      float* g_coeffs, double* partial_ws, int nparts, cudaStream_t s) {
  if (nterms == 0) return DLX_OK;
  dim3 grid(nparts, nterms);
  DLX_PDL_LAUNCH("basis_grad_partial_kernel", basis_grad_partial_kernel, grid, dim3(256), 0, s,
                 basis, g, npix, nparts, partial_ws);
  DLX_PDL_LAUNCH("basis_grad_finish_kernel", basis_grad_finish_kernel, dim3(nterms), dim3(256), 0,
                 s, partial_ws, nparts, g_coeffs);
  return DLX_OK;
}

// ---------------------------------------------------------------------------
// Detector: k x k block sum (utils/array_ops.py:124-162) x pixel response
// (layers/detector_layers.py:100-131), and the reverse.
// ---------------------------------------------------------------------------
// KC > 0: the block side known at compile time, so that all KC * KC loads of
// a thread are issued before its adds; KC = 0 reads k at run time. The sums
// run row by row in the same order either way.
template <int KC>
__global__ void downsample_kernel(const float* __restrict__ in, int n_in, int k, int mean,
                                  const float* __restrict__ flat, float* __restrict__ out) {
  pdl_enter();
  if (KC > 0) k = KC;
  const int n_out = n_in / k;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= n_out || c >= n_out) return;
  float acc = 0.f;
  if (KC > 0) {
    constexpr int K = KC > 0 ? KC : 1;
    float v[K][K];
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
      for (int j = 0; j < K; ++j) v[i][j] = __ldg(in + (long long)(a * K + i) * n_in + c * K + j);
#pragma unroll
    for (int i = 0; i < K; ++i) {
      float r = 0.f;
#pragma unroll
      for (int j = 0; j < K; ++j) r += v[i][j];
      acc += r;
    }
  } else {
    for (int i = 0; i < k; ++i) {
      const float* row = in + (long long)(a * k + i) * n_in + (long long)c * k;
      float r = 0.f;
      for (int j = 0; j < k; ++j) r += row[j];
      acc += r;
    }
  }
  if (mean) acc /= (float)(k * k);
  if (flat) acc *= flat[(long long)a * n_out + c];
  out[(long long)a * n_out + c] = acc;
}

int launch_downsample(const float* in, int n_in, int k, int mean, const float* flat, float* out,
                      cudaStream_t s) {
  const int n_out = n_in / k;
  if (n_out == 0) return DLX_OK;
  dim3 block(32, 8);
  dim3 grid(ceil_div(n_out, 32), ceil_div(n_out, 8));
  switch (k) {
    case 2:
      DLX_PDL_LAUNCH("downsample_kernel", downsample_kernel<2>, grid, block, 0, s, in, n_in, k,
                     mean, flat, out);
      break;
    case 3:
      DLX_PDL_LAUNCH("downsample_kernel", downsample_kernel<3>, grid, block, 0, s, in, n_in, k,
                     mean, flat, out);
      break;
    case 4:
      DLX_PDL_LAUNCH("downsample_kernel", downsample_kernel<4>, grid, block, 0, s, in, n_in, k,
                     mean, flat, out);
      break;
    default:
      DLX_PDL_LAUNCH("downsample_kernel", downsample_kernel<0>, grid, block, 0, s, in, n_in, k,
                     mean, flat, out);
  }
  return DLX_OK;
}

__global__ void downsample_bwd_kernel(const float* __restrict__ g_out, int n_in, int k, int mean,
                                      const float* __restrict__ flat, float* __restrict__ g_in) {
  pdl_enter();
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= n_in || y >= n_in) return;
  const int n_out = n_in / k;
  const long long o = (long long)(y / k) * n_out + (x / k);
  float v = g_out[o];
  if (flat) v *= flat[o];
  if (mean) v /= (float)(k * k);
  g_in[(long long)y * n_in + x] = v;
}

int launch_downsample_backward(const float* in, const float* g_out, int n_in, int k, int mean,
                               const float* flat, float* g_in, float* g_flat, cudaStream_t s) {
  const int n_out = n_in / k;
  if (g_in) {
    dim3 block(32, 8);
    dim3 grid(ceil_div(n_in, 32), ceil_div(n_in, 8));
    DLX_PDL_LAUNCH("downsample_bwd_kernel", downsample_bwd_kernel, grid, block, 0, s, g_out,
                   n_in, k, mean, flat, g_in);
  }
  if (g_flat) {
    // g_flat = g_out * downsample(in): reuse the forward kernel with flat = g_out.
    DLX_TRY(launch_downsample(in, n_in, k, mean, g_out, g_flat, s));
  }
  (void)n_out;
  return DLX_OK;
}

// ---------------------------------------------------------------------------
// Batched-object reductions (b = l * R + r): per-object wavelength sums of the
// intensity planes and of the pupil-gradient planes, plus the per-object
// weight and tilt gradients. Fixed summation order, so results are
// reproducible and independent of which other objects share the batch.
// ---------------------------------------------------------------------------
// kField: the planes are kept focal fields F (complex64), and each term is
// |F|^2 with the GEMM epilogues' own rounding (intensity_rn), so the sum is
// bitwise the one over intensity planes.
template <bool kField>
__global__ void obj_psf_reduce_kernel(ObjReduceArgs a) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const int R = a.objs.n;
  float total = 0.f;
  for (int r = 0; r < R; ++r) {
    float s = 0.f;
    // kPsfBatch planes' loads in flight (unmasked), then the rest one by
    // one; the sum keeps the wavelength order. Measured at 512^2 x 64 planes:
    // 13.2 us with 16 or 32, 13.9 with 8, 15.0-15.4 with an unrolled loop of
    // 8 (unrolled by 16 or 32: 19.8 and 31.9 us).
    constexpr int kPsfBatch = 16;
    const long long stride = (long long)R * a.npix;
    const long long off = (long long)r * a.npix + p;
    auto term = [&](int l) -> float {
      if constexpr (kField) {
        const float2 f = __ldg(a.fields + off + (long long)l * stride);
        return intensity_rn(f.x, f.y);
      } else {
        return __ldg(a.planes + off + (long long)l * stride);
      }
    };
    int l = 0;
    for (; l + kPsfBatch <= a.L; l += kPsfBatch) {
      float v[kPsfBatch];
#pragma unroll
      for (int u = 0; u < kPsfBatch; ++u) v[u] = term(l + u);
#pragma unroll
      for (int u = 0; u < kPsfBatch; ++u) s += v[u];
    }
    for (; l < a.L; ++l) s += term(l);
    if (a.outs.o[r].psf) a.outs.o[r].psf[p] = s;
    total += s;
  }
  if (a.psf_sum) a.psf_sum[p] = a.accumulate ? a.psf_sum[p] + total : total;
}

int launch_obj_psf_reduce(const ObjReduceArgs& a, cudaStream_t s) {
  if (a.npix == 0 || a.objs.n == 0) return DLX_OK;
  if (a.fields)
    DLX_PDL_LAUNCH("obj_psf_reduce_kernel", obj_psf_reduce_kernel<true>,
                   dim3(ceil_div(a.npix, 256)), dim3(256), 0, s, a);
  else
    DLX_PDL_LAUNCH("obj_psf_reduce_kernel", obj_psf_reduce_kernel<false>,
                   dim3(ceil_div(a.npix, 256)), dim3(256), 0, s, a);
  return DLX_OK;
}

// Pixel gradients summed over every object of the batch (shared pupil).
__global__ void obj_pupil_sum_kernel(ObjReduceArgs a) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const int R = a.objs.n;
  float sre = 0.f, sim = 0.f, sk = 0.f;
  for (int r = 0; r < R; ++r)
    for (int l = 0; l < a.L; ++l) {
      const long long o = ((long long)l * R + r) * a.npix + p;
      const float im = a.pim[o];
      sre += a.pre[o];
      sim += im;
      sk += (float)a.k_dev[l] * im;
    }
  if (a.sum_g_amp) a.sum_g_amp[p] = a.accumulate_sum ? a.sum_g_amp[p] + sre : sre;
  if (a.sum_g_phase) a.sum_g_phase[p] = a.accumulate_sum ? a.sum_g_phase[p] + sim : sim;
  if (a.sum_g_opd) a.sum_g_opd[p] = a.accumulate_sum ? a.sum_g_opd[p] + sk : sk;
}

__global__ void obj_pupil_pix_kernel(ObjReduceArgs a) {
  __shared__ double smem[32];
  const int r = blockIdx.y;
  const int R = a.objs.n;
  ObjOut out = a.outs.o[r];
  if (a.sum_pixels) out.g_amp = out.g_phase = out.g_opd = nullptr;
  if (!out.g_amp && !out.g_phase && !out.g_opd && !out.g_tilt) return;  // block-uniform
  const long long chunk = (a.npix + a.nparts - 1) / a.nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(a.npix, lo + chunk);
  const double half = 0.5 * (a.n_side - 1);
  double tx = 0.0, ty = 0.0;
  for (long long p = lo + threadIdx.x; p < hi; p += blockDim.x) {
    float sre = 0.f, sim = 0.f, sk = 0.f;
    for (int l = 0; l < a.L; ++l) {
      const long long o = ((long long)l * R + r) * a.npix + p;
      const float im = a.pim[o];
      sre += a.pre[o];
      sim += im;
      sk += (float)a.k_dev[l] * im;
    }
    if (out.g_amp) out.g_amp[p] = sre;
    if (out.g_phase) out.g_phase[p] = sim;
    if (out.g_opd) out.g_opd[p] = sk;
    if (out.g_tilt) {  // FP64 partials only when a tilt gradient is wanted
      const int y = (int)(p / a.n_side);
      const int x = (int)(p - (long long)y * a.n_side);
      tx += ((double)x - half) * a.pixel_scale * (double)sk;
      ty += ((double)y - half) * a.pixel_scale * (double)sk;
    }
  }
  if (out.g_tilt) {
    const double sx = block_sum<256>(tx, smem);
    const double sy = block_sum<256>(ty, smem);
    if (threadIdx.x == 0) {
      double* part = a.partial_ws + ((long long)r * a.nparts + blockIdx.x) * 2;
      part[0] = sx;
      part[1] = sy;
    }
  }
}

__global__ void obj_w_partial_kernel(ObjReduceArgs a) {
  __shared__ double smem[32];
  const int R = a.objs.n;
  const int r = blockIdx.y % R;
  const int l = blockIdx.y / R;
  const ObjDesc& od = a.objs.o[r];
  const long long chunk = (a.npix + a.nparts - 1) / a.nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(a.npix, lo + chunk);
  const float* pre = a.pre + ((long long)l * R + r) * a.npix;
  // exact products (FMA) summed in float pairs, widened once per thread
  float h = 0.f, lo_s = 0.f;
  for (long long p = lo + threadIdx.x; p < hi; p += blockDim.x) {
    const float x = pre[p], y = od.amp ? od.amp[p] : 1.0f;
    const float pr = x * y;
    const float t = h + pr;
    const float bv = t - h;
    lo_s += ((h - (t - bv)) + (pr - bv)) + fmaf(x, y, -pr);
    h = t;
  }
  const double t = block_sum_ff<256>(h, lo_s, smem);
  if (threadIdx.x == 0) {
    double* part = a.partial_ws + (long long)R * a.nparts * 2;
    part[((long long)r * a.L + l) * a.nparts + blockIdx.x] = t;
  }
}

__global__ void obj_finish_kernel(ObjReduceArgs a, int want_w) {
  pdl_enter();
  __shared__ double smem[32];
  const int r = blockIdx.x;
  const int R = a.objs.n;
  const ObjDesc& od = a.objs.o[r];
  const ObjOut& out = a.outs.o[r];
  if (out.g_tilt) {
    double sx = 0.0, sy = 0.0;
    for (int i = threadIdx.x; i < a.nparts; i += blockDim.x) {
      sx += a.partial_ws[((long long)r * a.nparts + i) * 2];
      sy += a.partial_ws[((long long)r * a.nparts + i) * 2 + 1];
    }
    const double tx = block_sum<256>(sx, smem);
    const double ty = block_sum<256>(sy, smem);
    if (threadIdx.x == 0) {
      out.g_tilt[0] = (float)tx;
      out.g_tilt[1] = (float)ty;
    }
  }
  if (want_w && out.g_w) {
    const double* part = a.partial_ws + (long long)R * a.nparts * 2;
    for (int l = 0; l < a.L; ++l) {
      double acc = 0.0;
      for (int i = threadIdx.x; i < a.nparts; i += blockDim.x)
        acc += part[((long long)r * a.L + l) * a.nparts + i];
      const double t = block_sum<256>(acc, smem);
      if (threadIdx.x == 0) {
        double v = t;
        if (od.amp_scale) v *= (double)*od.amp_scale;
        const double w = od.weights ? (double)od.weights[l] : 1.0;
        out.g_w[l] = (float)(v / (2.0 * w));
      }
    }
  }
}

// Fused reverse-pass pupil reduction. One block covers a chunk of pixels of
// one object; every thread owns a pixel and walks the wavelengths, forming
// the same per-wavelength planes as the pre/pim path from the pupil field
// Ebar and the unit phasor (recomputed from the phasor kernel's pairs):
//   pre_l = sqrt(w_l) Re(conj(u_l) Ebar_l),  pim_l = amp sqrt(w_l) Im(conj(u_l) Ebar_l)
// and summing them at once: pixel gradients (g_amp = sum pre, g_phase = sum
// pim, g_opd = sum k_l pim), tilt partials, and weight partials
// sum_p pre_l amp_p (per-warp float sums of one pixel each, then FP64).
template <bool kSplit>
__global__ void __launch_bounds__(256, 4) obj_pupil_fused_kernel(ObjReduceArgs a, int want_w) {
  pdl_enter();
  // dynamic shared memory: [L] float4 (1/lambda hi, lo, sqrt(w), k) then, when
  // weight gradients are wanted, [8 warps][L] double partials
  extern __shared__ double dyn[];
  float4* lam = reinterpret_cast<float4*>(dyn);
  double* wpart = dyn + 2 * a.L;
  __shared__ double tsm[32];
  const int r = blockIdx.y;
  const int R = a.objs.n;
  const ObjDesc od = a.objs.o[r];
  const ObjOut out = a.outs.o[r];
  const bool pix_out = !a.sum_pixels && (out.g_amp || out.g_phase || out.g_opd);
  const bool w_out = want_w && out.g_w;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int l = threadIdx.x; l < a.L; l += blockDim.x) {
    const float2 il = a.inv_lambda_ff[l];
    lam[l] = make_float4(il.x, il.y, od.weights ? sqrtf(od.weights[l]) : 1.0f,
                         (float)a.k_dev[l]);
  }
  if (w_out)
    for (int i = threadIdx.x; i < 8 * a.L; i += blockDim.x) wpart[i] = 0.0;
  __syncthreads();
  const long long chunk = (a.npix + a.nparts - 1) / a.nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(a.npix, lo + chunk);
  const double half = 0.5 * (a.n_side - 1);
  const float4* path = a.path + (long long)r * a.npix;
  double tx = 0.0, ty = 0.0;
  for (long long p0 = lo; p0 < hi; p0 += blockDim.x) {  // block-uniform trip count
    const long long p = p0 + threadIdx.x;
    const bool live = p < hi;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    float amp_raw = 1.0f, amp = 1.0f;
    if (live) {
      q = path[p];
      amp_raw = od.amp ? od.amp[p] : 1.0f;
      amp = amp_raw;
      if (od.amp_scale) amp *= *od.amp_scale;
    }
    float sre = 0.f, sim = 0.f, sk = 0.f;
    // The Ebar loads of eight wavelengths are issued before their arithmetic,
    // so that their latencies overlap.
    constexpr int kPre = 8;  // measured: 8 beats 4 (-6.5 us per 64-wavelength step) and 2
    // Whole live warps take the wavelengths in groups of kPreFast with no
    // per-element masks, then the rest in the masked loop below: the same
    // arithmetic in the same order. Measured at 512^2 x 64: 29.6 us with
    // groups of 16, 37.4 with 8, 43.9 with 4 (40.0 us with masks throughout).
    constexpr int kPreFast = 16;
    const bool fast = __all_sync(0xffffffffu, live) && !w_out;
    const int l_fast = fast ? a.L - a.L % kPreFast : 0;
    {
      const float2* ep = a.ebar + (long long)r * a.npix + p;
      const long long estride = (long long)R * a.npix;
      for (int l0 = 0; l0 < l_fast; l0 += kPreFast) {
        float2 ebq[kPreFast];
#pragma unroll
        for (int j = 0; j < kPreFast; ++j) ebq[j] = __ldg(ep + (long long)(l0 + j) * estride);
#pragma unroll
        for (int j = 0; j < kPreFast; ++j) {
          const float2 eb = ebq[j];
          const float4 c = lam[l0 + j];
          const float2 u = kSplit ? cis_ff_split(FF{q.x, q.y}, FF{c.x, c.y}, FF{q.z, q.w})
                                  : cis_ff(FF{q.x, q.y}, FF{c.x, c.y}, FF{q.z, q.w});
          const float sw = c.z;
          const float pr = u.x * eb.x + u.y * eb.y;
          const float pi = u.x * eb.y - u.y * eb.x;
          const float pre = sw * pr;
          const float pim = amp * sw * pi;
          sre += pre;
          sim += pim;
          sk += c.w * pim;
        }
      }
    }
    for (int l0 = l_fast; l0 < a.L; l0 += kPre) {
      float2 ebq[kPre];
#pragma unroll
      for (int j = 0; j < kPre; ++j)
        ebq[j] = (live && l0 + j < a.L) ? a.ebar[((long long)(l0 + j) * R + r) * a.npix + p]
                                        : make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < kPre; ++j) {
        const int l = l0 + j;
        if (l >= a.L) break;  // warp-uniform (l_fast is)
        float pre = 0.f;
        if (live) {
          const float2 eb = ebq[j];
          const float4 c = lam[l];
          const float2 u = kSplit ? cis_ff_split(FF{q.x, q.y}, FF{c.x, c.y}, FF{q.z, q.w})
                                  : cis_ff(FF{q.x, q.y}, FF{c.x, c.y}, FF{q.z, q.w});
          const float sw = c.z;
          const float pr = u.x * eb.x + u.y * eb.y;
          const float pi = u.x * eb.y - u.y * eb.x;
          pre = sw * pr;
          const float pim = amp * sw * pi;
          sre += pre;
          sim += pim;
          sk += c.w * pim;
        }
        if (w_out) {  // warp-uniform
          float v = pre * amp_raw;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
          if (lane == 0) wpart[warp * a.L + l] += (double)v;
        }
      }
    }
    if (live) {
      if (pix_out) {
        if (out.g_amp) out.g_amp[p] = sre;
        if (out.g_phase) out.g_phase[p] = sim;
        if (out.g_opd) out.g_opd[p] = sk;
      }
      if (a.sum_pixels) {
        float* sc = a.pix_scratch + (long long)r * 3 * a.npix;
        sc[p] = sre;
        sc[a.npix + p] = sim;
        sc[2 * a.npix + p] = sk;
      }
      if (out.g_tilt) {  // FP64 partials only when a tilt gradient is wanted
        const int y = (int)(p / a.n_side);
        const int x = (int)(p - (long long)y * a.n_side);
        tx += ((double)x - half) * a.pixel_scale * (double)sk;
        ty += ((double)y - half) * a.pixel_scale * (double)sk;
      }
    }
  }
  if (out.g_tilt) {
    const double sx = block_sum<256>(tx, tsm);
    const double sy = block_sum<256>(ty, tsm);
    if (threadIdx.x == 0) {
      double* part = a.partial_ws + ((long long)r * a.nparts + blockIdx.x) * 2;
      part[0] = sx;
      part[1] = sy;
    }
  }
  if (w_out) {
    __syncthreads();
    double* part = a.partial_ws + (long long)R * a.nparts * 2;
    for (int l = threadIdx.x; l < a.L; l += blockDim.x) {
      double t = 0.0;
      for (int w = 0; w < 8; ++w) t += wpart[w * a.L + l];
      part[((long long)r * a.L + l) * a.nparts + blockIdx.x] = t;
    }
  }
}

// Sum of the per-object pixel gradients over the objects, in object order.
__global__ void obj_pupil_sumr_kernel(ObjReduceArgs a) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  float sre = 0.f, sim = 0.f, sk = 0.f;
  for (int r = 0; r < a.objs.n; ++r) {
    const float* sc = a.pix_scratch + (long long)r * 3 * a.npix;
    sre += sc[p];
    sim += sc[a.npix + p];
    sk += sc[2 * a.npix + p];
  }
  if (a.sum_g_amp) a.sum_g_amp[p] = a.accumulate_sum ? a.sum_g_amp[p] + sre : sre;
  if (a.sum_g_phase) a.sum_g_phase[p] = a.accumulate_sum ? a.sum_g_phase[p] + sim : sim;
  if (a.sum_g_opd) a.sum_g_opd[p] = a.accumulate_sum ? a.sum_g_opd[p] + sk : sk;
}

int launch_obj_pupil_fused(const ObjReduceArgs& a, cudaStream_t s) {
  const int R = a.objs.n;
  if (a.npix == 0 || R == 0) return DLX_OK;
  if (a.L > kFusedPupilMaxL)
    return fail(DLX_ERR_SHAPE, "fused pupil reduction: too many wavelengths");
  bool want_w = false;
  for (int r = 0; r < R; ++r) want_w |= a.outs.o[r].g_w != nullptr;
  const size_t smem = sizeof(float4) * (size_t)a.L + (want_w ? sizeof(double) * 8 * (size_t)a.L : 0);
  static std::atomic<bool> attr_done[kMaxDevices];  // host side, once per device
  int dev = 0;
  DLX_TRY(current_device(&dev));
  if (smem > 48 * 1024 && !attr_done[dev].load()) {
    for (const void* k : {(const void*)obj_pupil_fused_kernel<true>,
                          (const void*)obj_pupil_fused_kernel<false>})
      DLX_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(sizeof(double) * 10 * kFusedPupilMaxL)));
    attr_done[dev].store(true);
  }
  if (a.split_form)
    DLX_PDL_LAUNCH("obj_pupil_fused_kernel", obj_pupil_fused_kernel<true>, dim3(a.nparts, R),
                   dim3(256), smem, s, a, want_w ? 1 : 0);
  else
    DLX_PDL_LAUNCH("obj_pupil_fused_kernel", obj_pupil_fused_kernel<false>, dim3(a.nparts, R),
                   dim3(256), smem, s, a, want_w ? 1 : 0);
  if (a.sum_pixels)
    DLX_PDL_LAUNCH("obj_pupil_sumr_kernel", obj_pupil_sumr_kernel, dim3(ceil_div(a.npix, 256)),
                   dim3(256), 0, s, a);
  DLX_PDL_LAUNCH("obj_finish_kernel", obj_finish_kernel, dim3(R), dim3(256), 0, s, a,
                 want_w ? 1 : 0);
  return DLX_OK;
}

int launch_obj_pupil_reduce(const ObjReduceArgs& a, cudaStream_t s) {
  const int R = a.objs.n;
  if (a.npix == 0 || R == 0) return DLX_OK;
  if (a.sum_pixels) {
    obj_pupil_sum_kernel<<<ceil_div(a.npix, 256), 256, 0, s>>>(a);
    DLX_LAUNCH_CHECK("obj_pupil_sum_kernel");
  }
  bool per_obj = false;
  for (int r = 0; r < R; ++r) {
    const ObjOut& o = a.outs.o[r];
    per_obj |= o.g_tilt != nullptr ||
               (!a.sum_pixels && (o.g_amp || o.g_phase || o.g_opd));
  }
  if (per_obj) {
    obj_pupil_pix_kernel<<<dim3(a.nparts, R), 256, 0, s>>>(a);
    DLX_LAUNCH_CHECK("obj_pupil_pix_kernel");
  }
  bool want_w = false;
  for (int r = 0; r < R; ++r) want_w |= a.outs.o[r].g_w != nullptr;
  if (want_w) {
    obj_w_partial_kernel<<<dim3(a.nparts, R * a.L), 256, 0, s>>>(a);
    DLX_LAUNCH_CHECK("obj_w_partial_kernel");
  }
  DLX_PDL_LAUNCH("obj_finish_kernel", obj_finish_kernel, dim3(R), dim3(256), 0, s, a,
                 want_w ? 1 : 0);
  return DLX_OK;
}

}  // namespace dlx

namespace dlx {

// ---------------------------------------------------------------------------
// Angular-spectrum transfer function (the ASM propagator of dLux's
// layers/abcd_propagators.py:380-459): the centred spectrum F[b][ky][kx] of a
// field sampled at dx is multiplied by
//   H = exp(2 pi i z sqrt(1/lambda^2 - fx^2 - fy^2))      (propagating waves)
//   H = exp(-2 pi z sqrt(fx^2 + fy^2 - 1/lambda^2))        (evanescent waves)
// with f = (k - floor(P/2)) / (P dx). The phase z/lambda sqrt(1 - lambda^2 f^2)
// is formed and reduced in FP64 (it reaches ~1e6 cycles at z = 1 m). H depends
// only on the plan (wavelengths, distance, grid), so it is tabulated once in
// complex64 when the plan is made; a call multiplies by the table (conj = 1:
// by conj(H), the adjoint). FP64 runs at about 1/64 of the FP32 rate here, and
// evaluating H on every call cost 1.5 ms of a 2.9 ms forward + adjoint at 16
// wavelengths of 1024^2.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 asm_h(int kx, int ky, int P, double df, double zl,
                                        double lam2) {
  const int c = P / 2;
  const double fx = (kx - c) * df, fy = (ky - c) * df;
  const double s = lam2 * (fx * fx + fy * fy);
  if (s <= 1.0) return cis_cycles(zl * sqrt(1.0 - s));
  return make_float2((float)exp(-2.0 * CUDART_PI * zl * sqrt(s - 1.0)), 0.0f);
}

__global__ void asm_table_kernel(float2* __restrict__ H, int P, double df,
                                 const double* __restrict__ zl,
                                 const double* __restrict__ lam2) {
  const long long npix = (long long)P * P;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (p >= npix) return;
  const int ky = (int)(p / P);
  const int kx = (int)(p - (long long)ky * P);
  H[(long long)b * npix + p] = asm_h(kx, ky, P, df, zl[b], lam2[b]);
}

__global__ void asm_apply_kernel(float2* __restrict__ f, const float2* __restrict__ H,
                                 long long n, int conj) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 h = H[i];
  if (conj) h.y = -h.y;
  f[i] = cmul(f[i], h);
}

int launch_asm_table(float2* H, int batch, int P, double df, const double* zl,
                     const double* lam2, cudaStream_t s) {
  if (batch <= 0 || P <= 0) return DLX_OK;
  dim3 grid(ceil_div((long long)P * P, 256), batch);
  asm_table_kernel<<<grid, 256, 0, s>>>(H, P, df, zl, lam2);
  DLX_LAUNCH_CHECK("asm_table_kernel");
  return DLX_OK;
}

int launch_asm_apply(float2* spec, const float2* H, int batch, int P, int conj,
                     cudaStream_t s) {
  const long long n = (long long)batch * P * P;
  if (n <= 0) return DLX_OK;
  asm_apply_kernel<<<ceil_div(n, 256), 256, 0, s>>>(spec, H, n, conj);
  DLX_LAUNCH_CHECK("asm_apply_kernel");
  return DLX_OK;
}

}  // namespace dlx
