// epilogue.cuh -- per-element GEMM epilogues shared by the FP32 and the
// tensor-core forms. `v` is the raw accumulator D[b][m][n]; alpha_b is the
// per-batch scale (the MFT normalisation nfringes / (N_in N_out)).
#pragma once

#include <math_constants.h>

#include "kernels.h"

namespace dlx {

__device__ __forceinline__ void store_split(__nv_bfloat16* base_b, long long plane, long long idx,
                                            float2 v) {
  __nv_bfloat16 h, l;
  split_bf16(v.x, h, l);
  base_b[idx] = h;
  base_b[plane + idx] = l;
  split_bf16(v.y, h, l);
  base_b[2 * plane + idx] = h;
  base_b[3 * plane + idx] = l;
}

// (t.x + i t.y)(x + i y): the per-column phasor of EpiArgs::coltilt.
__device__ __forceinline__ float2 ctilt(float2 t, float x, float y) {
  return make_float2(t.x * x - t.y * y, t.x * y + t.y * x);
}

// Wavelength and object of batch element b (b = l * R + r for a batched plan
// of R objects; R = 1 otherwise).
__device__ __forceinline__ int epi_objects(const EpiArgs& e) { return e.objs.n > 0 ? e.objs.n : 1; }

// Unit phasor of object r's pupil field at pixel p = y * n + x, wavelength l
// (recomputed in the reverse pass instead of stored).
__device__ __forceinline__ float2 pupil_unit_phasor(const EpiArgs& e, int l, int r, int y, int x,
                                                    int n, long long p) {
  // Same arithmetic as the phasor kernel so that forward and reverse agree.
  const float2 il = e.inv_lambda_ff[l];
  if (e.path) {
    // the phasor kernel's own (path, phase) pairs: no FP64 work per wavelength
    const float4 q = e.path[(long long)r * n * n + p];
    return cis_ff(FF{q.x, q.y}, FF{il.x, il.y}, FF{q.z, q.w});
  }
  const bool obj = e.objs.n > 0;
  const float* opd = obj ? e.objs.o[r].opd : e.opd;
  const float* phase = obj ? e.objs.o[r].phase : e.phase;
  const float4 t = obj ? tilt_pairs(e.objs.o[r].tilt_x, e.objs.o[r].tilt_y, e.pixel_scale)
                       : tilt_pairs(e.tilt_x, e.tilt_y, e.pixel_scale);
  const float half = 0.5f * (float)(n - 1);
  const FF path = pupil_path(opd ? opd[p] : 0.f, (float)x - half, (float)y - half, t);
  const FF ph = phase ? phase_cycles(phase[p]) : FF{0.f, 0.f};
  return cis_ff(path, FF{il.x, il.y}, ph);
}

// F-bar input of EPI_DOT: split planes (hi + lo) at split index sidx of planes
// of splane elements, or complex64 at dense index idx of planes of plane elements.
__device__ __forceinline__ float2 epi_read_in(const EpiArgs& e, int b, long long plane,
                                              long long idx, long long splane, long long sidx) {
  if (e.in_split) {
    const __nv_bfloat16* p = e.in_split + (long long)b * 4 * splane + sidx;
    return make_float2(__bfloat162float(p[0]) + __bfloat162float(p[splane]),
                       __bfloat162float(p[2 * splane]) + __bfloat162float(p[3 * splane]));
  }
  return e.in_c64[(long long)b * plane + idx];
}

// ---- per-element epilogues; l = wavelength, r = object, a = alpha_l ----
__device__ __forceinline__ void epi_gradf_value(const EpiArgs& e, int b, int r, float a,
                                                long long idx, float2& v) {
  // cotangent of F = alpha * D for <G, |F|^2>: 2 G F = 2 alpha G D; with no
  // cotangent (G null) the focal field F = alpha D itself, kept for a later
  // reverse pass
  const float* G = e.objs.n > 0 ? e.objs.o[r].G : e.G;
  float g = a;
  if (G) {
    g = 2.0f * a * G[idx];
    if (e.bweight) g *= e.bweight[b];
  }
  v = make_float2(g * v.x, g * v.y);
}

__device__ __forceinline__ void epi_pupil_store(const EpiArgs& e, int b, int l, int r, float a,
                                                int m, int n, int N, long long plane,
                                                long long idx, float2 v) {
  // D = Ebar / alpha at pupil pixel (y = m, x = n), square pupil M == N.
  const bool obj = e.objs.n > 0;
  const float* amp_p = obj ? e.objs.o[r].amp : e.amp;
  const float* amp_s = obj ? e.objs.o[r].amp_scale : e.amp_scale;
  const float* w_p = obj ? e.objs.o[r].weights : e.weights;
  const float2 eb = make_float2(a * v.x, a * v.y);
  const float2 u = pupil_unit_phasor(e, l, r, m, n, N, idx);
  const float sw = w_p ? sqrtf(w_p[l]) : 1.0f;
  float amp = amp_p ? amp_p[idx] : 1.0f;
  if (amp_s) amp *= *amp_s;
  // conj(u) * eb
  const float re = u.x * eb.x + u.y * eb.y;
  const float im = u.x * eb.y - u.y * eb.x;
  e.out_f32[(long long)b * plane + idx] = sw * re;
  e.out_f32b[(long long)b * plane + idx] = amp * sw * im;
}

__device__ __forceinline__ void epi_apply(const EpiArgs& e, int b, int m, int n, int M, int N,
                                          float2 v) {
  const int R = epi_objects(e);
  const int l = b / R;
  const int r = b - l * R;
  const float a = e.alpha ? e.alpha[l] : 1.0f;
  const long long plane = (long long)M * N;
  const long long idx = (long long)m * N + n;
  // split outputs and inputs have padded rows (split_ld)
  const long long splane = split_plane(M, N);
  const long long sidx = (long long)m * split_ld(N) + n;
  if (e.coltilt && (e.kind == EPI_C64 || e.kind == EPI_SPLIT || e.kind == EPI_SPLIT2)) {
    v = ctilt(e.coltilt[(long long)b * N + n], v.x, v.y);
  }
  switch (e.kind) {
    case EPI_C64: {
      e.out_c64[(long long)b * plane + idx] = make_float2(a * v.x, a * v.y);
      break;
    }
    case EPI_SPLIT: {
      store_split(e.out_split + (long long)b * 4 * splane, splane, sidx,
                  make_float2(a * v.x, a * v.y));
      break;
    }
    case EPI_INTENSITY: {
      e.out_f32[(long long)b * plane + idx] = intensity_rn(__fmul_rn(a, v.x), __fmul_rn(a, v.y));
      break;
    }
    case EPI_GRADF:
    case EPI_PSF_GRADF: {
      if (e.kind == EPI_PSF_GRADF && e.out_f32)
        e.out_f32[(long long)b * plane + idx] =
            intensity_rn(__fmul_rn(a, v.x), __fmul_rn(a, v.y));
      epi_gradf_value(e, b, r, a, idx, v);
      if (e.out_split)
        store_split(e.out_split + (long long)b * 4 * splane, splane, sidx, v);
      else
        e.out_c64[(long long)b * plane + idx] = v;
      break;
    }
    case EPI_PUPIL: {
      epi_pupil_store(e, b, l, r, a, m, n, N, plane, idx, v);
      break;
    }
    case EPI_SPLIT2: {
      const float2 av = make_float2(a * v.x, a * v.y);
      const float w = e.colw[n];
      if (e.out_split) {
        store_split(e.out_split + (long long)b * 4 * splane, splane, sidx, av);
        store_split(e.out_split2 + (long long)b * 4 * splane, splane, sidx,
                    make_float2(w * av.x, w * av.y));
      } else {
        e.out_c64[(long long)b * plane + idx] = av;
        e.out_c642[(long long)b * plane + idx] = make_float2(w * av.x, w * av.y);
      }
      break;
    }
    case EPI_DOT: {
      const float2 fb = epi_read_in(e, b, plane, idx, splane, sidx);
      e.out_f32[(long long)b * plane + idx] = e.kf[l] * a * (fb.y * v.x - fb.x * v.y);
      break;
    }
    default:
      break;
  }
}

// Column form used by the tensor-core kernels: one thread holds 32 values
// D[b][m0 + j][n], j = 0..31, of one output column n, and the 32 lanes of a
// warp hold consecutive n. Every load and store below is therefore one
// contiguous segment per warp. Rows m >= M are skipped; n < N is the
// caller's check.
// KIND >= 0 fixes the epilogue at compile time (one kernel instantiation per
// kind keeps each instantiation's registers to its own epilogue); -1 reads
// e.kind at run time.
template <int KIND = -1>
__device__ __forceinline__ void epi_col32(const EpiArgs& e, int b, int n, int m0, int M, int N,
                                          const float* re, const float* im) {
  const int R = epi_objects(e);
  const int l = b / R;
  const int r = b - l * R;
  const float a = e.alpha ? e.alpha[l] : 1.0f;
  const long long plane = (long long)M * N;
  const int mc = M - m0 < 32 ? M - m0 : 32;
  const long long idx0 = (long long)m0 * N + n;
  // split outputs and inputs have padded rows (split_ld)
  const int ld = split_ld(N);
  const long long splane = (long long)M * ld;
  const long long sidx0 = (long long)m0 * ld + n;
  switch (KIND >= 0 ? KIND : e.kind) {
    case EPI_C64:
    case EPI_SPLIT: {
      // (a, 0) without a tilt: a re - 0 im and a im + 0 re are exactly a re, a im
      float2 t = make_float2(a, 0.f);
      if (e.coltilt) {
        const float2 c = e.coltilt[(long long)b * N + n];
        t = make_float2(a * c.x, a * c.y);
      }
      if ((KIND >= 0 ? KIND : e.kind) == EPI_C64) {
        float2* o = e.out_c64 + (long long)b * plane + idx0;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (j < mc) o[(long long)j * N] = ctilt(t, re[j], im[j]);
      } else {
        __nv_bfloat16* o = e.out_split + (long long)b * 4 * splane + sidx0;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (j < mc) store_split(o, splane, (long long)j * ld, ctilt(t, re[j], im[j]));
      }
      break;
    }
    case EPI_INTENSITY: {
      float* o = e.out_f32 + (long long)b * plane + idx0;
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < mc)
          o[(long long)j * N] = intensity_rn(__fmul_rn(a, re[j]), __fmul_rn(a, im[j]));
      break;
    }
    case EPI_GRADF:
    case EPI_PSF_GRADF: {
      // no intensity planes when a forward keeps F (out_f32 null): the
      // wavelength sum then reads F itself
      if ((KIND >= 0 ? KIND : e.kind) == EPI_PSF_GRADF && e.out_f32) {
        float* o = e.out_f32 + (long long)b * plane + idx0;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (j < mc)
            o[(long long)j * N] = intensity_rn(__fmul_rn(a, re[j]), __fmul_rn(a, im[j]));
      }
      // 16 loads at a time, so that their latencies overlap. No cotangent (G
      // null, warp-uniform): the focal field F = alpha D itself is stored.
      const float* G0 = e.objs.n > 0 ? e.objs.o[r].G : e.G;
      const float* G = G0 ? G0 + idx0 : nullptr;
      const float s = G0 ? 2.0f * a * (e.bweight ? e.bweight[b] : 1.0f) : a;
#pragma unroll
      for (int h = 0; h < 32; h += 16) {
        float g[16];
#pragma unroll
        for (int j = 0; j < 16; ++j)
          g[j] = h + j < mc ? (G ? __ldg(G + (long long)(h + j) * N) : 1.0f) : 0.0f;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (h + j < mc) {
            const float gj = s * g[j];
            const float2 v = make_float2(gj * re[h + j], gj * im[h + j]);
            if (e.out_split)
              store_split(e.out_split + (long long)b * 4 * splane + sidx0, splane,
                          (long long)(h + j) * ld, v);
            else
              e.out_c64[(long long)b * plane + idx0 + (long long)(h + j) * N] = v;
          }
        }
      }
      break;
    }
    case EPI_SPLIT2: {
      const float w = e.colw[n];
      const float2 t = e.coltilt ? e.coltilt[(long long)b * N + n] : make_float2(1.f, 0.f);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (j < mc) {
          const float2 av = ctilt(t, a * re[j], a * im[j]);
          const long long o = idx0 + (long long)j * N;
          if (e.out_split) {
            const long long so = sidx0 + (long long)j * ld;
            store_split(e.out_split + (long long)b * 4 * splane, splane, so, av);
            store_split(e.out_split2 + (long long)b * 4 * splane, splane, so,
                        make_float2(w * av.x, w * av.y));
          } else {
            e.out_c64[(long long)b * plane + o] = av;
            e.out_c642[(long long)b * plane + o] = make_float2(w * av.x, w * av.y);
          }
        }
      }
      break;
    }
    case EPI_DOT: {
      const float ka = e.kf[l] * a;
      float* o = e.out_f32 + (long long)b * plane + idx0;
#pragma unroll
      for (int j0 = 0; j0 < 32; j0 += 8) {
        float2 fb[8];
#pragma unroll
        for (int t = 0; t < 8; ++t)
          fb[t] = j0 + t < mc ? epi_read_in(e, b, plane, idx0 + (long long)(j0 + t) * N, splane,
                                            sidx0 + (long long)(j0 + t) * ld)
                              : make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < 8; ++t)
          if (j0 + t < mc)
            o[(long long)(j0 + t) * N] = ka * (fb[t].y * re[j0 + t] - fb[t].x * im[j0 + t]);
      }
      break;
    }
    case EPI_PUPIL: {
      if (!e.path) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (j < mc)
            epi_pupil_store(e, b, l, r, a, m0 + j, n, N, plane, idx0 + (long long)j * N,
                            make_float2(re[j], im[j]));
        break;
      }
      // Same arithmetic as epi_pupil_store with the (path, phase) pairs of the
      // phasor kernel; loads are issued eight rows at a time ahead of the math.
      const bool obj = e.objs.n > 0;
      const float* amp_p = obj ? e.objs.o[r].amp : e.amp;
      const float* amp_s = obj ? e.objs.o[r].amp_scale : e.amp_scale;
      const float* w_p = obj ? e.objs.o[r].weights : e.weights;
      const float sw = w_p ? sqrtf(w_p[l]) : 1.0f;
      const float2 il = e.inv_lambda_ff[l];
      const float4* path = e.path + (long long)r * N * N + idx0;
      float* o_re = e.out_f32 + (long long)b * plane + idx0;
      float* o_im = e.out_f32b + (long long)b * plane + idx0;
#pragma unroll
      for (int j0 = 0; j0 < 32; j0 += 8) {
        float4 q[8];
        float am[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int j = j0 + t;
          q[t] = j < mc ? __ldg(path + (long long)j * N) : make_float4(0.f, 0.f, 0.f, 0.f);
          am[t] = (amp_p && j < mc) ? __ldg(amp_p + idx0 + (long long)j * N) : 1.0f;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int j = j0 + t;
          if (j < mc) {
            const float2 eb = make_float2(a * re[j], a * im[j]);
            const float2 u = cis_ff(FF{q[t].x, q[t].y}, FF{il.x, il.y}, FF{q[t].z, q[t].w});
            float amp = am[t];
            if (amp_s) amp *= *amp_s;
            const float pr = u.x * eb.x + u.y * eb.y;
            const float pi = u.x * eb.y - u.y * eb.x;
            o_re[(long long)j * N] = sw * pr;
            o_im[(long long)j * N] = amp * sw * pi;
          }
        }
      }
      break;
    }
    default:
      break;
  }
}

}  // namespace dlx
