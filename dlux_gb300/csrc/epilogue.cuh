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

// Wavelength and object of batch element b (b = l * R + r for a batched plan
// of R objects; R = 1 otherwise).
__device__ __forceinline__ int epi_objects(const EpiArgs& e) { return e.objs.n > 0 ? e.objs.n : 1; }

// Unit phasor of object r's pupil field at pixel p = y * n + x, wavelength l
// (recomputed in the reverse pass instead of stored).
__device__ __forceinline__ float2 pupil_unit_phasor(const EpiArgs& e, int l, int r, int y, int x,
                                                    int n, long long p) {
  // Same arithmetic as the phasor kernel so that forward and reverse agree.
  const bool obj = e.objs.n > 0;
  const float* opd = obj ? e.objs.o[r].opd : e.opd;
  const float* phase = obj ? e.objs.o[r].phase : e.phase;
  const double tx = obj ? e.objs.o[r].tilt_x : e.tilt_x;
  const double ty = obj ? e.objs.o[r].tilt_y : e.tilt_y;
  const double half = 0.5 * (n - 1);
  const double X = ((double)x - half) * e.pixel_scale;
  const double Y = ((double)y - half) * e.pixel_scale;
  const FF path = ff_from_double((opd ? (double)opd[p] : 0.0) + tx * X + ty * Y);
  const FF ph = ff_from_double(phase ? (double)phase[p] * (0.5 / CUDART_PI) : 0.0);
  const float2 il = e.inv_lambda_ff[l];
  return cis_ff(path, FF{il.x, il.y}, ph);
}

__device__ __forceinline__ void epi_apply(const EpiArgs& e, int b, int m, int n, int M, int N,
                                          float2 v) {
  const int R = epi_objects(e);
  const int l = b / R;
  const int r = b - l * R;
  const float a = e.alpha ? e.alpha[l] : 1.0f;
  const long long plane = (long long)M * N;
  const long long idx = (long long)m * N + n;
  switch (e.kind) {
    case EPI_C64: {
      e.out_c64[(long long)b * plane + idx] = make_float2(a * v.x, a * v.y);
      break;
    }
    case EPI_SPLIT: {
      store_split(e.out_split + (long long)b * 4 * plane, plane, idx, make_float2(a * v.x, a * v.y));
      break;
    }
    case EPI_INTENSITY: {
      e.out_f32[(long long)b * plane + idx] = a * a * (v.x * v.x + v.y * v.y);
      break;
    }
    case EPI_GRADF: {
      // cotangent of F = alpha * D for <G, |F|^2>: 2 G F = 2 alpha G D
      const float* G = e.objs.n > 0 ? e.objs.o[r].G : e.G;
      const float g = 2.0f * a * G[idx];
      float2 w = make_float2(g * v.x, g * v.y);
      if (e.out_split)
        store_split(e.out_split + (long long)b * 4 * plane, plane, idx, w);
      else
        e.out_c64[(long long)b * plane + idx] = w;
      break;
    }
    case EPI_PUPIL: {
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
      break;
    }
    default:
      break;
  }
}

}  // namespace dlx
