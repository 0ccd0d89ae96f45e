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

// Unit phasor of the pupil field at pixel p = y * n + x for batch b
// (recomputed in the reverse pass instead of stored).
__device__ __forceinline__ float2 pupil_unit_phasor(const EpiArgs& e, int b, int y, int x, int n,
                                                    long long p) {
  // Same arithmetic as the phasor kernel so that forward and reverse agree.
  const double half = 0.5 * (n - 1);
  const double X = ((double)x - half) * e.pixel_scale;
  const double Y = ((double)y - half) * e.pixel_scale;
  const FF path = ff_from_double((e.opd ? (double)e.opd[p] : 0.0) + e.tilt_x * X + e.tilt_y * Y);
  const FF ph = ff_from_double(e.phase ? (double)e.phase[p] * (0.5 / CUDART_PI) : 0.0);
  const float2 il = e.inv_lambda_ff[b];
  return cis_ff(path, FF{il.x, il.y}, ph);
}

__device__ __forceinline__ void epi_apply(const EpiArgs& e, int b, int m, int n, int M, int N,
                                          float2 v) {
  const float a = e.alpha ? e.alpha[b] : 1.0f;
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
      const float g = 2.0f * a * e.G[idx];
      float2 w = make_float2(g * v.x, g * v.y);
      if (e.out_split)
        store_split(e.out_split + (long long)b * 4 * plane, plane, idx, w);
      else
        e.out_c64[(long long)b * plane + idx] = w;
      break;
    }
    case EPI_PUPIL: {
      // D = Ebar / alpha at pupil pixel (y = m, x = n), square pupil M == N.
      const float2 eb = make_float2(a * v.x, a * v.y);
      const float2 u = pupil_unit_phasor(e, b, m, n, N, idx);
      const float sw = e.weights ? sqrtf(e.weights[b]) : 1.0f;
      float amp = e.amp ? e.amp[idx] : 1.0f;
      if (e.amp_scale) amp *= *e.amp_scale;
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
