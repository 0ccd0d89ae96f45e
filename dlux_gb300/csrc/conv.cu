// conv.cu -- 2-D convolution of a PSF with a small kernel, mode "same"
// (jax.scipy.signal.convolve as used by PSF.convolve, psfs.py:93-110;
// ResolvedSource / PointResolvedSource, sources.py:490-521 and :711-748;
// ApplyJitter, layers/detector_layers.py:134-199).
//
// out[i][j] = sum_{a,b} in[i + s0 - a][j + s1 - b] k[a][b], s = (K - 1) / 2 (the
// centre crop of the full convolution), zero outside `in`. The reverse pass
// needs:
//   g_in[m][n] = sum_{a,b} g_out[m - s0 + a][n - s1 + b] k[a][b]  (a correlation:
//                the same kernel flipped, with the mirrored offset)
//   g_k[a][b]  = sum_{i,j} g_out[i][j] in[i + s0 - a][j + s1 - b]
// A 32 x 32 output tile and its halo are staged in shared memory, and so is the
// kernel. The kernel gradient gives each kernel element one block with a
// fixed summation order.
#include <string>

#include "kernels.h"

namespace dlx {
namespace {

constexpr int CT = 32;  // output tile side

// flip = 0: convolution (out = in * k); flip = 1: correlation (out[m] = sum g[m - s + a] k[a]).
__global__ void conv2d_same_kernel(const float* __restrict__ in, int H, int W,
                                   const float* __restrict__ k, int K0, int K1, int flip,
                                   float* __restrict__ out) {
  extern __shared__ float sm[];
  const int s0 = (K0 - 1) / 2, s1 = (K1 - 1) / 2;
  const int TH = CT + K0 - 1, TW = CT + K1 - 1;
  float* tile = sm;               // [TH][TW]
  float* ks = sm + TH * TW;       // [K0][K1]
  const int b = blockIdx.z;
  const float* inb = in + (long long)b * H * W;
  const int i0 = blockIdx.y * CT, j0 = blockIdx.x * CT;
  // input rows needed: convolution i + s0 - a for a in [0, K0) -> [i0 + s0 - K0 + 1, i0 + CT - 1 + s0];
  // correlation m - s0 + a -> [i0 - s0, i0 + CT - 1 - s0 + K0 - 1]
  const int r_lo = flip ? i0 - s0 : i0 + s0 - K0 + 1;
  const int c_lo = flip ? j0 - s1 : j0 + s1 - K1 + 1;
  for (int t = threadIdx.x; t < TH * TW; t += blockDim.x) {
    const int r = r_lo + t / TW, c = c_lo + t % TW;
    tile[t] = (r >= 0 && r < H && c >= 0 && c < W) ? inb[(long long)r * W + c] : 0.0f;
  }
  for (int t = threadIdx.x; t < K0 * K1; t += blockDim.x) ks[t] = k[t];
  __syncthreads();
  // Each thread computes four adjacent outputs of one tile row (CT x CT / 4 =
  // 256 groups, one per thread), with a four-value window of the tile row that
  // slides by one element per kernel column: one shared-memory load for the
  // tile and one for the kernel per four FMAs. Every output keeps the term
  // order (kernel rows, then columns) of a one-output-per-thread loop.
  const int ti = threadIdx.x >> 3, tj0 = (threadIdx.x & 7) * 4;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int a = 0; a < K0; ++a) {
    // tile row of input index (convolution) i + s0 - a, (correlation) i - s0 + a
    const int tr = flip ? ti + a : ti + K0 - 1 - a;
    const float* row = tile + tr * TW;
    const float* krow = ks + a * K1;
    if (flip) {
      // output u, kernel column bb: tile column tj0 + u + bb
      float w0 = row[tj0], w1 = row[tj0 + 1], w2 = row[tj0 + 2], w3 = row[tj0 + 3];
      for (int bb = 0; bb < K1; ++bb) {
        const float k = krow[bb];
        acc[0] = fmaf(w0, k, acc[0]);
        acc[1] = fmaf(w1, k, acc[1]);
        acc[2] = fmaf(w2, k, acc[2]);
        acc[3] = fmaf(w3, k, acc[3]);
        if (bb + 1 < K1) {
          w0 = w1; w1 = w2; w2 = w3;
          w3 = row[tj0 + bb + 4];
        }
      }
    } else {
      // output u, kernel column bb: tile column tj0 + u + K1 - 1 - bb
      float w0 = row[tj0 + K1 - 1], w1 = row[tj0 + K1], w2 = row[tj0 + K1 + 1],
            w3 = row[tj0 + K1 + 2];
      for (int bb = 0; bb < K1; ++bb) {
        const float k = krow[bb];
        acc[0] = fmaf(w0, k, acc[0]);
        acc[1] = fmaf(w1, k, acc[1]);
        acc[2] = fmaf(w2, k, acc[2]);
        acc[3] = fmaf(w3, k, acc[3]);
        if (bb + 1 < K1) {
          w3 = w2; w2 = w1; w1 = w0;
          w0 = row[tj0 + K1 - 2 - bb];
        }
      }
    }
  }
  const int i = i0 + ti;
  if (i < H) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + tj0 + u;
      if (j < W) out[(long long)b * H * W + (long long)i * W + j] = acc[u];
    }
  }
}

// g_k[a][c] = sum_{i,j} g_out[i][j] in[i + s0 - a][j + s1 - c] over every batch
// element (kernel row a, kernel column c), in two stages.
// Stage 1: a block takes kernel row a, a chunk of KC kernel columns and a band
// of image rows, over every batch element. One g_out value meets the KC shifted
// input values of its row, which are read through L1. Each thread sums its
// products in FP32 kFold at a time and folds those partial sums into KC float
// pairs (Knuth's TwoSum), so the per-product cost is one FMA: a partial of 16
// products loses ~1e-6 of its own size at most, far below the tolerance, and
// the float pairs keep the long sum over the band exact to that order. The block's sums go to part[band][a][c] in double. Compared with
// one block per kernel element, g_out and the input are read from L2 once per
// chunk instead of once per kernel element. KC is chosen per kernel width so
// that the chunks divide it with the least padding.
// Stage 2: g_k[a][c] sums the bands in order, so the result is deterministic.
constexpr int kFold = 16;

template <int KC>
__global__ void __launch_bounds__(256) conv2d_kgrad_rows_kernel(
    const float* __restrict__ in, const float* __restrict__ g, int H, int W, int batch, int K0,
    int K1, int rows_per_band, double* __restrict__ part) {
  __shared__ double red[8][KC];
  const int a = blockIdx.x;
  const int c0 = blockIdx.y * KC;  // first kernel column of the chunk
  const int band = blockIdx.z;
  const int s0 = (K0 - 1) / 2, s1 = (K1 - 1) / 2;
  // rows i of the band with i + s0 - a in [0, H)
  const int i0 = max(band * rows_per_band, max(0, a - s0));
  const int i1 = min(min(H, (band + 1) * rows_per_band), H + a - s0);
  float hi[KC], lo[KC], acc[KC];
#pragma unroll
  for (int q = 0; q < KC; ++q) hi[q] = lo[q] = acc[q] = 0.f;
  auto fold = [&]() {
#pragma unroll
    for (int q = 0; q < KC; ++q) {
      const float t = hi[q] + acc[q];
      const float bv = t - hi[q];
      lo[q] += (hi[q] - (t - bv)) + (acc[q] - bv);
      hi[q] = t;
      acc[q] = 0.f;
    }
  };
  const long long npix = (long long)H * W;
  int terms = 0;
  for (int b = 0; b < batch; ++b) {
    for (int i = i0; i < i1; ++i) {
      const float* grow = g + b * npix + (long long)i * W;
      const float* xrow = in + b * npix + (long long)(i + s0 - a) * W;
      for (int j = threadIdx.x; j < W; j += blockDim.x) {
        const float x = grow[j];
#pragma unroll
        for (int q = 0; q < KC; ++q) {
          const int c = j + s1 - (c0 + q);  // input column of kernel column c0 + q
          if (c0 + q < K1 && c >= 0 && c < W) acc[q] = fmaf(x, __ldg(xrow + c), acc[q]);
        }
        if (++terms == kFold) {
          fold();
          terms = 0;
        }
      }
    }
  }
  fold();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < KC; ++q) {
    double v = (double)hi[q] + (double)lo[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < KC && c0 + (int)threadIdx.x < K1) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
    part[((long long)band * K0 + a) * K1 + c0 + threadIdx.x] = t;
  }
}

__global__ void conv2d_kgrad_sum_kernel(const double* __restrict__ part, int nband, int nk,
                                        float* __restrict__ g_k) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  double t = 0.0;
  for (int band = 0; band < nband; ++band) t += part[(long long)band * nk + k];
  g_k[k] = (float)t;
}

int launch_conv_kgrad(const float* in, const float* g, int H, int W, int batch, int K0, int K1,
                      float* g_k, cudaStream_t s) {
  // the chunk width with the least padding of K1 (ties to the wider chunk)
  int kc = 16;
  for (int c : {16, 12, 11, 8, 4})
    if (((K1 + c - 1) / c) * c < ((K1 + kc - 1) / kc) * kc) kc = c;
  const int nchunk = (K1 + kc - 1) / kc;
  // about two blocks per SM in all
  int sms = 0;
  DLX_TRY(device_sm_count(&sms));
  int nband = (2 * sms + K0 * nchunk - 1) / (K0 * nchunk);
  if (nband > H) nband = H;
  if (nband < 1) nband = 1;
  const int rows = (H + nband - 1) / nband;
  nband = (H + rows - 1) / rows;
  const int nk = K0 * K1;
  double* part = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&part, sizeof(double) * (size_t)nband * nk, s));
  const dim3 grid(K0, nchunk, nband);
  switch (kc) {
    case 4: conv2d_kgrad_rows_kernel<4><<<grid, 256, 0, s>>>(in, g, H, W, batch, K0, K1, rows, part); break;
    case 8: conv2d_kgrad_rows_kernel<8><<<grid, 256, 0, s>>>(in, g, H, W, batch, K0, K1, rows, part); break;
    case 11: conv2d_kgrad_rows_kernel<11><<<grid, 256, 0, s>>>(in, g, H, W, batch, K0, K1, rows, part); break;
    case 12: conv2d_kgrad_rows_kernel<12><<<grid, 256, 0, s>>>(in, g, H, W, batch, K0, K1, rows, part); break;
    default: conv2d_kgrad_rows_kernel<16><<<grid, 256, 0, s>>>(in, g, H, W, batch, K0, K1, rows, part); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    conv2d_kgrad_sum_kernel<<<(nk + 255) / 256, 256, 0, s>>>(part, nband, nk, g_k);
    e = cudaGetLastError();
  }
  cudaFreeAsync(part, s);
  if (e != cudaSuccess) return check_cuda(e, "conv2d kernel gradient");
  note_launch();
  note_launch();
  return DLX_OK;
}

int check_conv(int batch, int H, int W, int K0, int K1) {
  if (batch <= 0 || H <= 0 || W <= 0 || K0 <= 0 || K1 <= 0)
    return fail(DLX_ERR_SHAPE, "conv2d: sizes must be positive");
  if (K0 > 128 || K1 > 128)
    return fail(DLX_ERR_SHAPE, "conv2d: kernels up to 128 x 128 are supported");
  return DLX_OK;
}

int launch_conv(const float* in, int batch, int H, int W, const float* k, int K0, int K1, int flip,
                float* out, cudaStream_t s) {
  const size_t smem = sizeof(float) * ((size_t)(CT + K0 - 1) * (CT + K1 - 1) + (size_t)K0 * K1);
  if (smem > 48 * 1024)
    DLX_TRY_CUDA(cudaFuncSetAttribute(conv2d_same_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((W + CT - 1) / CT, (H + CT - 1) / CT, batch);
  // 256 threads: one group of four outputs of a CT x CT tile each
  static_assert(CT * CT / 4 == 256, "one output group per thread");
  conv2d_same_kernel<<<grid, 256, smem, s>>>(in, H, W, k, K0, K1, flip, out);
  DLX_LAUNCH_CHECK("conv2d_same_kernel");
  return DLX_OK;
}

}  // namespace
}  // namespace dlx

using namespace dlx;

extern "C" {

int dlx_conv2d_same(const float* in, int batch, int height, int width, const float* kernel,
                    int k0, int k1, float* out, void* stream) {
  DLX_TRY(check_conv(batch, height, width, k0, k1));
  if (!in || !kernel || !out) return fail(DLX_ERR_ARG, "conv2d: null pointer");
  return launch_conv(in, batch, height, width, kernel, k0, k1, 0, out,
                     static_cast<cudaStream_t>(stream));
}

int dlx_conv2d_same_backward(const float* in, int batch, int height, int width,
                             const float* kernel, int k0, int k1, const float* g_out,
                             float* g_in, float* g_kernel, void* stream) {
  DLX_TRY(check_conv(batch, height, width, k0, k1));
  if (!g_out || (g_in && !kernel) || (g_kernel && !in))
    return fail(DLX_ERR_ARG, "conv2d_backward: null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (g_in) DLX_TRY(launch_conv(g_out, batch, height, width, kernel, k0, k1, 1, g_in, s));
  if (g_kernel) DLX_TRY(launch_conv_kgrad(in, g_out, height, width, batch, k0, k1, g_kernel, s));
  return DLX_OK;
}

}  // extern "C"
