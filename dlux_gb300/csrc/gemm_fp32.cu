// gemm_fp32.cu -- plain FP32 batched complex GEMM on the CUDA cores.
//
//   D[b][m][n] = sum_k opA(A[b][m][k]) * B[b][n][k]     (complex64 operands)
//
// Both operands are K-contiguous. A CTA computes a 128 x 64 complex tile with
// 256 threads (8 x 4 complex per thread), stages BK = 8 complex of K per step
// in double-buffered shared memory (k-major, so the inner loop reads
// contiguous float4 runs) and prefetches the next K-slab from global memory
// into registers with float4 loads while the current slab is consumed.
// Every element's epilogue is applied in registers (epilogue.cuh).
#include "epilogue.cuh"

namespace dlx {
namespace {

constexpr int BM = 128;
constexpr int BN = 64;
constexpr int BK = 8;
constexpr int THREADS = 256;

template <bool CONJ_A, bool VEC>
__global__ __launch_bounds__(THREADS) void cgemm_fp32_kernel(GemmArgs g) {
  __shared__ __align__(16) float2 As[2][BK][BM];
  __shared__ __align__(16) float2 Bs[2][BK][BN];

  const int tid = threadIdx.x;
  const int tx = tid & 15;   // n direction
  const int ty = tid >> 4;   // m direction
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * BM;
  const int n0 = blockIdx.x * BN;
  const int M = g.M, N = g.N, K = g.K;

  const float2* Ab = g.A + (long long)(b / (g.a_batch_div > 0 ? g.a_batch_div : 1)) * g.a_bs;
  const float2* Bb = g.B + (long long)(b / (g.b_batch_div > 0 ? g.b_batch_div : 1)) * g.b_bs;

  // Global load mapping: A: row = tid/2, k = (tid&1)*4 .. +3 ; B: row = tid/4, k = (tid&3)*2 .. +1
  const int a_row = tid >> 1, a_k = (tid & 1) * 4;
  const int b_row = tid >> 2, b_k = (tid & 3) * 2;
  const int gm = m0 + a_row, gn = n0 + b_row;

  float2 ra[4], rb[2];
  auto load_slab = [&](int k0) {
    if (VEC) {
      // K % 8 == 0 and 16-byte aligned rows: the whole slab is in range along K.
      if (gm < M) {
        const float4* src = reinterpret_cast<const float4*>(Ab + (long long)gm * K + k0 + a_k);
        float4 v0 = __ldg(src), v1 = __ldg(src + 1);
        ra[0] = make_float2(v0.x, v0.y); ra[1] = make_float2(v0.z, v0.w);
        ra[2] = make_float2(v1.x, v1.y); ra[3] = make_float2(v1.z, v1.w);
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) ra[i] = make_float2(0.f, 0.f);
      }
      if (gn < N) {
        const float4* src = reinterpret_cast<const float4*>(Bb + (long long)gn * K + k0 + b_k);
        float4 v = __ldg(src);
        rb[0] = make_float2(v.x, v.y); rb[1] = make_float2(v.z, v.w);
      } else {
        rb[0] = rb[1] = make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k = k0 + a_k + i;
        ra[i] = (gm < M && k < K) ? __ldg(Ab + (long long)gm * K + k) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int k = k0 + b_k + i;
        rb[i] = (gn < N && k < K) ? __ldg(Bb + (long long)gn * K + k) : make_float2(0.f, 0.f);
      }
    }
  };
  auto store_slab = [&](int buf) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float2 v = ra[i];
      if (CONJ_A) v.y = -v.y;
      As[buf][a_k + i][a_row] = v;
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) Bs[buf][b_k + i][b_row] = rb[i];
  };

  float2 acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);

  const int nslabs = (K + BK - 1) / BK;
  load_slab(0);
  store_slab(0);
  __syncthreads();

  for (int s = 0; s < nslabs; ++s) {
    const int buf = s & 1;
    if (s + 1 < nslabs) load_slab((s + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float2 a[8], bv[4];
      const float4* pa = reinterpret_cast<const float4*>(&As[buf][kk][ty * 8]);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float4 t = pa[i];
        a[2 * i] = make_float2(t.x, t.y);
        a[2 * i + 1] = make_float2(t.z, t.w);
      }
      const float4* pb = reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float4 t = pb[j];
        bv[2 * j] = make_float2(t.x, t.y);
        bv[2 * j + 1] = make_float2(t.z, t.w);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x = fmaf(a[i].x, bv[j].x, acc[i][j].x);
          acc[i][j].x = fmaf(-a[i].y, bv[j].y, acc[i][j].x);
          acc[i][j].y = fmaf(a[i].x, bv[j].y, acc[i][j].y);
          acc[i][j].y = fmaf(a[i].y, bv[j].x, acc[i][j].y);
        }
    }
    if (s + 1 < nslabs) store_slab(buf ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int m = m0 + ty * 8 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n < N) epi_apply(g.epi, b, m, n, M, N, acc[i][j]);
    }
  }
}

}  // namespace

int launch_gemm_fp32(const GemmArgs& g, cudaStream_t s) {
  if (g.batch <= 0 || g.M <= 0 || g.N <= 0) return DLX_OK;
  const bool aligned = ((uintptr_t)g.A % 16 == 0) && ((uintptr_t)g.B % 16 == 0) &&
                       (g.a_bs % 2 == 0) && (g.b_bs % 2 == 0);
  const bool vec = aligned && (g.K % BK == 0);
  dim3 grid(ceil_div(g.N, BN), ceil_div(g.M, BM), g.batch);
  if (g.conj_a) {
    if (vec) cgemm_fp32_kernel<true, true><<<grid, THREADS, 0, s>>>(g);
    else cgemm_fp32_kernel<true, false><<<grid, THREADS, 0, s>>>(g);
  } else {
    if (vec) cgemm_fp32_kernel<false, true><<<grid, THREADS, 0, s>>>(g);
    else cgemm_fp32_kernel<false, false><<<grid, THREADS, 0, s>>>(g);
  }
  DLX_LAUNCH_CHECK("cgemm_fp32_kernel");
  return DLX_OK;
}

}  // namespace dlx
