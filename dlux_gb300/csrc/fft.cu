// fft.cu -- the padded, centred 2-D FFT of dLux (utils/propagation.py:8-64,
// utils/fourier.py:14-78, wavefronts.py:654-727) as power-of-two FFTs of
// lines in shared memory, for large pad * N where the exact DFT-GEMM pair
// costs O(P^2 N).
//
// The DFT-GEMM form uses A[k][j] = exp(2 pi i s (j + npad - c)(k - c) / P)
// times the input and output phase ramps. Since exp(2 pi i s j' k' / P) is
// P-periodic in j' and k', that is a plain length-P FFT whose input element j
// sits at slot (j + npad - c) mod P and whose output element k is read at slot
// (k - c) mod P. One kernel covers every pass. It loads n_in elements of each
// line through an input ramp, scatters them into bit-reversed slots, runs the
// log2(P) radix-2 butterfly stages in place and gathers n_out elements through
// an output ramp and a scale. The stages are grouped into radix-2^R passes: a
// thread keeps 2^R elements in registers for R consecutive stages, so shared
// memory is touched once per R stages; R is 3 up to P = 2048 and 4 from
// P = 4096 (max_radix_log2). A block holds 4 lines up to P = 1024 and 2 above
// (lines_per_block). The passes are:
//   forward   rows:    N lines of N -> P   (x), into tmp [N][P]
//             columns: P lines of N -> P   (y), from tmp into out [P][P]
//   adjoint   rows:    P lines of P -> N   (x, conjugate), into tmp [P][N]
//             columns: N lines of P -> N   (y, conjugate), into gin [N][N]
// Ramps exp(2 pi i (g j + d)) are reduced exactly in FP32 pairs (cis_ff), and
// the twiddles exp(2 pi i s k / P) come from sincospif of an exact argument,
// one table per plan with every stage's twiddles contiguous. The butterflies
// read the table from global memory through L1 (32 KB at P = 4096), which
// keeps the shared memory of a block to its lines.
#include <atomic>
#include <cmath>
#include <string>
#include <vector>

#include "kernels.h"

namespace dlx {

struct LineRamp {  // per batch element
  float2 g_in, d_in, g_out, d_out;  // float pairs (hi, lo), cycles per index / cycles
  float scale;
  int ramp_in, ramp_out;            // 0: the ramp is identically 1 (skipped)
};

namespace {

// Lines of one launch: line l of batch b starts at base + b * bs + l * ls and
// its elements are es apart.
struct LineIO {
  long long bs, ls, es;
};

// Shared-memory slot of element k of line li (P elements per line). The low
// four index bits are XORed with every higher nibble of k and with a
// per-line pattern, so that one wavefront of 16 threads (8-byte words) lands
// in 16 distinct bank pairs in the radix-16 passes (16 consecutive k, or k 16
// apart in the first pass) and in the gathers, also when a wavefront spans
// several lines (the column passes). The second radix-8 pass (two groups of
// 8 k, 64 apart) sees 2-way conflicts; removing them (bit 6 folded into bit
// 3 as well) measured no faster. Per-line patterns:
//   2 lines x 8 elements:  pattern 9 flips bits 0 and 3 of the second line;
//   4 lines x 4 elements:  pattern 5 li gives distinct low and high bit pairs.
// The bit-reversed scatter sees at most 2-way conflicts at the sizes used
// (4-way at P = 512 and 8192 with 2 lines per block). Every map is a
// bijection on [0, P): only the low nibble changes, by a value that depends
// on the other bits. For P < 16 it is the identity.
template <int LPB>
__device__ __forceinline__ int smem_slot(int li, int k, int P) {
  if (P < 16) return li * P + k;
  const int g = LPB == 2 ? 9 * li : (LPB == 4 ? 5 * li : li);
  return li * P + (k ^ (((k >> 4) ^ (k >> 8) ^ (k >> 12) ^ g) & 15));
}

// Butterfly stages s .. s + R - 1 of every line (half-lengths h = 2^lh, 2h,
// ..., 2^(R-1) h) as one pass: the 2^R elements k0 + m h of a group stay in
// registers across the R stages, so shared memory is read and written once
// per R stages. These are the same butterflies and twiddles, in the same
// order, as R radix-2 stages: at half-length H = 2^j h, element m (bit j
// clear) pairs with m + 2^j and takes the twiddle of position
// pos + (m mod 2^j) h.
template <int LPB, int R>
__device__ __forceinline__ void radix_pass(float2* x, const float2* __restrict__ tw, float sign,
                                           int log2p, int lh, int P) {
  constexpr int M = 1 << R;
  const int h = 1 << lh;
  const int gq = log2p - R;  // P / 2^R groups per line
  for (int t = threadIdx.x; t < (LPB << gq); t += blockDim.x) {
    const int li = t >> gq;
    const int i = t & ((1 << gq) - 1);
    const int grp = i >> lh;
    const int pos = i & (h - 1);
    const int k0 = (grp << (lh + R)) + pos;
    float2 v[M];
#pragma unroll
    for (int m = 0; m < M; ++m) v[m] = x[smem_slot<LPB>(li, k0 + m * h, P)];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int H = h << j;
#pragma unroll
      for (int m = 0; m < M; ++m) {
        if (m & (1 << j)) continue;
        float2 w = __ldg(tw + H - 1 + pos + (m & ((1 << j) - 1)) * h);
        w.y *= sign;
        const float2 u = v[m];
        const float2 q = cmul(v[m + (1 << j)], w);
        v[m] = make_float2(u.x + q.x, u.y + q.y);
        v[m + (1 << j)] = make_float2(u.x - q.x, u.y - q.y);
      }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) x[smem_slot<LPB>(li, k0 + m * h, P)] = v[m];
  }
}

// Registers are capped so that the shared memory sets the residency: radix-16
// passes (RMAX 4) at 80 registers, three blocks per SM (64 KB each at
// P = 4096); radix-8 passes at 64, four blocks.
template <int LPB, int RMAX>
__global__ void __launch_bounds__(256, RMAX >= 4 ? 3 : 4) fft_lines_kernel(
    const float2* __restrict__ in, LineIO io_in, int n_in, int off_in,
    float2* __restrict__ out, LineIO io_out, int n_out, int off_out, int lines, int log2p,
    float sign, const LineRamp* __restrict__ ramps, const float2* __restrict__ twg) {
  extern __shared__ float2 sm[];
  const int P = 1 << log2p;
  float2* x = sm;  // [LPB][P], slots by smem_slot
  const int b = blockIdx.y;
  const int l0 = blockIdx.x * LPB;
  const LineRamp rp = ramps[b];
  for (int i = threadIdx.x; i < LPB * P; i += blockDim.x) x[i] = make_float2(0.f, 0.f);
  __syncthreads();
  // load: consecutive threads take consecutive addresses (line-major when the
  // lines are adjacent in memory, element-major otherwise)
  const bool line_fast = io_in.ls == 1;
  for (int t = threadIdx.x; t < LPB * n_in; t += blockDim.x) {
    const int li = line_fast ? t % LPB : t / n_in;
    const int e = line_fast ? t / LPB : t % n_in;
    const int l = l0 + li;
    if (l >= lines) continue;
    float2 v = in[(long long)b * io_in.bs + (long long)l * io_in.ls + (long long)e * io_in.es];
    if (rp.ramp_in)
      v = cmul(v, cis_ff(FF{(float)e, 0.f}, FF{rp.g_in.x, rp.g_in.y}, FF{rp.d_in.x, rp.d_in.y}));
    const int slot = (e + off_in) & (P - 1);  // P is a power of two: also for e + off_in < 0
    const int k = log2p > 0 ? (int)(__brev((unsigned)slot) >> (32 - log2p)) : 0;
    x[smem_slot<LPB>(li, k, P)] = v;
  }
  __syncthreads();
  // Butterfly stages RMAX at a time (radix-2^RMAX passes), then one pass of
  // the remaining stages.
  for (int st = 1; st <= log2p;) {
    const int R = log2p - st + 1 < RMAX ? log2p - st + 1 : RMAX;
    switch (R) {
      case 4: if constexpr (RMAX >= 4) radix_pass<LPB, 4>(x, twg, sign, log2p, st - 1, P); break;
      case 3: radix_pass<LPB, 3>(x, twg, sign, log2p, st - 1, P); break;
      case 2: radix_pass<LPB, 2>(x, twg, sign, log2p, st - 1, P); break;
      default: radix_pass<LPB, 1>(x, twg, sign, log2p, st - 1, P); break;
    }
    __syncthreads();
    st += R;
  }
  const bool oline_fast = io_out.ls == 1;
  for (int t = threadIdx.x; t < LPB * n_out; t += blockDim.x) {
    const int li = oline_fast ? t % LPB : t / n_out;
    const int o = oline_fast ? t / LPB : t % n_out;
    const int l = l0 + li;
    if (l >= lines) continue;
    const int slot = (o + off_out) & (P - 1);
    float2 v = x[smem_slot<LPB>(li, slot, P)];
    if (rp.ramp_out)
      v = cmul(v, cis_ff(FF{(float)o, 0.f}, FF{rp.g_out.x, rp.g_out.y},
                         FF{rp.d_out.x, rp.d_out.y}));
    v.x *= rp.scale;
    v.y *= rp.scale;
    out[(long long)b * io_out.bs + (long long)l * io_out.ls + (long long)o * io_out.es] = v;
  }
}

// Twiddles of every butterfly stage, stage by stage: entry h - 1 + pos of the
// stage with half-length h is exp(i pi pos / h) (the direction's sign is
// applied when a block copies the table). pos / h is exact in FP32.
__global__ void fft_twiddle_kernel(int P, float2* __restrict__ tw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P - 1) return;
  const int h = 1 << (31 - __clz(k + 1));  // largest power of two <= k + 1
  const int pos = k + 1 - h;
  float sn, cs;
  sincospif((float)pos / (float)h, &sn, &cs);
  tw[k] = make_float2(cs, sn);
}

// Few lines per block keeps several blocks resident per SM (the butterfly
// stages are latency-bound); two lines keep column loads at 16-byte segments.
int lines_per_block(int P) { return P <= 1024 ? 4 : 2; }

// Stages per shared-memory pass. Measured forward + adjoint of 16 planes:
// radix-8 passes win up to P = 2048 (1.93 against 2.04 ms for radix-16 at
// P = 2048), radix-16 passes from P = 4096 (8.0 ms).
int max_radix_log2(int P) { return P >= 4096 ? 4 : 3; }

int launch_lines(const float2* in, LineIO io_in, int n_in, int off_in, float2* out, LineIO io_out,
                 int n_out, int off_out, int lines, int batch, int log2p, float sign,
                 const LineRamp* ramps, const float2* tw, cudaStream_t s) {
  const int P = 1 << log2p;
  const int lpb = lines_per_block(P);
  const int rmax = max_radix_log2(P);
  const size_t smem = sizeof(float2) * (size_t)lpb * P;
  static std::atomic<bool> attr_done[kMaxDevices];  // host side, once per device
  int dev = 0;
  DLX_TRY(current_device(&dev));
  if (!attr_done[dev].load()) {
    const int lim = 200 * 1024;  // covers P <= 8192 at the lines-per-block choice above
    DLX_TRY_CUDA(cudaFuncSetAttribute(fft_lines_kernel<4, 3>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    DLX_TRY_CUDA(cudaFuncSetAttribute(fft_lines_kernel<4, 4>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    DLX_TRY_CUDA(cudaFuncSetAttribute(fft_lines_kernel<2, 3>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    DLX_TRY_CUDA(cudaFuncSetAttribute(fft_lines_kernel<2, 4>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    attr_done[dev].store(true);
  }
  dim3 grid((lines + lpb - 1) / lpb, batch);
#define DLX_FFT_LAUNCH(L, R)                                                                \
  fft_lines_kernel<L, R><<<grid, 256, smem, s>>>(in, io_in, n_in, off_in, out, io_out, n_out, \
                                                 off_out, lines, log2p, sign, ramps, tw)
  if (lpb == 4) {
    if (rmax >= 4) DLX_FFT_LAUNCH(4, 4); else DLX_FFT_LAUNCH(4, 3);
  } else {
    if (rmax >= 4) DLX_FFT_LAUNCH(2, 4); else DLX_FFT_LAUNCH(2, 3);
  }
#undef DLX_FFT_LAUNCH
  DLX_LAUNCH_CHECK("fft_lines_kernel");
  return DLX_OK;
}

}  // namespace

int radix_fft_create(RadixFft* f, int batch, int N, int pad, bool inverse, const DftAxis* axes,
                     const float* alphas) {
  f->batch = batch;
  f->N = N;
  f->P = N * pad;
  int lg = 0;
  while ((1 << lg) < f->P) ++lg;
  if ((1 << lg) != f->P || f->P > 8192)
    return fail(DLX_ERR_SHAPE, "radix FFT: pad * n_in must be a power of two <= 8192");
  f->log2p = lg;
  f->npad = (N * (pad - 1)) / 2;
  f->c = f->P / 2;
  f->sign = inverse ? 1.0f : -1.0f;
  std::vector<LineRamp> rx(batch), ry(batch), rax(batch), ray(batch);
  auto ff2 = [](double v) {
    const FF f = ff_from_double(v);
    return make_float2(f.hi, f.lo);
  };
  for (int b = 0; b < batch; ++b) {
    const DftAxis& ax = axes[b];
    LineRamp r{};
    r.g_in = ff2(ax.g_in);
    r.d_in = ff2(ax.d_in);
    r.g_out = ff2(ax.g_out);
    r.d_out = ff2(ax.d_out);
    r.scale = (float)ax.scale;
    r.ramp_in = (ax.g_in != 0.0 || ax.d_in != 0.0) ? 1 : 0;
    r.ramp_out = (ax.g_out != 0.0 || ax.d_out != 0.0) ? 1 : 0;
    rx[b] = r;
    r.scale = (float)ax.scale * alphas[b];  // the normalisation goes on the last pass
    ry[b] = r;
    // adjoint: the conjugate output ramp on the input side and vice versa
    LineRamp q{};
    q.g_in = ff2(-ax.g_out);
    q.d_in = ff2(-ax.d_out);
    q.g_out = ff2(-ax.g_in);
    q.d_out = ff2(-ax.d_in);
    q.scale = (float)ax.scale;
    q.ramp_in = r.ramp_out;
    q.ramp_out = r.ramp_in;
    rax[b] = q;
    q.scale = (float)ax.scale * alphas[b];
    ray[b] = q;
  }
  for (auto* pr : {&f->ramps_x, &f->ramps_y, &f->ramps_ax, &f->ramps_ay})
    DLX_TRY_CUDA(cudaMalloc(pr, sizeof(LineRamp) * batch));
  DLX_TRY_CUDA(cudaMemcpy(f->ramps_x, rx.data(), sizeof(LineRamp) * batch, cudaMemcpyHostToDevice));
  DLX_TRY_CUDA(cudaMemcpy(f->ramps_y, ry.data(), sizeof(LineRamp) * batch, cudaMemcpyHostToDevice));
  DLX_TRY_CUDA(cudaMemcpy(f->ramps_ax, rax.data(), sizeof(LineRamp) * batch, cudaMemcpyHostToDevice));
  DLX_TRY_CUDA(cudaMemcpy(f->ramps_ay, ray.data(), sizeof(LineRamp) * batch, cudaMemcpyHostToDevice));
  const cudaError_t e = cudaMalloc(&f->tmp, sizeof(float2) * (size_t)batch * N * f->P);
  if (e != cudaSuccess) {
    f->tmp = nullptr;
    cudaGetLastError();
    return fail(DLX_ERR_NOMEM, "radix FFT: workspace allocation failed");
  }
  if (f->P > 1) {
    DLX_TRY_CUDA(cudaMalloc(&f->tw, sizeof(float2) * (size_t)(f->P - 1)));
    fft_twiddle_kernel<<<(f->P - 1 + 255) / 256, 256>>>(f->P, f->tw);
    DLX_LAUNCH_CHECK("fft_twiddle_kernel");
    // the table is read from the caller's streams, which need not wait for this one
    DLX_TRY_CUDA(cudaDeviceSynchronize());
  }
  return DLX_OK;
}

void radix_fft_release(RadixFft* f) {
  for (LineRamp* r : {f->ramps_x, f->ramps_y, f->ramps_ax, f->ramps_ay})
    if (r) cudaFree(r);
  if (f->tmp) cudaFree(f->tmp);
  if (f->tw) cudaFree(f->tw);
  f->ramps_x = f->ramps_y = f->ramps_ax = f->ramps_ay = nullptr;
  f->tmp = nullptr;
  f->tw = nullptr;
}

// out [b][P][P] = FFT of in [b][N][N] (the forward of the DFT-GEMM FFT plan).
int radix_fft_forward(const RadixFft& f, const float2* in, float2* out, cudaStream_t s) {
  const int N = f.N, P = f.P, off_in = f.npad - f.c, off_out = -f.c;
  // rows: line y of N elements (x), output row of P into tmp[b][y][:]
  DLX_TRY(launch_lines(in, LineIO{(long long)N * N, N, 1}, N, off_in, f.tmp,
                       LineIO{(long long)N * P, P, 1}, P, off_out, N, f.batch, f.log2p, f.sign,
                       f.ramps_x, f.tw, s));
  // columns: line kx of N elements (y, stride P), output column of P into out
  return launch_lines(f.tmp, LineIO{(long long)N * P, 1, P}, N, off_in, out,
                      LineIO{(long long)P * P, 1, P}, P, off_out, P, f.batch, f.log2p, f.sign,
                      f.ramps_y, f.tw, s);
}

// gin [b][N][N] = adjoint applied to gout [b][P][P].
int radix_fft_adjoint(const RadixFft& f, const float2* gout, float2* gin, cudaStream_t s) {
  const int N = f.N, P = f.P;
  // The adjoint reads slot (k - c) and writes slot (j + npad - c), with the
  // opposite sign and the conjugate ramps swapped between input and output.
  // rows: line ky of P elements (kx), output N elements (x) into tmp[b][ky][:]
  DLX_TRY(launch_lines(gout, LineIO{(long long)P * P, P, 1}, P, -f.c, f.tmp,
                       LineIO{(long long)P * N, N, 1}, N, f.npad - f.c, P, f.batch, f.log2p,
                       -f.sign, f.ramps_ax, f.tw, s));
  // columns: line x of P elements (ky, stride N), output N elements (y) into gin
  return launch_lines(f.tmp, LineIO{(long long)P * N, 1, N}, P, -f.c, gin,
                      LineIO{(long long)N * N, 1, N}, N, f.npad - f.c, N, f.batch, f.log2p,
                      -f.sign, f.ramps_ay, f.tw, s);
}

}  // namespace dlx
