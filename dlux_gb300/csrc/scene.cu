// scene.cu -- many point sources seen through one pupil (PointSources.model,
// sources.py:392-411) without a pupil field per source.
//
// A source at angle (tx, ty) tilts the pupil field by exp(i k (tx X + ty Y))
// (wavefronts.py:370-395). In the two-step MFT that factor folds into the
// DFT matrices: with in = (i - c)/N and out = (j - c_out) s_out, the
// x-matrix of the tilted field is
//     A'x[u][x] = exp(-2 pi i in_x (out_u - tx N dx / lambda)),
// i.e. the untilted matrix with its output coordinates shifted. So
//   * the pupil field E_l is built once per wavelength and shared by every
//     source (B operand with batch divisor R);
//   * the shift factors: A'[b][u][x] = A0[l][u][x] t_b[x] with the untilted
//     matrix A0 (made once per plan by an error-free FP32 kernel) and the
//     tilt phasor t_b[x] = exp(2 pi i x theta N dx / lambda);
//   * each (source, wavelength) gets its own M x N matrix A'x (M x N elements
//     instead of an N x N field per source: 8x less at N = 1024, M = 128),
//     written by a store-bound pass A0 * tx;
//   * the y tilt multiplies column y of the first GEMM's output D1 in its
//     epilogue, so the second GEMM reads the shared A0 of the wavelength
//     (F = alpha A0 (ty.D1)^T), which stays in L2;
//   * position gradients come from dF/dtx = i k alpha A'y (A'x (X.E))^T and
//     dF/dty = i k alpha A'y (Y.D1)^T dotted with F-bar (again with A'y D =
//     A0 (ty.D)), with no per-source pupil-plane reverse pass.
// image = sum_{s,l} w[s][l] |F_{s,l}|^2 for per-(source, wavelength) weights
// w (spectrum x flux). The reverse pass returns d/dw and d/d(position).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "epilogue.cuh"

namespace dlx {
namespace {

// (i - c) / N style coordinates as float pairs, from FP64.
__global__ void scene_xtable_kernel(int n, double a, double b, float2* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const FF f = ff_from_double(a * (double)i + b);
  out[i] = make_float2(f.hi, f.lo);
}

// A0[l][j][i] = exp(-2 pi i x_i u_lj), u_lj = a_out[l] j + b_out[l]: the untilted
// DFT matrix of every wavelength (the same for both axes), reduced exactly in
// FP32 pairs (cis_ff). Written as c64 and, for the tensor-core form, as split
// planes [l][4][j][split_ld(N)].
__global__ void scene_a0_kernel(int M, int N, const float2* __restrict__ xin,
                                const double* __restrict__ a_out,
                                const double* __restrict__ b_out, float2* __restrict__ a0,
                                __nv_bfloat16* __restrict__ a0s) {
  const long long mn = (long long)M * N;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (p >= mn) return;
  const int j = (int)(p / N);
  const int i = (int)(p - (long long)j * N);
  const float2 x = xin[i];
  const FF u = ff_from_double(a_out[l] * (double)j + b_out[l]);
  const float2 c = cis_ff(FF{x.x, x.y}, u, FF{0.f, 0.f});
  const float2 v = make_float2(c.x, -c.y);  // forward transform: exp(-2 pi i t)
  a0[(long long)l * mn + p] = v;
  if (a0s) {
    const long long smn = split_plane(M, N);
    __nv_bfloat16* base = a0s + (long long)l * 4 * smn + (long long)j * split_ld(N) + i;
    __nv_bfloat16 h, lo;
    split_bf16(v.x, h, lo);
    base[0] = h;
    base[smn] = lo;
    split_bf16(v.y, h, lo);
    base[2 * smn] = h;
    base[3 * smn] = lo;
  }
}

// Source tilt as a phasor per pupil column (x) and row (y): for batch element
// b = l Rc + r,
//   tx[b][i] = exp(+2 pi i x_i theta_{r,x} / fringe_l), ty likewise with theta_{r,y},
// so that the tilted matrices are A'[b][j][i] = A0[l][j][i] t[b][i]
// (exp(-2 pi i x (u - theta / fringe)) = exp(-2 pi i x u) exp(2 pi i x theta / fringe)).
__global__ void scene_tilt_kernel(int N, int Rc, const float2* __restrict__ xin,
                                  const double* __restrict__ inv_fringe,
                                  const double* __restrict__ pos, float2* __restrict__ tx,
                                  float2* __restrict__ ty) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  const int l = b / Rc, r = b - (b / Rc) * Rc;
  // theta / fringe of this (source, wavelength) as float pairs, formed once
  // per block in FP64
  __shared__ float4 st;
  if (threadIdx.x == 0) {
    const FF sx = ff_from_double(pos[2 * r] * inv_fringe[l]);
    const FF sy = ff_from_double(pos[2 * r + 1] * inv_fringe[l]);
    st = make_float4(sx.hi, sx.lo, sy.hi, sy.lo);
  }
  __syncthreads();
  if (i >= N) return;
  const float2 x = xin[i];
  tx[(long long)b * N + i] = cis_ff(FF{x.x, x.y}, FF{st.x, st.y}, FF{0.f, 0.f});
  ty[(long long)b * N + i] = cis_ff(FF{x.x, x.y}, FF{st.z, st.w}, FF{0.f, 0.f});
}

struct alignas(8) Bf16x4 {
  __nv_bfloat16 v[4];
};

// A'x[b][j][i] = A0[l][j][i] tx[b][i] for the sources r0 .. r0 + rg - 1 of
// wavelength l = blockIdx.y (r0 = blockIdx.z rg): a store-bound pass, each
// thread holding V consecutive elements of one matrix row (V = 4 needs N % 4 == 0)
// and reusing its A0 values for every source of the group. Split rows are
// padded to split_ld(N).
template <int V>
__global__ void scene_ax_kernel(int M, int N, int Rc, int rg, const float2* __restrict__ a0,
                                const float2* __restrict__ tx, __nv_bfloat16* __restrict__ ax_s,
                                float2* __restrict__ ax_c) {
  const long long mn = (long long)M * N;
  const long long p0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * V;
  const int l = blockIdx.y;
  const int r0 = blockIdx.z * rg;
  if (p0 >= mn) return;
  const int j0 = (int)(p0 / N);
  const int i0 = (int)(p0 - (long long)j0 * N);
  const long long smn = split_plane(M, N);
  float2 a[V];
#pragma unroll
  for (int k = 0; k < V; ++k) a[k] = a0[(long long)l * mn + p0 + k];
  const int r1 = r0 + rg < Rc ? r0 + rg : Rc;
  for (int r = r0; r < r1; ++r) {
    const long long b = (long long)l * Rc + r;
    float2 v[V];
#pragma unroll
    for (int k = 0; k < V; ++k) v[k] = ctilt(tx[b * N + i0 + k], a[k].x, a[k].y);
    if (ax_s) {
      Bf16x4 q[4];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        split_bf16(v[k].x, q[0].v[k], q[1].v[k]);
        split_bf16(v[k].y, q[2].v[k], q[3].v[k]);
      }
      __nv_bfloat16* base = ax_s + b * 4 * smn + (long long)j0 * split_ld(N) + i0;
      if (V == 4) {
#pragma unroll
        for (int c = 0; c < 4; ++c) *reinterpret_cast<Bf16x4*>(base + c * smn) = q[c];
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
          for (int k = 0; k < V; ++k) base[c * smn + k] = q[c].v[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < V; ++k) ax_c[b * mn + p0 + k] = v[k];
    }
  }
}

// Untilted pupil field of every wavelength, E_l = amp scale cis(k_l opd + phase)
// (the phasor kernel's arithmetic for one object with unit weight), and
// X.E_l with X the pupil x coordinate (m).
__global__ void scene_field_kernel(int n, int L, double pixel_scale, const float* __restrict__ amp,
                                   const float* __restrict__ amp_scale,
                                   const float* __restrict__ opd, const float* __restrict__ phase,
                                   const float2* __restrict__ inv_lambda_ff,
                                   __nv_bfloat16* __restrict__ e_s, __nv_bfloat16* __restrict__ ex_s,
                                   float2* __restrict__ e_c, float2* __restrict__ ex_c) {
  const long long npix = (long long)n * n;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int y = (int)(p / n);
  const int x = (int)(p - (long long)y * n);
  const float X = (float)(((double)x - 0.5 * (n - 1)) * pixel_scale);
  const FF path{opd ? opd[p] : 0.f, 0.f};
  const FF ph = phase ? phase_cycles(phase[p]) : FF{0.f, 0.f};
  float a = amp ? amp[p] : 1.0f;
  if (amp_scale) a *= *amp_scale;
  for (int l = 0; l < L; ++l) {
    const float2 il = inv_lambda_ff[l];
    const float2 u = cis_ff(path, FF{il.x, il.y}, ph);
    const float2 v = make_float2(u.x * a, u.y * a);
    const float2 w = make_float2(v.x * X, v.y * X);
    if (e_s) {
      // split rows padded to split_ld(n)
      const long long sp = split_plane(n, n);
      const long long o = (long long)l * 4 * sp + (long long)y * split_ld(n) + x;
      __nv_bfloat16* b0 = e_s + o;
      __nv_bfloat16* b1 = ex_s + o;
      __nv_bfloat16 h, lo;
      split_bf16(v.x, h, lo); b0[0] = h; b0[sp] = lo;
      split_bf16(v.y, h, lo); b0[2 * sp] = h; b0[3 * sp] = lo;
      split_bf16(w.x, h, lo); b1[0] = h; b1[sp] = lo;
      split_bf16(w.y, h, lo); b1[2 * sp] = h; b1[3 * sp] = lo;
    } else {
      e_c[(long long)l * npix + p] = v;
      ex_c[(long long)l * npix + p] = w;
    }
  }
}

// image[p] (+)= sum_b w[s][l] planes[b][p], b = l R + r, source s = s0 + r; fixed order.
__global__ void scene_image_kernel(const float* __restrict__ planes, int R, int L, long long npix,
                                   const float* __restrict__ w, int s0, int accumulate,
                                   float* __restrict__ image) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  float acc = 0.f;
  for (int l = 0; l < L; ++l)
    for (int r = 0; r < R; ++r)
      acc += w[(long long)(s0 + r) * L + l] * planes[((long long)l * R + r) * npix + p];
  image[p] = accumulate ? image[p] + acc : acc;
}

// out[b] = sum_p planes[b][p] (times G[p] when given), float-pair accumulation.
__global__ void scene_bsum_kernel(const float* __restrict__ planes, long long npix,
                                  const float* __restrict__ G, double* __restrict__ out) {
  __shared__ double smem[32];
  const int b = blockIdx.x;
  const float* row = planes + (long long)b * npix;
  float hi = 0.f, lo = 0.f;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    const float x = row[p];
    const float y = G ? G[p] : 1.0f;
    const float pr = x * y;
    const float pe = fmaf(x, y, -pr);
    const float t = hi + pr;
    const float bv = t - hi;
    lo += ((hi - (t - bv)) + (pr - bv)) + pe;
    hi = t;
  }
  double v = (double)hi + (double)lo;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += smem[i];
    out[b] = t;
  }
}

// Per source: g_w[s][l] = bsum[l R + r] (weights) or g_pos[s][axis] = sum_l bsum[l R + r].
__global__ void scene_finish_kernel(const double* __restrict__ bsum, int R, int L, int s0,
                                    float* __restrict__ g_w, float* __restrict__ g_pos, int axis) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  if (g_w)
    for (int l = 0; l < L; ++l) g_w[(long long)(s0 + r) * L + l] = (float)bsum[l * R + r];
  if (g_pos) {
    double t = 0.0;
    for (int l = 0; l < L; ++l) t += bsum[l * R + r];
    g_pos[2 * (s0 + r) + axis] = (float)t;
  }
}

// bw[b] = w[s0 + r][l] for b = l Rc + r: the cotangent weight of every batch element.
__global__ void scene_gather_weights_kernel(const float* __restrict__ w, int Rc, int L, int s0,
                                            float* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= Rc * L) return;
  const int l = b / Rc, r = b - (b / Rc) * Rc;
  out[b] = w[(long long)(s0 + r) * L + l];
}

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  int alloc(size_t n) {
    if (n == 0) return DLX_OK;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return fail(DLX_ERR_NOMEM, "scene plan: cudaMalloc of " + std::to_string(n) + " bytes failed");
    }
    bytes = n;
    return DLX_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

}  // namespace
}  // namespace dlx

using namespace dlx;

struct dlx_scene_plan_s {
  int L = 0, N = 0, M = 0, R = 0, variant = 0;
  double ps_in = 0, ps_out = 0, focal = 0;
  std::vector<double> wl;
  // constants
  Buf alpha, kf, a_out, b_out, inv_fringe, inv_lambda_ff, xin, yw, a0, a0s;
  // workspace
  Buf e, ex, ax, d1, d1y, fbar, planes, tx, ty, bsum, bw;
  const double* pos = nullptr;  // device [S][2] positions of the current call
  // Forward-to-backward retention (dlx_scene_forward_token / reuse_forward):
  // a forward that fits retain_limit keeps every chunk's D1 and Y.D1 (the
  // half-transformed fields, M x N per source and wavelength), so that the
  // backward starts from them instead of repeating the first GEMM; it still
  // recomputes the focal field from D1.
  Buf retain;  // per chunk: D1 [R L][M][N] then Y.D1 (chunk_bytes())
  size_t retain_limit = (size_t)48 << 30;
  unsigned long long epoch = 0, fwd_token = 0, reuse_req = 0;
  const void* fwd_in[6] = {};
  int fwd_S = 0;

  bool split() const { return variant == DLX_VARIANT_SPLIT_BF16; }

  void release() {
    for (Buf* b : {&alpha, &kf, &a_out, &b_out, &inv_fringe, &inv_lambda_ff, &xin, &yw, &a0,
                   &a0s, &e, &ex, &ax, &d1, &d1y, &fbar, &planes, &tx, &ty, &bsum, &bw,
                   &retain})
      b->release();
  }
  size_t footprint() const {
    size_t t = 0;
    for (const Buf* b : {&alpha, &kf, &a_out, &b_out, &inv_fringe, &inv_lambda_ff, &xin, &yw,
                         &a0, &a0s, &e, &ex, &ax, &d1, &d1y, &fbar, &planes, &tx, &ty, &bsum,
                         &bw, &retain})
      t += b->bytes;
    return t;
  }

  GemmArgs gemm(int batch, int Mg, int Ng, int K, const void* A, int a_div, const void* B,
                int b_div, const EpiArgs& e) const {
    GemmArgs g{};
    g.batch = batch; g.M = Mg; g.N = Ng; g.K = K;
    g.a_batch_div = a_div;
    g.b_batch_div = b_div;
    if (split()) {
      g.As = static_cast<const __nv_bfloat16*>(A);
      g.Bs = static_cast<const __nv_bfloat16*>(B);
    } else {
      g.A = static_cast<const float2*>(A);
      g.a_bs = (long long)Mg * K;
      g.B = static_cast<const float2*>(B);
      g.b_bs = (long long)Ng * K;
    }
    g.epi = e;
    return g;
  }
  int run(const GemmArgs& g, cudaStream_t s) const { return run_gemm_timed(variant, g, s); }
  EpiArgs epi(int kind, int Rc, const float* G = nullptr) const {
    EpiArgs e{};
    e.kind = kind;
    e.objs.n = Rc;
    for (int r = 0; r < Rc; ++r) e.objs.o[r].G = G;
    e.alpha = alpha.as<float>();
    e.kf = kf.as<float>();
    return e;
  }
  void set_out(EpiArgs& e, void* out) const {
    if (split()) e.out_split = static_cast<__nv_bfloat16*>(out);
    else e.out_c64 = static_cast<float2*>(out);
  }

  int build_field(const float* amp, const float* amp_scale, const float* opd, const float* phase,
                  cudaStream_t s) {
    const long long npix = (long long)N * N;
    scene_field_kernel<<<ceil_div(npix, 256), 256, 0, s>>>(
        N, L, ps_in, amp, amp_scale, opd, phase, inv_lambda_ff.as<float2>(),
        split() ? e.as<__nv_bfloat16>() : nullptr, split() ? ex.as<__nv_bfloat16>() : nullptr,
        split() ? nullptr : e.as<float2>(), split() ? nullptr : ex.as<float2>());
    DLX_LAUNCH_CHECK("scene_field_kernel");
    return DLX_OK;
  }

  // Tilt phasors of sources s0 .. s0 + Rc - 1 (positions already in `pos`) and
  // their x-axis matrices A'x. The y-axis tilt is applied by the first GEMM's
  // epilogue (EpiArgs::coltilt), so every second GEMM reads the shared A0.
  int build_matrices(int s0, int Rc, cudaStream_t s) {
    const int B = Rc * L;
    dim3 gt(ceil_div(N, 256), B);
    scene_tilt_kernel<<<gt, 256, 0, s>>>(N, Rc, xin.as<float2>(), inv_fringe.as<double>(),
                                         pos + 2 * s0, tx.as<float2>(), ty.as<float2>());
    DLX_LAUNCH_CHECK("scene_tilt_kernel");
    const long long mn = (long long)M * N;
    const int rg = 8;
    if (split() && N % 4 == 0) {
      dim3 grd(ceil_div(mn / 4, 256), L, ceil_div(Rc, rg));
      scene_ax_kernel<4><<<grd, 256, 0, s>>>(M, N, Rc, rg, a0.as<float2>(), tx.as<float2>(),
                                             ax.as<__nv_bfloat16>(), nullptr);
    } else {
      dim3 grd(ceil_div(mn, 256), L, ceil_div(Rc, rg));
      scene_ax_kernel<1><<<grd, 256, 0, s>>>(M, N, Rc, rg, a0.as<float2>(), tx.as<float2>(),
                                             split() ? ax.as<__nv_bfloat16>() : nullptr,
                                             split() ? nullptr : ax.as<float2>());
    }
    DLX_LAUNCH_CHECK("scene_ax_kernel");
    return DLX_OK;
  }
  // The shared y-axis matrix of every wavelength (A operand, batch divisor Rc).
  const void* ay0() const { return split() ? a0s.p : a0.p; }

  // one chunk of retained D1 and Y.D1 ([R L][M][N] each, split rows padded)
  size_t chunk_bytes() const { return 2 * split_bytes((long long)R * L, M, N); }
  void* keep_d1(int c) const { return retain.as<char>() + (size_t)c * chunk_bytes(); }
  void* keep_d1y(int c) const { return static_cast<char*>(keep_d1(c)) + chunk_bytes() / 2; }

  // Room for the retained fields of S sources: within retain_limit, and
  // allocated only outside stream capture (a capture runs without retention).
  bool ensure_retain(int S, cudaStream_t s) {
    const size_t need = (size_t)((S + R - 1) / R) * chunk_bytes();
    if (need == 0 || need > retain_limit) return false;
    if (retain.bytes >= need) return true;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (cs != cudaStreamCaptureStatusNone) return false;
    retain.release();
    return retain.alloc(need) == DLX_OK;  // out of memory: run without retention
  }

  // D1 (and, when d1y_out is set, Y.D1) of chunk s0 into the given buffers.
  int first_gemm(int Rc, void* d1_out, void* d1y_out, cudaStream_t s) {
    const int B = Rc * L;
    // D1[b][u][y] = sum_x A'x[b][u][x] E_l[y][x], times the y tilt ty[b][y]
    EpiArgs e1 = epi(d1y_out ? EPI_SPLIT2 : (split() ? EPI_SPLIT : EPI_C64), Rc);
    e1.alpha = nullptr;
    e1.coltilt = ty.as<float2>();
    if (d1y_out) {
      e1.colw = yw.as<float>();  // Y along the y index = GEMM column n
      if (split()) {
        e1.out_split = static_cast<__nv_bfloat16*>(d1_out);
        e1.out_split2 = static_cast<__nv_bfloat16*>(d1y_out);
      } else {
        e1.out_c64 = static_cast<float2*>(d1_out);
        e1.out_c642 = static_cast<float2*>(d1y_out);
      }
    } else {
      set_out(e1, d1_out);
    }
    return run(gemm(B, M, N, N, ax.p, 1, e.p, Rc, e1), s);
  }

  int forward(const float* amp, const float* amp_scale, const float* opd, const float* phase,
              const double* positions, const float* weights, int S, float* image, int accumulate,
              cudaStream_t s) {
    pos = positions;
    fwd_token = 0;
    const bool keep = ensure_retain(S, s);
    DLX_TRY(build_field(amp, amp_scale, opd, phase, s));
    for (int s0 = 0; s0 < S; s0 += R) {
      const int Rc = std::min(R, S - s0), B = Rc * L, c = s0 / R;
      DLX_TRY(build_matrices(s0, Rc, s));
      void* d1src = keep ? keep_d1(c) : d1.p;
      DLX_TRY(first_gemm(Rc, d1src, keep ? keep_d1y(c) : nullptr, s));
      // |F[b][v][u]|^2, F = alpha_l sum_y A0[l][v][y] D1[b][u][y]
      EpiArgs e2 = epi(EPI_INTENSITY, Rc);
      e2.out_f32 = planes.as<float>();
      DLX_TRY(run(gemm(B, M, M, N, ay0(), Rc, d1src, 1, e2), s));
      const long long npix = (long long)M * M;
      scene_image_kernel<<<ceil_div(npix, 256), 256, 0, s>>>(planes.as<float>(), Rc, L, npix,
                                                             weights, s0,
                                                             (s0 > 0 || accumulate) ? 1 : 0, image);
      DLX_LAUNCH_CHECK("scene_image_kernel");
    }
    if (keep) {
      fwd_token = ++epoch;
      const void* in[6] = {amp, amp_scale, opd, phase, positions, weights};
      std::copy(in, in + 6, fwd_in);
      fwd_S = S;
    }
    return DLX_OK;
  }

  bool can_reuse(unsigned long long req, const void* const in[6], int S) const {
    if (req == 0 || req != fwd_token || S != fwd_S) return false;
    for (int i = 0; i < 6; ++i)
      if (in[i] != fwd_in[i]) return false;
    return true;
  }

  int backward(const float* amp, const float* amp_scale, const float* opd, const float* phase,
               const double* positions, const float* weights, int S, const float* g_image,
               float* g_pos, float* g_w, cudaStream_t s) {
    const unsigned long long req = reuse_req;
    reuse_req = 0;  // a request covers one backward call
    const void* in[6] = {amp, amp_scale, opd, phase, positions, weights};
    const bool reuse = can_reuse(req, in, S);
    pos = positions;
    DLX_TRY(build_field(amp, amp_scale, opd, phase, s));
    const long long npix = (long long)M * M;
    for (int s0 = 0; s0 < S; s0 += R) {
      const int Rc = std::min(R, S - s0), B = Rc * L, c = s0 / R;
      DLX_TRY(build_matrices(s0, Rc, s));  // A'x is needed for D1X either way
      // D1 and D1Y = Y.D1, both y-tilted: retained by the forward, or recomputed
      const void* d1src = reuse ? keep_d1(c) : d1.p;
      const void* d1ysrc = reuse ? keep_d1y(c) : d1y.p;
      if (!reuse) DLX_TRY(first_gemm(Rc, d1.p, d1y.p, s));
      // intensity planes and F-bar = 2 w alpha G D
      EpiArgs e2 = epi(EPI_PSF_GRADF, Rc, g_image);
      e2.out_f32 = planes.as<float>();
      set_out(e2, fbar.p);
      // per-(source, wavelength) weight of the cotangent: w[s0 + r][l] at b = l Rc + r
      scene_gather_weights_kernel<<<ceil_div(B, 256), 256, 0, s>>>(weights, Rc, L, s0,
                                                                    bw.as<float>());
      DLX_LAUNCH_CHECK("scene_gather_weights_kernel");
      e2.bweight = bw.as<float>();
      DLX_TRY(run(gemm(B, M, M, N, ay0(), Rc, d1src, 1, e2), s));
      if (g_w) {
        scene_bsum_kernel<<<B, 256, 0, s>>>(planes.as<float>(), npix, g_image,
                                            bsum.as<double>());
        DLX_LAUNCH_CHECK("scene_bsum_kernel");
        scene_finish_kernel<<<ceil_div(Rc, 64), 64, 0, s>>>(bsum.as<double>(), Rc, L, s0, g_w,
                                                            nullptr, 0);
        DLX_LAUNCH_CHECK("scene_finish_kernel");
      }
      if (!g_pos) continue;
      // d/dty: k alpha Im-part of conj(F-bar) . (A'y (Y.D1)^T)
      EpiArgs ed = epi(EPI_DOT, Rc);
      ed.out_f32 = planes.as<float>();
      if (split()) ed.in_split = fbar.as<__nv_bfloat16>();
      else ed.in_c64 = fbar.as<float2>();
      DLX_TRY(run(gemm(B, M, M, N, ay0(), Rc, d1ysrc, 1, ed), s));
      DLX_TRY(pos_reduce(Rc, s0, g_pos, 1, s));
      // d/dtx: D1X = A'x (X.E)^T (into d1), then the same dot
      EpiArgs ex1 = epi(split() ? EPI_SPLIT : EPI_C64, Rc);
      ex1.alpha = nullptr;
      ex1.coltilt = ty.as<float2>();
      set_out(ex1, d1.p);
      DLX_TRY(run(gemm(B, M, N, N, ax.p, 1, ex.p, Rc, ex1), s));
      DLX_TRY(run(gemm(B, M, M, N, ay0(), Rc, d1.p, 1, ed), s));
      DLX_TRY(pos_reduce(Rc, s0, g_pos, 0, s));
    }
    return DLX_OK;
  }

  int pos_reduce(int Rc, int s0, float* g_pos, int axis, cudaStream_t s) {
    const long long npix = (long long)M * M;
    scene_bsum_kernel<<<Rc * L, 256, 0, s>>>(planes.as<float>(), npix, nullptr, bsum.as<double>());
    DLX_LAUNCH_CHECK("scene_bsum_kernel");
    scene_finish_kernel<<<ceil_div(Rc, 64), 64, 0, s>>>(bsum.as<double>(), Rc, L, s0, nullptr,
                                                        g_pos, axis);
    DLX_LAUNCH_CHECK("scene_finish_kernel");
    return DLX_OK;
  }
};

namespace {

int upload(Buf& b, const void* host, size_t bytes) {
  DLX_TRY(b.alloc(bytes));
  DLX_TRY_CUDA(cudaMemcpy(b.p, host, bytes, cudaMemcpyHostToDevice));
  return DLX_OK;
}

int scene_create(const dlx_scene_desc* d, const double* wl, dlx_scene_plan_s* p) {
  const int L = d->n_wavelengths, N = d->n_in, M = d->n_out, R = d->max_sources;
  p->L = L; p->N = N; p->M = M; p->R = R; p->variant = d->variant;
  p->ps_in = d->pixel_scale_in; p->ps_out = d->pixel_scale_out;
  p->focal = d->focal_length > 0 ? d->focal_length : 0.0;
  p->wl.assign(wl, wl + L);
  std::vector<float> alpha(L), kf(L);
  std::vector<double> a_out(L), b_out(L), invf(L);
  std::vector<float2> ilff(L);
  for (int l = 0; l < L; ++l) {
    const double lam = wl[l];
    const double fringe = lam / (p->ps_in * N);
    double s_out = p->ps_out / fringe;
    if (p->focal > 0) s_out /= p->focal;
    a_out[l] = s_out;
    b_out[l] = -0.5 * (M - 1) * s_out;
    invf[l] = 1.0 / fringe;   // tilt (rad) -> output-coordinate shift
    double out_size = M * p->ps_out;
    if (p->focal > 0) out_size /= p->focal;
    alpha[l] = (float)((out_size / fringe) / ((double)N * (double)M));
    kf[l] = (float)(2.0 * M_PI / lam);
    const FF f = ff_from_double(1.0 / lam);
    ilff[l] = make_float2(f.hi, f.lo);
  }
  std::vector<float> yw(N);
  for (int i = 0; i < N; ++i) yw[i] = (float)(((double)i - 0.5 * (N - 1)) * p->ps_in);
  DLX_TRY(upload(p->alpha, alpha.data(), sizeof(float) * L));
  DLX_TRY(upload(p->kf, kf.data(), sizeof(float) * L));
  DLX_TRY(upload(p->a_out, a_out.data(), sizeof(double) * L));
  DLX_TRY(upload(p->b_out, b_out.data(), sizeof(double) * L));
  DLX_TRY(upload(p->inv_fringe, invf.data(), sizeof(double) * L));
  DLX_TRY(upload(p->inv_lambda_ff, ilff.data(), sizeof(float2) * L));
  DLX_TRY(upload(p->yw, yw.data(), sizeof(float) * N));
  DLX_TRY(p->xin.alloc(sizeof(float2) * N));
  scene_xtable_kernel<<<ceil_div(N, 256), 256>>>(N, 1.0 / N, -0.5 * (N - 1) / N,
                                                 p->xin.as<float2>());
  DLX_LAUNCH_CHECK("scene_xtable_kernel");
  const size_t B = (size_t)R * L, nn = (size_t)N * N, mn = (size_t)M * N, mm = (size_t)M * M;
  DLX_TRY(p->a0.alloc(L * mn * sizeof(float2)));
  if (p->split()) DLX_TRY(p->a0s.alloc(split_bytes(L, M, N)));
  scene_a0_kernel<<<dim3(ceil_div((long long)mn, 256), L), 256>>>(
      M, N, p->xin.as<float2>(), p->a_out.as<double>(), p->b_out.as<double>(),
      p->a0.as<float2>(), p->split() ? p->a0s.as<__nv_bfloat16>() : nullptr);
  DLX_LAUNCH_CHECK("scene_a0_kernel");
  // complex64, or split planes with padded rows (at least as large)
  DLX_TRY(p->e.alloc(split_bytes(L, N, N)));
  DLX_TRY(p->ex.alloc(split_bytes(L, N, N)));
  DLX_TRY(p->ax.alloc(split_bytes(B, M, N)));
  DLX_TRY(p->d1.alloc(split_bytes(B, M, N)));
  DLX_TRY(p->d1y.alloc(split_bytes(B, M, N)));
  DLX_TRY(p->fbar.alloc(split_bytes(B, M, M)));
  DLX_TRY(p->planes.alloc(B * mm * sizeof(float)));
  DLX_TRY(p->tx.alloc(B * N * sizeof(float2)));
  DLX_TRY(p->ty.alloc(B * N * sizeof(float2)));
  DLX_TRY(p->bsum.alloc(B * sizeof(double)));
  DLX_TRY(p->bw.alloc(B * sizeof(float)));
  DLX_TRY_CUDA(cudaDeviceSynchronize());
  return DLX_OK;
}

}  // namespace

extern "C" {

int dlx_scene_plan_create(const dlx_scene_desc* d, const double* wavelengths,
                          dlx_scene_plan* plan) {
  if (!d || !wavelengths || !plan) return fail(DLX_ERR_ARG, "scene_plan_create: null pointer");
  *plan = nullptr;
  if (d->n_wavelengths <= 0 || d->n_in <= 0 || d->n_out <= 0)
    return fail(DLX_ERR_SHAPE, "scene_plan_create: sizes must be positive");
  if (d->max_sources <= 0 || d->max_sources > kMaxObj)
    return fail(DLX_ERR_ARG, "scene_plan_create: max_sources must lie in [1, " +
                                 std::to_string(kMaxObj) + "]");
  if (!(d->pixel_scale_in > 0) || !(d->pixel_scale_out > 0))
    return fail(DLX_ERR_ARG, "scene_plan_create: pixel scales must be positive");
  DLX_TRY(check_focal(d->focal_length, "scene_plan_create"));
  if (d->variant != DLX_VARIANT_FP32 && d->variant != DLX_VARIANT_SPLIT_BF16)
    return fail(DLX_ERR_ARG, "scene_plan_create: unknown variant");
  if (d->variant == DLX_VARIANT_SPLIT_BF16) {
    if (!tc_supported())
      return fail(DLX_ERR_UNSUPPORTED, "the split-BF16 form needs an sm_103a (GB300) device");
  }
  auto* p = new (std::nothrow) dlx_scene_plan_s();
  if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
  const int st = scene_create(d, wavelengths, p);
  if (st != DLX_OK) {
    p->release();
    delete p;
    return st;
  }
  *plan = p;
  return DLX_OK;
}

int dlx_scene_plan_destroy(dlx_scene_plan plan) {
  if (!plan) return DLX_OK;
  cudaDeviceSynchronize();
  plan->release();
  delete plan;
  return DLX_OK;
}

int dlx_scene_plan_footprint(dlx_scene_plan plan, size_t* bytes) {
  if (!plan || !bytes) return fail(DLX_ERR_ARG, "scene_plan_footprint: null pointer");
  *bytes = plan->footprint();
  return DLX_OK;
}

int dlx_scene_forward(dlx_scene_plan plan, const float* amp, const float* amp_scale,
                      const float* opd, const float* phase, const double* positions,
                      const float* weights, int n_sources, float* image, int accumulate,
                      void* stream) {
  if (!plan || !positions || !weights || !image)
    return fail(DLX_ERR_ARG, "scene_forward: null pointer");
  if (n_sources <= 0) return fail(DLX_ERR_ARG, "scene_forward: n_sources must be positive");
  return plan->forward(amp, amp_scale, opd, phase, positions, weights, n_sources, image,
                       accumulate, static_cast<cudaStream_t>(stream));
}

int dlx_scene_forward_token(dlx_scene_plan plan, unsigned long long* token) {
  if (!plan || !token) return fail(DLX_ERR_ARG, "scene_forward_token: null pointer");
  *token = plan->fwd_token;
  return DLX_OK;
}

int dlx_scene_reuse_forward(dlx_scene_plan plan, unsigned long long token) {
  if (!plan) return fail(DLX_ERR_ARG, "scene_reuse_forward: null plan");
  plan->reuse_req = token;
  return DLX_OK;
}

int dlx_scene_set_retain_limit(dlx_scene_plan plan, size_t bytes) {
  if (!plan) return fail(DLX_ERR_ARG, "scene_set_retain_limit: null plan");
  cudaDeviceSynchronize();
  plan->retain_limit = bytes;
  plan->fwd_token = 0;
  if (plan->retain.bytes > bytes) plan->retain.release();
  return DLX_OK;
}

int dlx_scene_backward(dlx_scene_plan plan, const float* amp, const float* amp_scale,
                       const float* opd, const float* phase, const double* positions,
                       const float* weights, int n_sources, const float* g_image, float* g_pos,
                       float* g_weights, void* stream) {
  if (!plan || !positions || !weights || !g_image)
    return fail(DLX_ERR_ARG, "scene_backward: null pointer");
  if (n_sources <= 0) return fail(DLX_ERR_ARG, "scene_backward: n_sources must be positive");
  return plan->backward(amp, amp_scale, opd, phase, positions, weights, n_sources, g_image,
                        g_pos, g_weights, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
