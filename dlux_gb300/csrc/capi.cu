// capi.cu -- the extern "C" entry points declared in include/dluxgb.h, the
// plan objects that own cached DFT matrices and intermediate buffers, and the
// orchestration of the two-step MFT:
//
//   forward   D1[u][y] = sum_x AxT[u][x] E[y][x]          (contract x)
//             F[v][u]  = alpha * sum_y AyT[v][y] D1[u][y]  (contract y)
//   adjoint   Xt[x][v] = sum_u conj(Ax[x][u]) Fbar[v][u]
//             Ebar[y][x] = alpha * sum_v conj(Ay[y][v]) Xt[x][v]
//
// where Ax[x][u] is dLux's transfer_matrix (utils/propagation.py:67-127) and
// AxT its transpose. Every GEMM is "D = A * B^T" with both operands
// K-contiguous, so all stores are row-major and coalesced.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"

namespace dlx {

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void set_error(const std::string& msg) { g_err = msg; }
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int check_cuda(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return DLX_ERR_CUDA;
}

int current_device(int* dev) {
  DLX_TRY_CUDA(cudaGetDevice(dev));
  if (*dev < 0 || *dev >= kMaxDevices)
    return fail(DLX_ERR_UNSUPPORTED, "device index " + std::to_string(*dev) +
                                         " is beyond the library's per-device tables");
  return DLX_OK;
}

int check_focal(double focal_length, const char* who) {
  if (focal_length >= 0) return DLX_OK;
  return fail(DLX_ERR_ARG, std::string(who) +
                               ": focal_length must be positive (0 selects the angular form)");
}

static std::atomic<int> g_sm_count[kMaxDevices];
int device_sm_count(int* sms) {
  int dev = 0;
  DLX_TRY(current_device(&dev));
  int n = g_sm_count[dev].load();
  if (n <= 0) {
    DLX_TRY_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    if (n <= 0) return fail(DLX_ERR_CUDA, "device reports no multiprocessors");
    g_sm_count[dev].store(n);
  }
  *sms = n;
  return DLX_OK;
}

namespace {

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// dLux transfer_matrix axis (utils/propagation.py:67-127), FP64.
DftAxis mft_axis(double wl, int n_in, double ps_in, int n_out, double ps_out, double shift,
                 double focal, bool inverse) {
  DftAxis a{};
  const double fringe = wl / (ps_in * n_in);
  double s_out = ps_out / fringe;
  if (focal > 0) s_out /= focal;
  a.a_in = 1.0 / n_in;
  a.b_in = -(0.5 * (n_in - 1) + shift) / n_in;
  a.a_out = s_out;
  a.b_out = -(0.5 * (n_out - 1) + shift) * s_out;
  a.sigma = inverse ? 1.0 : -1.0;
  a.scale = 1.0;
  return a;
}

// nfringes / (N_in N_out) (utils/propagation.py:130-175, 246-254), FP64.
double mft_alpha(double wl, int n_in, double ps_in, int n_out, double ps_out, double focal) {
  double out_size = n_out * ps_out;
  if (focal > 0) out_size /= focal;
  const double nfringes = out_size / (wl / (n_in * ps_in));
  return nfringes / ((double)n_in * (double)n_out);
}

// fft_spec (utils/fourier.py:14-45): output pixel scale and centre.
void fft_spec(int n, double ps, double wl, double focal, double* d, double* c) {
  double d_out = wl / (n * ps);
  if (focal > 0) d_out *= focal;
  *d = d_out;
  *c = (n % 2 != 0) ? 0.0 : -0.5 * d_out;
}

// Output side of dLux's padded FFT: N zero-padded by (N (pad - 1)) // 2 on
// each side (utils/propagation.py:52-53), i.e. N pad, or N pad - 1 when
// N (pad - 1) is odd.
int fft_out_side(int n_in, int pad) { return n_in + 2 * ((n_in * (pad - 1)) / 2); }

// One axis of the padded centred FFT (utils/propagation.py:8-64) with the
// propagate_FFT ramps (wavefronts.py:683-712, utils/fourier.py:48-78).
DftAxis fft_axis(const dlx_fft_desc& d, double wl) {
  DftAxis a{};
  const int N = d.n_in, P = fft_out_side(d.n_in, d.pad);
  const int npad = (N * (d.pad - 1)) / 2;
  const int c = P / 2;
  a.a_in = 1.0;
  a.b_in = (double)(npad - c);
  a.a_out = 1.0 / P;
  a.b_out = -(double)c / P;
  a.sigma = d.inverse ? 1.0 : -1.0;
  a.scale = 1.0;
  if (d.apply_ramps) {
    const double f = d.focal_length > 0 ? d.focal_length : 0.0;
    const double alpha = f > 0 ? wl * f : wl;
    const double sign = d.inverse ? -1.0 : 1.0;
    double d_fft, c_fft;
    fft_spec(P, d.pixel_scale_in, wl, f, &d_fft, &c_fft);
    const double shift_in = c_fft - d.center_out;
    a.g_in = sign * shift_in * d.pixel_scale_in / alpha;
    a.d_in = sign * shift_in / alpha * (d.center_in - 0.5 * (N - 1) * d.pixel_scale_in);
    double d2, shift_out;
    fft_spec(P, d_fft, wl, f, &d2, &shift_out);
    a.g_out = sign * shift_out * d_fft / alpha;
    a.d_out = sign * shift_out / alpha * (d.center_out - 0.5 * (P - 1) * d_fft);
  }
  return a;
}

// Device buffer owned by a plan.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool owned = true;  // false: a view into caller-provided workspace
  void view(void* ptr, size_t n) {
    release();
    p = ptr;
    bytes = n;
    owned = false;
  }
  int alloc(size_t n) {
    owned = true;
    if (n == 0) return DLX_OK;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return fail(DLX_ERR_NOMEM, std::string("cudaMalloc of ") + std::to_string(n) +
                                     " bytes failed: " + cudaGetErrorString(e));
    }
    bytes = n;
    return DLX_OK;
  }
  void release() {
    if (p && owned) cudaFree(p);
    p = nullptr;
    bytes = 0;
    owned = true;
  }
  size_t owned_bytes() const { return owned ? bytes : 0; }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

// Cached transfer matrices of a batch of two-step transforms.
struct TwoStep {
  int batch = 0, n_in = 0, n_out = 0, variant = 0;
  bool shared_xy = true;
  // c64 matrices (FP32 form) or split matrices (tensor-core form).
  DevBuf atx, aty, anx, any;   // T layout [b][n_out][n_in], N layout [b][n_in][n_out]
  DevBuf alpha;                // float [b]
  DevBuf inv_lambda, kvec;     // double [b]
  DevBuf inv_lambda_ff;        // float2 [b]: 1/lambda as a (hi, lo) pair
  std::vector<double> wl;

  // T layout (rows n_out, cols n_in) or N layout (rows n_in, cols n_out); split
  // matrices have padded rows (split_ld).
  size_t mat_bytes(bool t_layout) const {
    const int rows = t_layout ? n_out : n_in, cols = t_layout ? n_in : n_out;
    if (variant == DLX_VARIANT_SPLIT_BF16) return split_bytes(batch, rows, cols);
    return (size_t)batch * rows * cols * sizeof(float2);
  }

  // The tensor-core form streams cached split DFT matrices through TMA, or
  // (operand_mode 1) builds the DFT operand inside the GEMM from `axes`: no
  // cached matrices and half the operand bytes, but measured slower at 512^3
  // (0.52 vs 0.36 ms per launch); it suits plans that must stay small.
  bool gen_a = false;
  DevBuf axes;                 // DftAxis [2][b]: x axes then y axes (kept on the device)

  struct AOp {
    const void* mat;
    const DftAxis* axes;
    bool rows_out;
  };
  AOp opATx() const { return {atx.p, axes.as<DftAxis>(), true}; }
  AOp opANx() const { return {anx.p, axes.as<DftAxis>(), false}; }
  AOp opATy() const { return {ATy(), axes.as<DftAxis>() + (shared_xy ? 0 : batch), true}; }
  AOp opANy() const { return {ANy(), axes.as<DftAxis>() + (shared_xy ? 0 : batch), false}; }

  int build(const std::vector<DftAxis>& ax_x, const std::vector<DftAxis>& ax_y,
            const std::vector<float>& alphas, bool generate_operand = false) {
    shared_xy = std::memcmp(ax_x.data(), ax_y.data(), sizeof(DftAxis) * batch) == 0;
    // The in-CTA generator assumes a phase affine along K: no quadratic terms.
    bool affine = true;
    for (int b = 0; b < batch; ++b)
      affine = affine && ax_x[b].q_in == 0.0 && ax_x[b].q_out == 0.0 &&
               ax_y[b].q_in == 0.0 && ax_y[b].q_out == 0.0;
    gen_a = variant == DLX_VARIANT_SPLIT_BF16 && generate_operand && affine;
    DLX_TRY(axes.alloc(sizeof(DftAxis) * batch * 2));
    int st = DLX_OK;
    do {
      cudaError_t e = cudaMemcpy(axes.p, ax_x.data(), sizeof(DftAxis) * batch,
                                 cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(axes.as<DftAxis>() + batch, ax_y.data(), sizeof(DftAxis) * batch,
                       cudaMemcpyHostToDevice);
      if (e != cudaSuccess) { st = check_cuda(e, "cudaMemcpy(axes)"); break; }
      if (!gen_a) {
        if ((st = atx.alloc(mat_bytes(true))) != DLX_OK) break;
        if ((st = anx.alloc(mat_bytes(false))) != DLX_OK) break;
        if (!shared_xy) {
          if ((st = aty.alloc(mat_bytes(true))) != DLX_OK) break;
          if ((st = any.alloc(mat_bytes(false))) != DLX_OK) break;
        }
        const bool split = variant == DLX_VARIANT_SPLIT_BF16;
        auto gen = [&](DevBuf& buf, const DftAxis* ax, bool t_layout) {
          const int rows = t_layout ? n_out : n_in, cols = t_layout ? n_in : n_out;
          return launch_dft_gen(ax, batch, rows, cols, t_layout,
                                split ? nullptr : buf.as<float2>(), (long long)rows * cols,
                                split ? buf.as<__nv_bfloat16>() : nullptr, 0);
        };
        if ((st = gen(atx, axes.as<DftAxis>(), true)) != DLX_OK) break;
        if ((st = gen(anx, axes.as<DftAxis>(), false)) != DLX_OK) break;
        if (!shared_xy) {
          if ((st = gen(aty, axes.as<DftAxis>() + batch, true)) != DLX_OK) break;
          if ((st = gen(any, axes.as<DftAxis>() + batch, false)) != DLX_OK) break;
        }
      }
      if ((st = alpha.alloc(sizeof(float) * batch)) != DLX_OK) break;
      e = cudaMemcpy(alpha.p, alphas.data(), sizeof(float) * batch, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) { st = check_cuda(e, "cudaMemcpy(alpha)"); break; }
      std::vector<double> il(batch), kv(batch);
      for (int b = 0; b < batch; ++b) {
        il[b] = 1.0 / wl[b];
        kv[b] = 2.0 * M_PI / wl[b];
      }
      std::vector<float2> ilff(batch);
      for (int b = 0; b < batch; ++b) {
        const FF f = ff_from_double(il[b]);
        ilff[b] = make_float2(f.hi, f.lo);
      }
      if ((st = inv_lambda.alloc(sizeof(double) * batch)) != DLX_OK) break;
      if ((st = inv_lambda_ff.alloc(sizeof(float2) * batch)) != DLX_OK) break;
      if ((st = kvec.alloc(sizeof(double) * batch)) != DLX_OK) break;
      e = cudaMemcpy(inv_lambda.p, il.data(), sizeof(double) * batch, cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(inv_lambda_ff.p, ilff.data(), sizeof(float2) * batch,
                       cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(kvec.p, kv.data(), sizeof(double) * batch, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) { st = check_cuda(e, "cudaMemcpy(lambda)"); break; }
      e = cudaDeviceSynchronize();
      if (e != cudaSuccess) { st = check_cuda(e, "transfer-matrix generation"); break; }
    } while (0);
    return st;
  }
  const void* ATy() const { return shared_xy ? atx.p : aty.p; }
  const void* ANy() const { return shared_xy ? anx.p : any.p; }
  void release() {
    atx.release(); aty.release(); anx.release(); any.release();
    alpha.release(); inv_lambda.release(); kvec.release(); inv_lambda_ff.release();
    axes.release();
  }
  size_t footprint() const {
    return atx.bytes + aty.bytes + anx.bytes + any.bytes + alpha.bytes + inv_lambda.bytes +
           inv_lambda_ff.bytes + kvec.bytes + axes.bytes;
  }
};

int validate_variant(int variant) {
  if (variant == DLX_VARIANT_FP32) return DLX_OK;
  if (variant == DLX_VARIANT_SPLIT_BF16) {
    if (!tc_supported())
      return fail(DLX_ERR_UNSUPPORTED,
                  "the split-BF16 tensor-core form needs an sm_103a (GB300) device");
    return DLX_OK;
  }
  return fail(DLX_ERR_ARG, "variant must be DLX_VARIANT_FP32 or DLX_VARIANT_SPLIT_BF16");
}

// Optional CUDA-event timing of every GEMM launch (dlx_gemm_timing_*), used
// to measure the dominant kernel inside a timed region on its own stream.
struct GemmTiming {
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  double flops = 0.0;  // algorithmic complex-GEMM flops of the recorded launches
};
GemmTiming g_timing;

int run_gemm(int variant, const GemmArgs& g, cudaStream_t s) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (g_timing.on) {
    DLX_TRY_CUDA(cudaEventCreate(&a));
    DLX_TRY_CUDA(cudaEventCreate(&b));
    DLX_TRY_CUDA(cudaEventRecord(a, s));
  }
  int st = variant == DLX_VARIANT_SPLIT_BF16 ? launch_gemm_tc(g, s) : launch_gemm_fp32(g, s);
  if (g_timing.on) {
    DLX_TRY_CUDA(cudaEventRecord(b, s));
    g_timing.ev.emplace_back(a, b);
    g_timing.flops += 8.0 * g.batch * (double)g.M * g.N * g.K;
  }
  return st;
}

GemmArgs gemm_c64(int batch, int M, int N, int K, const void* A, bool conj_a, const void* B,
                  const EpiArgs& epi) {
  GemmArgs g{};
  g.batch = batch; g.M = M; g.N = N; g.K = K;
  g.A = reinterpret_cast<const float2*>(A);
  g.a_bs = (long long)M * K;
  g.B = reinterpret_cast<const float2*>(B);
  g.b_bs = (long long)N * K;
  g.conj_a = conj_a;
  g.a_batch_div = 1;
  g.epi = epi;
  return g;
}

GemmArgs gemm_split(int batch, int M, int N, int K, const void* A, bool conj_a, const void* B,
                    const EpiArgs& epi) {
  GemmArgs g{};
  g.batch = batch; g.M = M; g.N = N; g.K = K;
  g.As = reinterpret_cast<const __nv_bfloat16*>(A);
  g.Bs = reinterpret_cast<const __nv_bfloat16*>(B);
  g.conj_a = conj_a;
  g.a_batch_div = 1;
  g.epi = epi;
  return g;
}

// A is a cached DFT matrix of the plan (op.mat) or, in the tensor-core form
// with generated operands, its axis description (op.axes).
GemmArgs gemm_for(int variant, int batch, int M, int N, int K, const TwoStep::AOp& op,
                  bool conj_a, const void* B, const EpiArgs& epi) {
  if (variant != DLX_VARIANT_SPLIT_BF16) return gemm_c64(batch, M, N, K, op.mat, conj_a, B, epi);
  GemmArgs g = gemm_split(batch, M, N, K, op.mat, conj_a, B, epi);
  if (!op.mat) {
    g.a_axes = op.axes;
    g.a_rows_are_out = op.rows_out;
  }
  return g;
}

EpiArgs epi_store(int variant, void* out, const float* alpha) {
  EpiArgs e{};
  e.alpha = alpha;
  if (variant == DLX_VARIANT_SPLIT_BF16) {
    e.kind = EPI_SPLIT;
    e.out_split = reinterpret_cast<__nv_bfloat16*>(out);
  } else {
    e.kind = EPI_C64;
    e.out_c64 = reinterpret_cast<float2*>(out);
  }
  return e;
}

EpiArgs epi_c64(void* out, const float* alpha) {
  EpiArgs e{};
  e.kind = EPI_C64;
  e.alpha = alpha;
  e.out_c64 = reinterpret_cast<float2*>(out);
  return e;
}

}  // namespace

// The GEMM launcher of every plan type, with the optional per-launch timing.
int run_gemm_timed(int variant, const GemmArgs& g, cudaStream_t s) { return run_gemm(variant, g, s); }

}  // namespace dlx

using namespace dlx;

// ---------------------------------------------------------------------------
// Generic two-step transform plan (MFT and FFT share it).
// ---------------------------------------------------------------------------
struct TwoStepPlan {
  TwoStep ts;
  DevBuf in_split;   // [b][4][n_in][n_in]   (split form: converted input)
  DevBuf mid;        // [b][n_out][n_in] (forward) / [b][n_in][n_out] (adjoint) intermediate
  DevBuf gout_split; // [b][4][n_out][n_out] (split form: converted cotangent)

  int alloc_buffers() {
    const size_t b = ts.batch, ni = ts.n_in, no = ts.n_out;
    if (ts.variant == DLX_VARIANT_SPLIT_BF16) {
      // split planes with padded rows: D1 [b][4][n_out][n_in], Xt [b][4][n_in][n_out]
      const size_t m1 = split_bytes(b, ts.n_out, ts.n_in), m2 = split_bytes(b, ts.n_in, ts.n_out);
      DLX_TRY(mid.alloc(m1 > m2 ? m1 : m2));
      DLX_TRY(in_split.alloc(split_bytes(b, ts.n_in, ts.n_in)));
      DLX_TRY(gout_split.alloc(split_bytes(b, ts.n_out, ts.n_out)));
    } else {
      DLX_TRY(mid.alloc(b * ni * no * 8));
    }
    return DLX_OK;
  }
  int forward(const void* in, void* out, cudaStream_t s) {
    const int B = ts.batch, N = ts.n_in, M = ts.n_out, v = ts.variant;
    const void* field = in;
    if (v == DLX_VARIANT_SPLIT_BF16) {
      DLX_TRY(launch_c64_to_split_batched(reinterpret_cast<const float2*>(in), N, N, B,
                                          in_split.as<__nv_bfloat16>(), s));
      field = in_split.p;
    }
    // D1[u][y] = sum_x AxT[u][x] E[y][x]
    DLX_TRY(run_gemm(v, gemm_for(v, B, M, N, N, ts.opATx(), false, field,
                                 epi_store(v, mid.p, nullptr)), s));
    // F[v][u] = alpha sum_y AyT[v][y] D1[u][y]
    DLX_TRY(run_gemm(v, gemm_for(v, B, M, M, N, ts.opATy(), false, mid.p,
                                 epi_c64(out, ts.alpha.as<float>())), s));
    return DLX_OK;
  }
  int adjoint(const void* gout, void* gin, cudaStream_t s) {
    const int B = ts.batch, N = ts.n_in, M = ts.n_out, v = ts.variant;
    const void* g = gout;
    if (v == DLX_VARIANT_SPLIT_BF16) {
      DLX_TRY(launch_c64_to_split_batched(reinterpret_cast<const float2*>(gout), M, M, B,
                                          gout_split.as<__nv_bfloat16>(), s));
      g = gout_split.p;
    }
    // Xt[x][v] = sum_u conj(Ax[x][u]) Fbar[v][u]
    DLX_TRY(run_gemm(v, gemm_for(v, B, N, M, M, ts.opANx(), true, g,
                                 epi_store(v, mid.p, nullptr)), s));
    // Ebar[y][x] = alpha sum_v conj(Ay[y][v]) Xt[x][v]
    DLX_TRY(run_gemm(v, gemm_for(v, B, N, N, M, ts.opANy(), true, mid.p,
                                 epi_c64(gin, ts.alpha.as<float>())), s));
    return DLX_OK;
  }
  void release() {
    ts.release();
    in_split.release();
    mid.release();
    gout_split.release();
  }
};

struct dlx_mft_plan_s {
  TwoStepPlan p;
};
struct dlx_fft_plan_s {
  TwoStepPlan p;
  bool radix = false;  // DLX_VARIANT_RADIX: line FFTs instead of the DFT-GEMM pair
  RadixFft rf;
};

extern "C" {

const char* dlx_last_error(void) { return g_err.c_str(); }
int dlx_version(void) { return 100; }
long long dlx_launch_count(void) { return g_launches.load(); }

int dlx_gemm_timing_begin(void) {
  for (auto& p : g_timing.ev) {
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  g_timing.ev.clear();
  g_timing.flops = 0.0;
  g_timing.on = true;
  return DLX_OK;
}

int dlx_gemm_timing_end(double* total_ms, int* launches, double* flops) {
  g_timing.on = false;
  double t = 0.0;
  int st = DLX_OK;
  for (auto& p : g_timing.ev) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(p.second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, p.first, p.second);
    if (e != cudaSuccess && st == DLX_OK) st = check_cuda(e, "gemm timing");
    t += ms;
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  if (total_ms) *total_ms = t;
  if (launches) *launches = (int)g_timing.ev.size();
  if (flops) *flops = g_timing.flops;
  g_timing.ev.clear();
  g_timing.flops = 0.0;
  return st;
}

int dlx_transfer_matrix(const double* wavelengths_host, int batch, int n_in,
                        double pixel_scale_in, int n_out, double pixel_scale_out, double shift,
                        double focal_length, int inverse, int transpose, void* out_c64,
                        void* stream) {
  if (batch < 0 || n_in <= 0 || n_out <= 0)
    return fail(DLX_ERR_SHAPE, "transfer_matrix: batch >= 0, n_in > 0 and n_out > 0 required");
  if (batch == 0) return DLX_OK;
  if (!wavelengths_host || !out_c64) return fail(DLX_ERR_ARG, "transfer_matrix: null pointer");
  DLX_TRY(check_focal(focal_length, "transfer_matrix"));
  cudaStream_t s = as_stream(stream);
  std::vector<DftAxis> ax(batch);
  for (int b = 0; b < batch; ++b) {
    if (!(wavelengths_host[b] > 0))
      return fail(DLX_ERR_ARG, "transfer_matrix: wavelengths must be positive");
    ax[b] = mft_axis(wavelengths_host[b], n_in, pixel_scale_in, n_out, pixel_scale_out, shift,
                     focal_length, inverse != 0);
  }
  DftAxis* dev = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&dev, sizeof(DftAxis) * batch, s));
  cudaError_t e = cudaMemcpyAsync(dev, ax.data(), sizeof(DftAxis) * batch,
                                  cudaMemcpyHostToDevice, s);
  int st = (e == cudaSuccess) ? DLX_OK : check_cuda(e, "cudaMemcpyAsync(axes)");
  if (st == DLX_OK) {
    const bool t = transpose != 0;
    st = launch_dft_gen(dev, batch, t ? n_out : n_in, t ? n_in : n_out, t,
                        reinterpret_cast<float2*>(out_c64), (long long)n_in * n_out, nullptr, s);
  }
  // The host vector must outlive the copy: wait for it before returning.
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFreeAsync(dev, s);
  if (st == DLX_OK && e2 != cudaSuccess) st = check_cuda(e2, "transfer_matrix");
  return st;
}

// ---- MFT plan ---------------------------------------------------------------
int dlx_mft_plan_create(const dlx_mft_desc* d, const double* wl, dlx_mft_plan* plan) {
  if (!d || !wl || !plan) return fail(DLX_ERR_ARG, "mft_plan_create: null pointer");
  *plan = nullptr;
  if (d->batch <= 0 || d->n_in <= 0 || d->n_out <= 0)
    return fail(DLX_ERR_SHAPE, "mft_plan_create: batch, n_in and n_out must be positive");
  if (!(d->pixel_scale_in > 0) || !(d->pixel_scale_out > 0))
    return fail(DLX_ERR_ARG, "mft_plan_create: pixel scales must be positive");
  DLX_TRY(check_focal(d->focal_length, "mft_plan_create"));
  DLX_TRY(validate_variant(d->variant));
  auto* p = new (std::nothrow) dlx_mft_plan_s();
  if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
  TwoStep& ts = p->p.ts;
  ts.batch = d->batch; ts.n_in = d->n_in; ts.n_out = d->n_out; ts.variant = d->variant;
  ts.wl.assign(wl, wl + d->batch);
  std::vector<DftAxis> ax(d->batch), ay(d->batch);
  std::vector<float> alphas(d->batch);
  for (int b = 0; b < d->batch; ++b) {
    if (!(wl[b] > 0)) {
      delete p;
      return fail(DLX_ERR_ARG, "mft_plan_create: wavelengths must be positive");
    }
    ax[b] = mft_axis(wl[b], d->n_in, d->pixel_scale_in, d->n_out, d->pixel_scale_out, d->shift_x,
                     d->focal_length, d->inverse != 0);
    ay[b] = mft_axis(wl[b], d->n_in, d->pixel_scale_in, d->n_out, d->pixel_scale_out, d->shift_y,
                     d->focal_length, d->inverse != 0);
    alphas[b] = (float)mft_alpha(wl[b], d->n_in, d->pixel_scale_in, d->n_out, d->pixel_scale_out,
                                 d->focal_length);
  }
  int st = ts.build(ax, ay, alphas);
  if (st == DLX_OK) st = p->p.alloc_buffers();
  if (st != DLX_OK) {
    p->p.release();
    delete p;
    return st;
  }
  *plan = p;
  return DLX_OK;
}

int dlx_mft_plan_destroy(dlx_mft_plan plan) {
  if (!plan) return DLX_OK;
  cudaDeviceSynchronize();
  plan->p.release();
  delete plan;
  return DLX_OK;
}

int dlx_mft_forward(dlx_mft_plan plan, const void* in, void* out, void* stream) {
  if (!plan || !in || !out) return fail(DLX_ERR_ARG, "mft_forward: null pointer");
  return plan->p.forward(in, out, as_stream(stream));
}

int dlx_mft_adjoint(dlx_mft_plan plan, const void* gout, void* gin, void* stream) {
  if (!plan || !gout || !gin) return fail(DLX_ERR_ARG, "mft_adjoint: null pointer");
  return plan->p.adjoint(gout, gin, as_stream(stream));
}

// ---- FFT plan ---------------------------------------------------------------
int dlx_fft_plan_create(const dlx_fft_desc* d, const double* wl, dlx_fft_plan* plan) {
  if (!d || !wl || !plan) return fail(DLX_ERR_ARG, "fft_plan_create: null pointer");
  *plan = nullptr;
  if (d->batch <= 0 || d->n_in <= 0 || d->pad <= 0)
    return fail(DLX_ERR_SHAPE, "fft_plan_create: batch, n_in and pad must be positive");
  if (!(d->pixel_scale_in > 0)) return fail(DLX_ERR_ARG, "fft_plan_create: pixel scale <= 0");
  DLX_TRY(check_focal(d->focal_length, "fft_plan_create"));
  if (d->apply_ramps && fft_out_side(d->n_in, d->pad) != d->n_in * d->pad)
    return fail(DLX_ERR_SHAPE, "fft_plan_create: the output phase ramps span n_in * pad "
                               "pixels, but the padded FFT of an odd n_in (pad - 1) has one "
                               "fewer");
  if (d->variant == DLX_VARIANT_RADIX) {
    if (fft_out_side(d->n_in, d->pad) != d->n_in * d->pad)
      return fail(DLX_ERR_SHAPE, "fft_plan_create: the radix form needs n_in (pad - 1) even");
    auto* p = new (std::nothrow) dlx_fft_plan_s();
    if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
    p->radix = true;
    std::vector<DftAxis> ax(d->batch);
    std::vector<float> alphas(d->batch, 1.0f / (float)fft_out_side(d->n_in, d->pad));
    for (int b = 0; b < d->batch; ++b) {
      if (!(wl[b] > 0)) {
        delete p;
        return fail(DLX_ERR_ARG, "fft_plan_create: wavelengths must be positive");
      }
      ax[b] = fft_axis(*d, wl[b]);
    }
    const int st = radix_fft_create(&p->rf, d->batch, d->n_in, d->pad, d->inverse != 0,
                                    ax.data(), alphas.data());
    if (st != DLX_OK) {
      radix_fft_release(&p->rf);
      delete p;
      return st;
    }
    *plan = p;
    return DLX_OK;
  }
  DLX_TRY(validate_variant(d->variant));
  auto* p = new (std::nothrow) dlx_fft_plan_s();
  if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
  TwoStep& ts = p->p.ts;
  ts.batch = d->batch; ts.n_in = d->n_in; ts.n_out = fft_out_side(d->n_in, d->pad);
  ts.variant = d->variant;
  ts.wl.assign(wl, wl + d->batch);
  std::vector<DftAxis> ax(d->batch);
  std::vector<float> alphas(d->batch, 1.0f / (float)fft_out_side(d->n_in, d->pad));
  for (int b = 0; b < d->batch; ++b) {
    if (!(wl[b] > 0)) {
      delete p;
      return fail(DLX_ERR_ARG, "fft_plan_create: wavelengths must be positive");
    }
    ax[b] = fft_axis(*d, wl[b]);
  }
  int st = ts.build(ax, ax, alphas);
  if (st == DLX_OK) st = p->p.alloc_buffers();
  if (st != DLX_OK) {
    p->p.release();
    delete p;
    return st;
  }
  *plan = p;
  return DLX_OK;
}

int dlx_fft_plan_destroy(dlx_fft_plan plan) {
  if (!plan) return DLX_OK;
  cudaDeviceSynchronize();
  radix_fft_release(&plan->rf);
  plan->p.release();
  delete plan;
  return DLX_OK;
}

int dlx_fft_forward(dlx_fft_plan plan, const void* in, void* out, void* stream) {
  if (!plan || !in || !out) return fail(DLX_ERR_ARG, "fft_forward: null pointer");
  if (plan->radix)
    return radix_fft_forward(plan->rf, static_cast<const float2*>(in), static_cast<float2*>(out),
                             as_stream(stream));
  return plan->p.forward(in, out, as_stream(stream));
}

int dlx_fft_adjoint(dlx_fft_plan plan, const void* gout, void* gin, void* stream) {
  if (!plan || !gout || !gin) return fail(DLX_ERR_ARG, "fft_adjoint: null pointer");
  if (plan->radix)
    return radix_fft_adjoint(plan->rf, static_cast<const float2*>(gout), static_cast<float2*>(gin),
                             as_stream(stream));
  return plan->p.adjoint(gout, gin, as_stream(stream));
}

// ---- elementwise entry points ----------------------------------------------
int dlx_phasor(const void* in, const float* amp, const float* opd, const float* phase,
               const float* amp_scale, const float* weights, double const_scale,
               const double* wavelengths_host, int batch, int n, double pixel_scale,
               double tilt_x, double tilt_y, void* out, void* stream) {
  if (batch < 0 || n < 0) return fail(DLX_ERR_SHAPE, "phasor: negative size");
  if (batch == 0 || n == 0) return DLX_OK;
  if (!out || !wavelengths_host) return fail(DLX_ERR_ARG, "phasor: null pointer");
  cudaStream_t s = as_stream(stream);
  for (int b0 = 0; b0 < batch; b0 += kMaxBatchArg) {
    const int nb = (batch - b0) < kMaxBatchArg ? (batch - b0) : kMaxBatchArg;
    BatchFF il;
    for (int i = 0; i < kMaxBatchArg; ++i) il.v[i] = make_float2(0.f, 0.f);
    for (int i = 0; i < nb; ++i) {
      const double w = wavelengths_host[b0 + i];
      if (!(w > 0)) return fail(DLX_ERR_ARG, "phasor: wavelengths must be positive");
      const FF f = ff_from_double(1.0 / w);
      il.v[i] = make_float2(f.hi, f.lo);
    }
    const long long off = (long long)b0 * n * n;
    PhasorArgs a{};
    a.in = in ? reinterpret_cast<const float2*>(in) + off : nullptr;
    a.amp = amp; a.opd = opd; a.phase = phase; a.amp_scale = amp_scale;
    a.weights = weights ? weights + b0 : nullptr;
    a.inv_lambda_ff = nullptr;
    a.const_scale = const_scale;
    a.batch = nb; a.n = n;
    a.pixel_scale = pixel_scale; a.tilt_x = tilt_x; a.tilt_y = tilt_y;
    a.out_c64 = reinterpret_cast<float2*>(out) + off;
    a.out_split = nullptr;
    DLX_TRY(launch_phasor(a, &il, s));
  }
  return DLX_OK;
}

int dlx_power_scale(const void* in, int batch, int n, double value, float* out_scale,
                    void* stream) {
  if (batch < 0 || n < 0) return fail(DLX_ERR_SHAPE, "power_scale: negative size");
  if (!in || !out_scale) return fail(DLX_ERR_ARG, "power_scale: null pointer");
  return launch_power_scale(reinterpret_cast<const float2*>(in), batch, (long long)n * n, value,
                            out_scale, as_stream(stream));
}

static int with_partials(size_t count, cudaStream_t s, double** ws) {
  DLX_TRY_CUDA(cudaMallocAsync((void**)ws, sizeof(double) * (count > 0 ? count : 1), s));
  return DLX_OK;
}

int dlx_amp_norm(const float* amp, int n, double value, float* out_scale, void* stream) {
  if (n <= 0) return fail(DLX_ERR_SHAPE, "amp_norm: n must be positive");
  if (!amp || !out_scale) return fail(DLX_ERR_ARG, "amp_norm: null pointer");
  cudaStream_t s = as_stream(stream);
  const int nparts = 128;
  double* ws = nullptr;
  DLX_TRY(with_partials(nparts, s, &ws));
  int st = launch_amp_norm(amp, (long long)n * n, value, out_scale, ws, nparts, s);
  cudaFreeAsync(ws, s);
  return st;
}

int dlx_amp_norm_backward(const float* amp, const float* g_eff, int n, double value,
                          float* g_amp, void* stream) {
  if (n <= 0) return fail(DLX_ERR_SHAPE, "amp_norm_backward: n must be positive");
  if (!amp || !g_eff || !g_amp) return fail(DLX_ERR_ARG, "amp_norm_backward: null pointer");
  cudaStream_t s = as_stream(stream);
  const int nparts = 128;
  double* ws = nullptr;
  // partials, then (n, c) as float pairs (16 bytes)
  DLX_TRY(with_partials(2 * nparts + 2, s, &ws));
  int st = launch_amp_norm_backward(amp, g_eff, (long long)n * n, value, g_amp, ws, nparts, s);
  cudaFreeAsync(ws, s);
  return st;
}

int dlx_basis_eval(const float* basis, const float* coeffs, const float* base, int nterms,
                   long long npix, float* out, void* stream) {
  if (nterms < 0 || npix < 0) return fail(DLX_ERR_SHAPE, "basis_eval: negative size");
  if (!out || (nterms > 0 && (!basis || !coeffs)))
    return fail(DLX_ERR_ARG, "basis_eval: null pointer");
  return launch_basis_eval(basis, coeffs, base, nterms, npix, out, as_stream(stream));
}

int dlx_basis_grad(const float* basis, const float* g, int nterms, long long npix,
                   float* g_coeffs, void* stream) {
  if (nterms < 0 || npix < 0) return fail(DLX_ERR_SHAPE, "basis_grad: negative size");
  if (nterms == 0) return DLX_OK;
  if (!basis || !g || !g_coeffs) return fail(DLX_ERR_ARG, "basis_grad: null pointer");
  cudaStream_t s = as_stream(stream);
  int sms = 0;
  DLX_TRY(device_sm_count(&sms));
  const int nparts = basis_grad_parts(nterms, npix, sms);
  double* ws = nullptr;
  DLX_TRY(with_partials((size_t)nparts * nterms, s, &ws));
  int st = launch_basis_grad(basis, g, nterms, npix, g_coeffs, ws, nparts, s);
  cudaFreeAsync(ws, s);
  return st;
}

int dlx_psf_sum(const void* in, int batch, long long npix, float* psf, void* stream) {
  if (batch < 0 || npix < 0) return fail(DLX_ERR_SHAPE, "psf_sum: negative size");
  if (!in || !psf) return fail(DLX_ERR_ARG, "psf_sum: null pointer");
  return launch_psf_sum(reinterpret_cast<const float2*>(in), batch, npix, psf,
                        as_stream(stream));
}

int dlx_downsample(const float* in, int n_in, int k, int mean, const float* flat, float* out,
                   void* stream) {
  if (k <= 0) return fail(DLX_ERR_ARG, "downsample: kernel size must be greater than 0");
  if (n_in % k != 0)
    return fail(DLX_ERR_SHAPE, "downsample: input size " + std::to_string(n_in) +
                                   " is not divisible by " + std::to_string(k));
  if (!in || !out) return fail(DLX_ERR_ARG, "downsample: null pointer");
  return launch_downsample(in, n_in, k, mean, flat, out, as_stream(stream));
}

int dlx_downsample_backward(const float* in, const float* g_out, int n_in, int k, int mean,
                            const float* flat, float* g_in, float* g_flat, void* stream) {
  if (k <= 0) return fail(DLX_ERR_ARG, "downsample: kernel size must be greater than 0");
  if (n_in % k != 0) return fail(DLX_ERR_SHAPE, "downsample: size not divisible");
  if (!g_out || (g_flat && !in)) return fail(DLX_ERR_ARG, "downsample_backward: null pointer");
  return launch_downsample_backward(in, g_out, n_in, k, mean, flat, g_in, g_flat,
                                    as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Fused polychromatic PSF plan over a batch of objects.
//
// A plan serves up to max_objects independent objects (requests or point
// sources) per launch. Batch element b = l * R + r holds wavelength l of
// object r, so the per-wavelength DFT operands are shared (A index = b / R).
// Larger object counts run in chunks of max_objects.
// ---------------------------------------------------------------------------
// Pixel chunks of the reverse-pass reductions (enough blocks to fill the GPU):
// the most a plan uses; small pupils use fewer, of at least 256 pixels each.
constexpr int kPolyParts = 1024;

// Pixel chunks of a plan's reductions: 256 pupil pixels or more each (one per
// thread of a block), at most kPolyParts. The workspace size depends on it.
static int poly_nparts(int n_in) {
  return (int)std::max(1LL, std::min((long long)kPolyParts, ((long long)n_in * n_in + 255) / 256));
}

struct dlx_poly_plan_s {
  TwoStep ts;
  double pixel_scale_in = 0;
  int max_obj = 1;
  DevBuf field;      // E: [L*R][N][N] c64 or [L*R][4][N][N] split
  DevBuf mid;        // D1 [L*R][M][N] / Xt [L*R][N][M]
  DevBuf fbar;       // [L*R][M][M] c64 or split
  DevBuf planes;     // intensity [L*R][M][M] f32, or pre/pim [2][L*R][N][N] f32
  DevBuf partial;    // double reduction partials
  DevBuf pathff;     // [R][N][N] float4 (path, phase) pairs, then [R][3][N][N] pixel sums
  DevBuf splitws;    // split-K partial sums of the GEMMs that split (see split_k)
  int nparts = kPolyParts;
  // Split K for GEMMs whose tiles leave most SMs idle, decided from the
  // plan's capacity (wavelengths x max_objects), not from the call's object
  // count, so an object's result is the same alone and in a batch of the
  // plan. Plans on a shared workspace (serving buckets, which fill the GPU by
  // batching requests) do not split.
  bool split_k = false;
  // Launch form chosen for this plan (dlx_poly_plan_set_gemm_form): the
  // paired GEMM mode of GemmArgs::pair_mode, and whether the K split decided
  // at creation is used.
  int pair_mode = 0;
  bool split_allowed = true;
  // Forward-to-backward reuse (dlx_poly_forward_token / dlx_poly_reuse_forward):
  // after a single-chunk forward, `field`, `mid` (the first-stage product D1)
  // and `pathff` hold that forward's state until the next call on the plan.
  unsigned long long epoch = 0;      // counts single-chunk forwards
  unsigned long long fwd_token = 0;  // token of the intact forward state, 0 if none
  unsigned long long reuse_req = 0;  // token the next backward may start from
  // Focal fields kept by the forward (dlx_poly_keep_focal): the y-contraction
  // also writes F = alpha D (complex64, into `fbar`), so that a backward that
  // reuses this forward forms F-bar = 2 G F elementwise instead of repeating
  // the y-contraction GEMM.
  bool keep_req = false;             // the next single-chunk forward keeps F
  bool fwd_focal = false;            // the intact forward state includes F
  std::vector<dlx_poly_object> fwd_objs;

  static bool same_inputs(const dlx_poly_object& a, const dlx_poly_object& b) {
    return a.amp == b.amp && a.amp_scale == b.amp_scale && a.opd == b.opd &&
           a.phase == b.phase && a.weights == b.weights && a.tilt_x == b.tilt_x &&
           a.tilt_y == b.tilt_y;
  }
  bool can_reuse(unsigned long long token, const dlx_poly_object* objs, int n) const {
    if (token == 0 || token != fwd_token || n != (int)fwd_objs.size()) return false;
    for (int r = 0; r < n; ++r)
      if (!same_inputs(objs[r], fwd_objs[r])) return false;
    return true;
  }

  // Device bytes this plan owns: an attached workspace belongs to the caller.
  size_t footprint() const {
    return ts.footprint() + field.owned_bytes() + mid.owned_bytes() + fbar.owned_bytes() +
           planes.owned_bytes() + partial.owned_bytes() + pathff.owned_bytes() +
           splitws.owned_bytes();
  }
  void release() {
    ts.release(); field.release(); mid.release(); fbar.release(); planes.release();
    partial.release(); pathff.release(); splitws.release();
  }

  static void tables(const dlx_poly_object* objs, int n, ObjTable* t, OutTable* o) {
    *t = ObjTable{};
    *o = OutTable{};
    t->n = n;
    o->n = n;
    for (int r = 0; r < n; ++r) {
      const dlx_poly_object& q = objs[r];
      t->o[r] = ObjDesc{q.amp, q.amp_scale, q.opd, q.phase, q.weights, q.g_psf, q.tilt_x,
                        q.tilt_y};
      o->o[r] = ObjOut{q.psf, q.g_amp, q.g_opd, q.g_phase, q.g_w, q.g_tilt};
    }
  }

  int build_field(const ObjTable& t, cudaStream_t s, float4* out_path = nullptr) {
    PhasorArgs a{};
    a.out_path = out_path;
    a.objs = t;
    a.inv_lambda_ff = ts.inv_lambda_ff.as<float2>();
    a.const_scale = 1.0;
    a.batch = ts.batch * t.n;
    a.n = ts.n_in;
    a.pixel_scale = pixel_scale_in;
    if (ts.variant == DLX_VARIANT_SPLIT_BF16) a.out_split = field.as<__nv_bfloat16>();
    else a.out_c64 = field.as<float2>();
    return launch_phasor(a, nullptr, s);
  }

  GemmArgs gemm(const TwoStep::AOp& op, int R, int M, int N, int K, bool conj, const void* B,
                const EpiArgs& e) const {
    GemmArgs g = gemm_for(ts.variant, ts.batch * R, M, N, K, op, conj, B, e);
    g.a_batch_div = R;
    g.a_bs = (long long)M * K;
    g.pair_mode = pair_mode;
    if (split_k && split_allowed && op.mat) {
      const long long tiles = (long long)ts.batch * max_obj * ((M + 127) / 128) * ((N + 127) / 128);
      const int sk = split_k_count(tiles, K);
      if (sk > 1) {
        g.splits = sk;
        g.split_ws = splitws.as<float2>();
      }
    }
    return g;
  }

  // keep: also write the focal fields F = alpha D (complex64) into `fbar`.
  int forward_chunk(const dlx_poly_object* objs, int R, float* psf_sum, int accumulate,
                    cudaStream_t s, bool keep = false) {
    const int L = ts.batch, N = ts.n_in, M = ts.n_out, v = ts.variant;
    if (!field.p)
      return fail(DLX_ERR_ARG, "poly plan: no workspace (dlx_poly_attach_workspace first)");
    fwd_token = 0;
    ObjTable t;
    OutTable o;
    tables(objs, R, &t, &o);
    // the (path, phase) pairs too, so that a backward can start from this state
    DLX_TRY(build_field(t, s, pathff.as<float4>()));
    EpiArgs e1 = epi_store(v, mid.p, nullptr);
    e1.objs = t;
    DLX_TRY(run_gemm(v, gemm(ts.opATx(), R, M, N, N, false, field.p, e1), s));
    EpiArgs e{};
    e.kind = EPI_INTENSITY;
    e.objs = t;
    e.alpha = ts.alpha.as<float>();
    e.out_f32 = planes.as<float>();
    if (keep) {
      // F = alpha D only (the complex64 store epilogue, no intensity planes):
      // the wavelength sum forms |F|^2 from F. (The PSF + cotangent epilogue
      // with no cotangent stores the same values and measured 136.6 against
      // 128.9 us per launch at 512^2 x 64.)
      e.kind = EPI_C64;
      e.out_c64 = fbar.as<float2>();
      e.out_f32 = nullptr;
    }
    DLX_TRY(run_gemm(v, gemm(ts.opATy(), R, M, M, N, false, mid.p, e), s));
    ObjReduceArgs ra{};
    ra.objs = t;
    ra.outs = o;
    ra.L = L;
    ra.npix = (long long)M * M;
    ra.planes = planes.as<float>();
    if (keep) ra.fields = fbar.as<float2>();
    ra.psf_sum = psf_sum;
    ra.accumulate = accumulate;
    return launch_obj_psf_reduce(ra, s);
  }

  // reuse: `mid` and `pathff` still hold the forward state of these objects
  // (checked by the caller), so the pupil field and D1 are not rebuilt; with
  // `focal`, `fbar` holds that forward's focal fields F as well, and F-bar =
  // 2 G F is formed elementwise (into `planes` in the split form, in place in
  // the FP32 form) instead of by the y-contraction GEMM.
  int backward_chunk(const dlx_poly_object* objs, int R, cudaStream_t s, float* sum_amp = nullptr,
                     float* sum_opd = nullptr, float* sum_phase = nullptr,
                     bool sum_pixels = false, bool accumulate_sum = false, bool reuse = false,
                     bool focal = false) {
    const int N = ts.n_in, M = ts.n_out, v = ts.variant;
    if (!field.p)
      return fail(DLX_ERR_ARG, "poly plan: no workspace (dlx_poly_attach_workspace first)");
    fwd_token = 0;  // the reverse pass overwrites mid
    ObjTable t;
    OutTable o;
    tables(objs, R, &t, &o);
    for (int r = 0; r < R; ++r)
      if (!t.o[r].G) return fail(DLX_ERR_ARG, "poly backward: every object needs g_psf");
    if (reuse && focal) {
      const bool split = v == DLX_VARIANT_SPLIT_BF16;
      DLX_TRY(launch_focal_gradf(fbar.as<float2>(), t, ts.batch * R, M,
                                 split ? planes.as<__nv_bfloat16>() : nullptr,
                                 split ? nullptr : fbar.as<float2>(), s));
      return reverse_from_fbar(t, o, R, s, sum_amp, sum_opd, sum_phase, sum_pixels,
                               accumulate_sum, split ? planes.p : fbar.p);
    }
    if (!reuse) {
      // Recompute the forward fields.
      DLX_TRY(build_field(t, s, pathff.as<float4>()));
      EpiArgs e1 = epi_store(v, mid.p, nullptr);
      e1.objs = t;
      DLX_TRY(run_gemm(v, gemm(ts.opATx(), R, M, N, N, false, field.p, e1), s));
    }
    // The per-wavelength focal field is recomputed here from D1 in every case.
    // Fbar[v][u] = 2 alpha G[v][u] D[v][u]
    EpiArgs eg{};
    eg.kind = EPI_GRADF;
    eg.objs = t;
    eg.alpha = ts.alpha.as<float>();
    if (v == DLX_VARIANT_SPLIT_BF16) eg.out_split = fbar.as<__nv_bfloat16>();
    else eg.out_c64 = fbar.as<float2>();
    DLX_TRY(run_gemm(v, gemm(ts.opATy(), R, M, M, N, false, mid.p, eg), s));
    return reverse_from_fbar(t, o, R, s, sum_amp, sum_opd, sum_phase, sum_pixels,
                             accumulate_sum, fbar.p);
  }

  // PSF and reverse pass in one sweep, for objects whose cotangent g_psf is
  // known before the forward pass (serving requests, linear functionals): the
  // forward's y-contraction writes the intensity planes and F̄ = 2αG⊙D at
  // once, so the reverse pass starts at the adjoint GEMMs with no recompute.
  int forward_backward_chunk(const dlx_poly_object* objs, int R, cudaStream_t s) {
    const int L = ts.batch, N = ts.n_in, M = ts.n_out, v = ts.variant;
    if (!field.p)
      return fail(DLX_ERR_ARG, "poly plan: no workspace (dlx_poly_attach_workspace first)");
    fwd_token = 0;
    ObjTable t;
    OutTable o;
    tables(objs, R, &t, &o);
    for (int r = 0; r < R; ++r)
      if (!t.o[r].G) return fail(DLX_ERR_ARG, "poly forward_backward: every object needs g_psf");
    DLX_TRY(build_field(t, s, pathff.as<float4>()));
    EpiArgs e1 = epi_store(v, mid.p, nullptr);
    e1.objs = t;
    DLX_TRY(run_gemm(v, gemm(ts.opATx(), R, M, N, N, false, field.p, e1), s));
    EpiArgs e{};
    e.kind = EPI_PSF_GRADF;
    e.objs = t;
    e.alpha = ts.alpha.as<float>();
    e.out_f32 = planes.as<float>();
    if (v == DLX_VARIANT_SPLIT_BF16) e.out_split = fbar.as<__nv_bfloat16>();
    else e.out_c64 = fbar.as<float2>();
    DLX_TRY(run_gemm(v, gemm(ts.opATy(), R, M, M, N, false, mid.p, e), s));
    ObjReduceArgs rp{};
    rp.objs = t;
    rp.outs = o;
    rp.L = L;
    rp.npix = (long long)M * M;
    rp.planes = planes.as<float>();
    DLX_TRY(launch_obj_psf_reduce(rp, s));
    return reverse_from_fbar(t, o, R, s, nullptr, nullptr, nullptr, false, false, fbar.p);
  }

  // Adjoint GEMMs from F̄ (at `fb`: `fbar`, or `planes` after kept focal
  // fields) and the pupil reductions.
  int reverse_from_fbar(const ObjTable& t, const OutTable& o, int R, cudaStream_t s,
                        float* sum_amp, float* sum_opd, float* sum_phase, bool sum_pixels,
                        bool accumulate_sum, const void* fb) {
    const int L = ts.batch, N = ts.n_in, M = ts.n_out, v = ts.variant;
    // Xt[x][v] = sum_u conj(Ax[x][u]) Fbar[v][u]
    EpiArgs e3 = epi_store(v, mid.p, nullptr);
    e3.objs = t;
    DLX_TRY(run_gemm(v, gemm(ts.opANx(), R, N, M, M, true, fb, e3), s));
    ObjReduceArgs ra{};
    ra.objs = t;
    ra.outs = o;
    ra.L = L;
    ra.npix = (long long)N * N;
    ra.k_dev = ts.kvec.as<double>();
    ra.n_side = N;
    ra.pixel_scale = pixel_scale_in;
    ra.partial_ws = partial.as<double>();
    ra.nparts = nparts;
    ra.sum_pixels = sum_pixels ? 1 : 0;
    ra.sum_g_amp = sum_amp;
    ra.sum_g_opd = sum_opd;
    ra.sum_g_phase = sum_phase;
    ra.accumulate_sum = accumulate_sum ? 1 : 0;
    if (L <= kFusedPupilMaxL) {
      // Ebar[y][x] = alpha sum_v conj(Ay[y][v]) Xt[x][v] as complex planes; the
      // fused reduction forms the per-wavelength pupil terms and sums them.
      EpiArgs ec{};
      ec.kind = EPI_C64;
      ec.objs = t;
      ec.alpha = ts.alpha.as<float>();
      ec.out_c64 = planes.as<float2>();
      DLX_TRY(run_gemm(v, gemm(ts.opANy(), R, N, N, M, true, mid.p, ec), s));
      ra.ebar = planes.as<float2>();
      ra.path = pathff.as<float4>();
      ra.split_form = v == DLX_VARIANT_SPLIT_BF16 ? 1 : 0;
      ra.inv_lambda_ff = ts.inv_lambda_ff.as<float2>();
      ra.pix_scratch = reinterpret_cast<float*>(pathff.as<float4>() + (size_t)R * N * N);
      return launch_obj_pupil_fused(ra, s);
    }
    // Ebar[y][x] = alpha sum_v conj(Ay[y][v]) Xt[x][v] -> pupil-gradient planes
    float* pre = planes.as<float>();
    float* pim = pre + (size_t)L * R * N * N;
    EpiArgs ep{};
    ep.kind = EPI_PUPIL;
    ep.objs = t;
    ep.alpha = ts.alpha.as<float>();
    ep.out_f32 = pre;
    ep.out_f32b = pim;
    ep.inv_lambda_ff = ts.inv_lambda_ff.as<float2>();
    ep.pixel_scale = pixel_scale_in;
    ep.path = pathff.as<float4>();
    DLX_TRY(run_gemm(v, gemm(ts.opANy(), R, N, N, M, true, mid.p, ep), s));
    ra.pre = pre;
    ra.pim = pim;
    return launch_obj_pupil_reduce(ra, s);
  }
};

// Byte sizes of the per-call buffers of a plan: field, mid, fbar, planes,
// partial, pathff and the split-K partials (split_on: the plan splits K).
constexpr int kPolyBuffers = 7;
static void poly_ws_sizes(int L, int N, int M, int R, int nparts, bool split_on,
                          size_t sz[kPolyBuffers]) {
  const size_t lr = (size_t)L * R, n = N, m = M;
  // complex64 planes, or split planes with padded rows (split_ld), whichever
  // is larger: E [N][N], D1 [M][N] or Xt [N][M], F-bar [M][M]
  sz[0] = split_bytes(lr, N, N);
  const size_t d1 = split_bytes(lr, M, N), xt = split_bytes(lr, N, M);
  sz[1] = d1 > xt ? d1 : xt;
  sz[2] = split_bytes(lr, M, M);
  // intensity [M][M] f32, pupil planes 2 x [N][N] f32, or Ē [N][N] complex64;
  // and, after kept focal fields, F-bar as split planes [M][M]
  const size_t a = lr * m * m * 4, b = 2 * lr * n * n * 4, c = split_bytes(lr, M, M);
  sz[3] = std::max(a, std::max(b, c));
  sz[4] = sizeof(double) * (size_t)nparts * R * (L + 2);
  sz[5] = (sizeof(float4) + 3 * sizeof(float)) * (size_t)R * n * n;  // (path, phase) + pixel sums
  sz[6] = 0;
  if (split_on) {
    // the four GEMM shapes of a plan: rows x cols, inner size
    const int shapes[4][3] = {{M, N, N}, {M, M, N}, {N, M, M}, {N, N, M}};
    for (const auto& sh : shapes) {
      const long long tiles = (long long)lr * ((sh[0] + 127) / 128) * ((sh[1] + 127) / 128);
      const size_t bytes = split_k_bytes(split_k_count(tiles, sh[2]), (long long)lr, sh[0], sh[1]);
      if (bytes > sz[6]) sz[6] = bytes;
    }
  }
  for (int i = 0; i < kPolyBuffers; ++i) sz[i] = (sz[i] + 255) / 256 * 256;
}

// Plans of the tensor-core form with cached operands split K where their
// GEMMs leave most SMs idle (read once, at creation).
static bool poly_split_on(const dlx_poly_desc& d) {
  return d.variant == DLX_VARIANT_SPLIT_BF16 && d.operand_mode == 0 && split_k_enabled();
}

static int poly_create(const dlx_poly_desc* d, const double* wl, int max_objects,
                       dlx_poly_plan* plan, bool own_workspace = true) {
  if (!d || !wl || !plan) return fail(DLX_ERR_ARG, "poly_plan_create: null pointer");
  *plan = nullptr;
  if (d->n_wavelengths <= 0 || d->n_in <= 0 || d->n_out <= 0)
    return fail(DLX_ERR_SHAPE, "poly_plan_create: sizes must be positive");
  if (max_objects <= 0 || max_objects > kMaxObj)
    return fail(DLX_ERR_ARG, "poly_plan_create: max_objects must lie in [1, " +
                                 std::to_string(kMaxObj) + "]");
  if (!(d->pixel_scale_in > 0) || !(d->pixel_scale_out > 0))
    return fail(DLX_ERR_ARG, "poly_plan_create: pixel scales must be positive");
  DLX_TRY(check_focal(d->focal_length, "poly_plan_create"));
  DLX_TRY(validate_variant(d->variant));
  auto* p = new (std::nothrow) dlx_poly_plan_s();
  if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
  const int L = d->n_wavelengths, N = d->n_in, M = d->n_out;
  TwoStep& ts = p->ts;
  ts.batch = L; ts.n_in = N; ts.n_out = M; ts.variant = d->variant;
  ts.wl.assign(wl, wl + L);
  p->pixel_scale_in = d->pixel_scale_in;
  p->max_obj = max_objects;
  p->nparts = poly_nparts(d->n_in);
  std::vector<DftAxis> ax(L);
  std::vector<float> alphas(L);
  for (int b = 0; b < L; ++b) {
    if (!(wl[b] > 0)) {
      delete p;
      return fail(DLX_ERR_ARG, "poly_plan_create: wavelengths must be positive");
    }
    ax[b] = mft_axis(wl[b], N, d->pixel_scale_in, M, d->pixel_scale_out, 0.0, d->focal_length,
                     false);
    alphas[b] = (float)mft_alpha(wl[b], N, d->pixel_scale_in, M, d->pixel_scale_out,
                                 d->focal_length);
  }
  if (d->operand_mode != 0 && d->operand_mode != 1) {
    delete p;
    return fail(DLX_ERR_ARG, "poly_plan_create: operand_mode must be 0 or 1");
  }
  int st = ts.build(ax, ax, alphas, d->operand_mode == 1);
  p->split_k = own_workspace && poly_split_on(*d);
  if (st == DLX_OK && own_workspace) {
    size_t sz[kPolyBuffers];
    poly_ws_sizes(L, N, M, max_objects, p->nparts, p->split_k, sz);
    if (st == DLX_OK) st = p->field.alloc(sz[0]);
    if (st == DLX_OK) st = p->mid.alloc(sz[1]);
    if (st == DLX_OK) st = p->fbar.alloc(sz[2]);
    if (st == DLX_OK) st = p->planes.alloc(sz[3]);
    if (st == DLX_OK) st = p->partial.alloc(sz[4]);
    if (st == DLX_OK) st = p->pathff.alloc(sz[5]);
    if (st == DLX_OK) st = p->splitws.alloc(sz[6]);
  }
  if (st != DLX_OK) {
    p->release();
    delete p;
    return st;
  }
  *plan = p;
  return DLX_OK;
}

extern "C" {

int dlx_poly_plan_set_gemm_form(dlx_poly_plan plan, int pair_mode, int split_k) {
  if (!plan) return fail(DLX_ERR_ARG, "poly_plan_set_gemm_form: null plan");
  if (pair_mode < 0 || pair_mode > 2)
    return fail(DLX_ERR_ARG, "poly_plan_set_gemm_form: pair_mode must be 0, 1 or 2");
  plan->pair_mode = pair_mode;
  plan->split_allowed = split_k != 0;
  return DLX_OK;
}

int dlx_poly_plan_create(const dlx_poly_desc* d, const double* wl, dlx_poly_plan* plan) {
  return poly_create(d, wl, 1, plan);
}

int dlx_poly_plan_create_batched(const dlx_poly_desc* d, const double* wl, int max_objects,
                                 dlx_poly_plan* plan) {
  return poly_create(d, wl, max_objects, plan);
}

int dlx_poly_plan_create_shared(const dlx_poly_desc* d, const double* wl, int max_objects,
                                dlx_poly_plan* plan) {
  return poly_create(d, wl, max_objects, plan, false);
}

int dlx_poly_workspace_bytes(const dlx_poly_desc* d, int max_objects, size_t* bytes) {
  if (!d || !bytes) return fail(DLX_ERR_ARG, "poly_workspace_bytes: null pointer");
  if (d->n_wavelengths <= 0 || d->n_in <= 0 || d->n_out <= 0 || max_objects <= 0)
    return fail(DLX_ERR_SHAPE, "poly_workspace_bytes: sizes must be positive");
  size_t sz[kPolyBuffers];
  poly_ws_sizes(d->n_wavelengths, d->n_in, d->n_out, max_objects, poly_nparts(d->n_in), false,
                sz);
  *bytes = 0;
  for (int i = 0; i < kPolyBuffers; ++i) *bytes += sz[i];
  return DLX_OK;
}

int dlx_poly_attach_workspace(dlx_poly_plan plan, void* workspace, size_t bytes) {
  if (!plan || !workspace) return fail(DLX_ERR_ARG, "poly_attach_workspace: null pointer");
  plan->fwd_token = 0;
  if ((uintptr_t)workspace % 256 != 0)
    return fail(DLX_ERR_ARG, "poly_attach_workspace: workspace must be 256-byte aligned");
  size_t sz[kPolyBuffers];
  poly_ws_sizes(plan->ts.batch, plan->ts.n_in, plan->ts.n_out, plan->max_obj, plan->nparts,
                plan->split_k, sz);
  size_t need = 0;
  for (int i = 0; i < kPolyBuffers; ++i) need += sz[i];
  if (bytes < need)
    return fail(DLX_ERR_SHAPE, "poly_attach_workspace: " + std::to_string(bytes) +
                                   " bytes given, " + std::to_string(need) + " needed");
  char* w = static_cast<char*>(workspace);
  plan->field.view(w, sz[0]);
  w += sz[0];
  plan->mid.view(w, sz[1]);
  w += sz[1];
  plan->fbar.view(w, sz[2]);
  w += sz[2];
  plan->planes.view(w, sz[3]);
  w += sz[3];
  plan->partial.view(w, sz[4]);
  w += sz[4];
  plan->pathff.view(w, sz[5]);
  w += sz[5];
  plan->splitws.view(w, sz[6]);
  return DLX_OK;
}

int dlx_poly_plan_destroy(dlx_poly_plan plan) {
  if (!plan) return DLX_OK;
  cudaDeviceSynchronize();
  plan->release();
  delete plan;
  return DLX_OK;
}

int dlx_poly_plan_footprint(dlx_poly_plan plan, size_t* bytes) {
  if (!plan || !bytes) return fail(DLX_ERR_ARG, "poly_plan_footprint: null pointer");
  *bytes = plan->footprint();
  return DLX_OK;
}

int dlx_poly_plan_info(dlx_poly_plan plan, int* n_wavelengths, int* n_in, int* n_out,
                       int* max_objects) {
  if (!plan) return fail(DLX_ERR_ARG, "poly_plan_info: null plan");
  if (n_wavelengths) *n_wavelengths = plan->ts.batch;
  if (n_in) *n_in = plan->ts.n_in;
  if (n_out) *n_out = plan->ts.n_out;
  if (max_objects) *max_objects = plan->max_obj;
  return DLX_OK;
}

int dlx_poly_forward(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                     float* psf_sum, int accumulate, void* stream) {
  if (!plan || (n_objects > 0 && !objs)) return fail(DLX_ERR_ARG, "poly_forward: null pointer");
  if (n_objects < 0) return fail(DLX_ERR_ARG, "poly_forward: negative object count");
  cudaStream_t s = as_stream(stream);
  // focal fields are kept only by a single-chunk forward (a reusable state)
  const bool keep = plan->keep_req && n_objects >= 1 && n_objects <= plan->max_obj;
  plan->keep_req = false;  // a request applies to one forward call
  for (int o0 = 0; o0 < n_objects; o0 += plan->max_obj) {
    const int R = std::min(plan->max_obj, n_objects - o0);
    DLX_TRY(plan->forward_chunk(objs + o0, R, psf_sum, (o0 > 0) ? 1 : accumulate, s, keep));
  }
  if (n_objects >= 1 && n_objects <= plan->max_obj) {
    plan->fwd_token = ++plan->epoch;
    plan->fwd_objs.assign(objs, objs + n_objects);
    plan->fwd_focal = keep;
  }
  return DLX_OK;
}

int dlx_poly_backward(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                      void* stream) {
  if (!plan || (n_objects > 0 && !objs)) return fail(DLX_ERR_ARG, "poly_backward: null pointer");
  if (n_objects < 0) return fail(DLX_ERR_ARG, "poly_backward: negative object count");
  cudaStream_t s = as_stream(stream);
  const unsigned long long req = plan->reuse_req;
  plan->reuse_req = 0;  // a request applies to one backward call
  const bool reuse = plan->can_reuse(req, objs, n_objects);
  const bool focal = reuse && plan->fwd_focal;
  for (int o0 = 0; o0 < n_objects; o0 += plan->max_obj) {
    const int R = std::min(plan->max_obj, n_objects - o0);
    DLX_TRY(plan->backward_chunk(objs + o0, R, s, nullptr, nullptr, nullptr, false, false,
                                 reuse, focal));
  }
  return DLX_OK;
}

int dlx_poly_forward_token(dlx_poly_plan plan, unsigned long long* token) {
  if (!plan || !token) return fail(DLX_ERR_ARG, "poly_forward_token: null pointer");
  *token = plan->fwd_token;
  return DLX_OK;
}

int dlx_poly_reuse_forward(dlx_poly_plan plan, unsigned long long token) {
  if (!plan) return fail(DLX_ERR_ARG, "poly_reuse_forward: null plan");
  plan->reuse_req = token;
  return DLX_OK;
}

int dlx_poly_keep_focal(dlx_poly_plan plan, int keep) {
  if (!plan) return fail(DLX_ERR_ARG, "poly_keep_focal: null plan");
  plan->keep_req = keep != 0;
  return DLX_OK;
}

int dlx_poly_forward_backward(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                              void* stream) {
  if (!plan || (n_objects > 0 && !objs))
    return fail(DLX_ERR_ARG, "poly_forward_backward: null pointer");
  if (n_objects < 0) return fail(DLX_ERR_ARG, "poly_forward_backward: negative object count");
  cudaStream_t s = as_stream(stream);
  for (int o0 = 0; o0 < n_objects; o0 += plan->max_obj) {
    const int R = std::min(plan->max_obj, n_objects - o0);
    DLX_TRY(plan->forward_backward_chunk(objs + o0, R, s));
  }
  return DLX_OK;
}

int dlx_poly_backward_sum(dlx_poly_plan plan, const dlx_poly_object* objs, int n_objects,
                          float* g_amp, float* g_opd, float* g_phase, void* stream) {
  if (!plan || (n_objects > 0 && !objs))
    return fail(DLX_ERR_ARG, "poly_backward_sum: null pointer");
  if (n_objects < 0) return fail(DLX_ERR_ARG, "poly_backward_sum: negative object count");
  cudaStream_t s = as_stream(stream);
  plan->reuse_req = 0;
  for (int o0 = 0; o0 < n_objects; o0 += plan->max_obj) {
    const int R = std::min(plan->max_obj, n_objects - o0);
    DLX_TRY(plan->backward_chunk(objs + o0, R, s, g_amp, g_opd, g_phase, true, o0 > 0));
  }
  return DLX_OK;
}

int dlx_poly_psf(dlx_poly_plan plan, const float* amp, const float* amp_scale, const float* opd,
                 const float* phase, const float* weights, double tilt_x, double tilt_y,
                 float* psf_out, void* stream) {
  if (!plan || !psf_out) return fail(DLX_ERR_ARG, "poly_psf: null pointer");
  dlx_poly_object o{};
  o.amp = amp; o.amp_scale = amp_scale; o.opd = opd; o.phase = phase; o.weights = weights;
  o.tilt_x = tilt_x; o.tilt_y = tilt_y;
  o.psf = psf_out;
  return dlx_poly_forward(plan, &o, 1, nullptr, 0, stream);
}

int dlx_poly_psf_grad(dlx_poly_plan plan, const float* amp, const float* amp_scale,
                      const float* opd, const float* phase, const float* weights, double tilt_x,
                      double tilt_y, const float* g_psf, float* g_amp, float* g_opd,
                      float* g_phase, float* g_w, void* stream) {
  if (!plan || !g_psf) return fail(DLX_ERR_ARG, "poly_psf_grad: null pointer");
  dlx_poly_object o{};
  o.amp = amp; o.amp_scale = amp_scale; o.opd = opd; o.phase = phase; o.weights = weights;
  o.tilt_x = tilt_x; o.tilt_y = tilt_y;
  o.g_psf = g_psf;
  o.g_amp = g_amp; o.g_opd = g_opd; o.g_phase = g_phase;
  o.g_w = weights ? g_w : nullptr;
  return dlx_poly_backward(plan, &o, 1, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Separable transforms with caller-described axes, and the angular-spectrum
// propagator: the device side of dLux's ABCD propagators
// (layers/abcd_propagators.py:245-459), whose arithmetic the reference takes
// from the abcdLux package (lct.lct_prop, lct.lct_prop_fft, asm.asm_prop).
// ---------------------------------------------------------------------------
struct dlx_xform_plan_s {
  TwoStepPlan p;
};

struct dlx_asm_plan_s {
  TwoStepPlan fwd;   // centred DFT of the zero-padded field: N -> P
  TwoStepPlan inv;   // centred inverse DFT: P -> P
  DevBuf spec;       // [b][P][P] c64 spectrum
  DevBuf H;          // [b][P][P] c64 transfer function, tabulated at creation
  DevBuf zl, lam2;   // double [b]: distance / lambda, lambda^2
  double df = 0;     // frequency step 1 / (P dx)
  int P = 0;
};

namespace {

DftAxis to_axis(const dlx_xform_axis& a) {
  DftAxis d{};
  d.a_in = a.a_in; d.b_in = a.b_in; d.a_out = a.a_out; d.b_out = a.b_out;
  d.sigma = a.sigma; d.q_in = a.q_in; d.q_out = a.q_out;
  d.d_out = a.phase;
  d.scale = a.scale;
  return d;
}

int make_two_step(TwoStepPlan* t, int batch, int n_in, int n_out, int variant,
                  const std::vector<DftAxis>& ax, const std::vector<DftAxis>& ay) {
  TwoStep& ts = t->ts;
  ts.batch = batch; ts.n_in = n_in; ts.n_out = n_out; ts.variant = variant;
  ts.wl.assign(batch, 1.0);  // no wavelength enters the matrices: they are given
  std::vector<float> ones(batch, 1.0f);
  DLX_TRY(ts.build(ax, ay, ones));
  return t->alloc_buffers();
}

}  // namespace

extern "C" {

int dlx_xform_plan_create(const dlx_xform_desc* d, const dlx_xform_axis* ax_x,
                          const dlx_xform_axis* ax_y, dlx_xform_plan* plan) {
  if (!d || !ax_x || !ax_y || !plan) return fail(DLX_ERR_ARG, "xform_plan_create: null pointer");
  *plan = nullptr;
  if (d->batch <= 0 || d->n_in <= 0 || d->n_out <= 0)
    return fail(DLX_ERR_SHAPE, "xform_plan_create: batch, n_in and n_out must be positive");
  DLX_TRY(validate_variant(d->variant));
  auto* p = new (std::nothrow) dlx_xform_plan_s();
  if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
  std::vector<DftAxis> ax(d->batch), ay(d->batch);
  for (int b = 0; b < d->batch; ++b) {
    ax[b] = to_axis(ax_x[b]);
    ay[b] = to_axis(ax_y[b]);
  }
  const int st = make_two_step(&p->p, d->batch, d->n_in, d->n_out, d->variant, ax, ay);
  if (st != DLX_OK) {
    p->p.release();
    delete p;
    return st;
  }
  *plan = p;
  return DLX_OK;
}

int dlx_xform_plan_destroy(dlx_xform_plan plan) {
  if (!plan) return DLX_OK;
  cudaDeviceSynchronize();
  plan->p.release();
  delete plan;
  return DLX_OK;
}

int dlx_xform_forward(dlx_xform_plan plan, const void* in, void* out, void* stream) {
  if (!plan || !in || !out) return fail(DLX_ERR_ARG, "xform_forward: null pointer");
  return plan->p.forward(in, out, as_stream(stream));
}

int dlx_xform_adjoint(dlx_xform_plan plan, const void* gout, void* gin, void* stream) {
  if (!plan || !gout || !gin) return fail(DLX_ERR_ARG, "xform_adjoint: null pointer");
  return plan->p.adjoint(gout, gin, as_stream(stream));
}

int dlx_asm_plan_create(const dlx_asm_desc* d, const double* wavelengths_host,
                        dlx_asm_plan* plan) {
  if (!d || !wavelengths_host || !plan) return fail(DLX_ERR_ARG, "asm_plan_create: null pointer");
  *plan = nullptr;
  const int B = d->batch, N = d->n_in, P = d->n_pad;
  if (B <= 0 || N <= 0 || P < N)
    return fail(DLX_ERR_SHAPE, "asm_plan_create: need batch, n_in > 0 and n_pad >= n_in");
  if (!(d->pixel_scale > 0)) return fail(DLX_ERR_ARG, "asm_plan_create: pixel_scale must be > 0");
  for (int b = 0; b < B; ++b)
    if (!(wavelengths_host[b] > 0))
      return fail(DLX_ERR_ARG, "asm_plan_create: wavelengths must be positive");
  DLX_TRY(validate_variant(d->variant));
  auto* p = new (std::nothrow) dlx_asm_plan_s();
  if (!p) return fail(DLX_ERR_NOMEM, "host allocation failed");
  p->P = P;
  p->df = 1.0 / (P * d->pixel_scale);
  // Centred transforms (fftshift o fft o ifftshift): index j sits at j - c with
  // c = floor(P / 2); the input lands at slot i + (P - N) / 2 of the padded grid.
  const int c = P / 2, npad = (P - N) / 2;
  DftAxis f{};
  f.a_in = 1.0; f.b_in = (double)(npad - c);
  f.a_out = 1.0; f.b_out = -(double)c;
  f.sigma = -1.0 / P;
  f.scale = 1.0;
  DftAxis g{};
  g.a_in = 1.0; g.b_in = -(double)c;
  g.a_out = 1.0; g.b_out = -(double)c;
  g.sigma = 1.0 / P;
  g.scale = 1.0 / P;
  std::vector<DftAxis> fa(B, f), ga(B, g);
  std::vector<double> zl(B), l2(B);
  for (int b = 0; b < B; ++b) {
    zl[b] = d->distance / wavelengths_host[b];
    l2[b] = wavelengths_host[b] * wavelengths_host[b];
  }
  int st = make_two_step(&p->fwd, B, N, P, d->variant, fa, fa);
  if (st == DLX_OK) st = make_two_step(&p->inv, B, P, P, d->variant, ga, ga);
  if (st == DLX_OK) st = p->spec.alloc(sizeof(float2) * (size_t)B * P * P);
  if (st == DLX_OK) st = p->zl.alloc(sizeof(double) * B);
  if (st == DLX_OK) st = p->lam2.alloc(sizeof(double) * B);
  auto upload = [&](DevBuf& dst, const std::vector<double>& src) {
    const cudaError_t e =
        cudaMemcpy(dst.p, src.data(), sizeof(double) * src.size(), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? DLX_OK : check_cuda(e, "cudaMemcpy(asm constants)");
  };
  if (st == DLX_OK) st = upload(p->zl, zl);
  if (st == DLX_OK) st = upload(p->lam2, l2);
  if (st == DLX_OK) st = p->H.alloc(sizeof(float2) * (size_t)B * P * P);
  if (st == DLX_OK)
    st = launch_asm_table(p->H.as<float2>(), B, P, p->df, p->zl.as<double>(),
                          p->lam2.as<double>(), 0);
  if (st == DLX_OK) {
    // the table is read from the caller's streams, which need not wait for this one
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) st = check_cuda(e, "asm transfer table");
  }
  if (st != DLX_OK) {
    p->fwd.release(); p->inv.release(); p->spec.release(); p->H.release(); p->zl.release();
    p->lam2.release();
    delete p;
    return st;
  }
  *plan = p;
  return DLX_OK;
}

int dlx_asm_plan_destroy(dlx_asm_plan plan) {
  if (!plan) return DLX_OK;
  cudaDeviceSynchronize();
  plan->fwd.release(); plan->inv.release(); plan->spec.release(); plan->H.release();
  plan->zl.release(); plan->lam2.release();
  delete plan;
  return DLX_OK;
}

int dlx_asm_forward(dlx_asm_plan plan, const void* in, void* out, void* stream) {
  if (!plan || !in || !out) return fail(DLX_ERR_ARG, "asm_forward: null pointer");
  cudaStream_t s = as_stream(stream);
  DLX_TRY(plan->fwd.forward(in, plan->spec.p, s));
  DLX_TRY(launch_asm_apply(plan->spec.as<float2>(), plan->H.as<float2>(), plan->fwd.ts.batch,
                           plan->P, 0, s));
  return plan->inv.forward(plan->spec.p, out, s);
}

int dlx_asm_adjoint(dlx_asm_plan plan, const void* gout, void* gin, void* stream) {
  if (!plan || !gout || !gin) return fail(DLX_ERR_ARG, "asm_adjoint: null pointer");
  cudaStream_t s = as_stream(stream);
  DLX_TRY(plan->inv.adjoint(gout, plan->spec.p, s));
  DLX_TRY(launch_asm_apply(plan->spec.as<float2>(), plan->H.as<float2>(), plan->fwd.ts.batch,
                           plan->P, 1, s));
  return plan->fwd.adjoint(plan->spec.p, gin, s);
}

}  // extern "C"
