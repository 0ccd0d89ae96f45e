// noalloc.cu -- an MFT entry point that allocates no device memory.
//
// dlx_mft_forward_noalloc computes the same batched MFT as a
// dlx_mft_plan created with DLX_VARIANT_FP32, but it never calls
// cudaMalloc/cudaFree (nor anything that allocates). Its scratch -- the two
// DFT matrices and the half-transformed field of one wavelength -- lives in a
// fixed, file-scope device array that is loaded with the library.
//
// It exists for callers that may not allocate device memory:
//   * a JAX/XLA custom call: XLA preallocates most of the GPU for its own
//     allocator (75% by default), so a cudaMalloc inside the handler can fail
//     or fragment XLA's pool;
//   * control or real-time loops that forbid allocation after start-up;
//   * hosts that hand the library every buffer and own the rest of the device.
//
// Costs and rules:
//   * every GPU that loads the library holds kNoAllocScratchBytes (8 MiB)
//     for the life of the process;
//   * sizes needing more than that are rejected (DLX_ERR_SHAPE): a call
//     needs 3 * roundup(n_in * n_out * 8, 256) + 256 bytes (three complex64
//     matrices, each rounded up to 256 bytes, plus the normalisation scalar),
//     e.g. n_in = n_out = 512 fits and 592 x 592 does not;
//   * focal_length 0 selects the angular form; a negative one is refused;
//   * all calls share the one array, so calls that may overlap on the GPU
//     (different streams, no ordering between them) race and must be
//     serialised by the caller; calls on one stream are ordered;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress; make that first call before any stream capture.
#include <cmath>
#include <mutex>

#include "kernels.h"

namespace dlx {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // 8 MiB
constexpr size_t kNoAllocAlign = 256;

// The scratch itself. Host code must not use this name as a pointer: on the
// host it is only a stand-in for the symbol, so its device address is looked
// up once per device (scratch_address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_addr_mutex;
void* g_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (set-up on first use).
int scratch_address(void** out) {
  int dev = 0;
  DLX_TRY(current_device(&dev));
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return check_cuda(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return DLX_OK;
}

// One axis of dLux's transfer matrix (utils/propagation.py:67-127) as FP64
// affine coefficients: phase = sigma * x_i * u_j cycles.
DftAxis axis_for(double wl, int n_in, double ps_in, int n_out, double ps_out, double shift,
                 double focal, bool inverse) {
  DftAxis a{};
  double s_out = ps_out / (wl / (ps_in * n_in));
  if (focal != 0) s_out /= focal;  // 0: angular (focal_length=None)
  a.a_in = 1.0 / n_in;
  a.b_in = -(0.5 * (n_in - 1) + shift) / n_in;
  a.a_out = s_out;
  a.b_out = -(0.5 * (n_out - 1) + shift) * s_out;
  a.sigma = inverse ? 1.0 : -1.0;
  a.scale = 1.0;
  return a;
}

// [n_out][n_in] transfer matrix (transposed layout) from an axis passed by value.
__global__ void noalloc_dft_kernel(DftAxis ax, int rows, int cols, float2* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;  // input index
  const int r = blockIdx.y * blockDim.y + threadIdx.y;  // output index
  if (r >= rows || c >= cols) return;
  const double x = ax.a_in * (double)c + ax.b_in;
  const double u = ax.a_out * (double)r + ax.b_out;
  out[(long long)r * cols + c] = cis_cycles(ax.sigma * x * u);
}

__global__ void noalloc_set_kernel(float* dst, float v) { *dst = v; }

}  // namespace
}  // namespace dlx

using namespace dlx;

extern "C" int dlx_mft_forward_noalloc(const void* in_c64, int batch, int n_in,
                                       double pixel_scale_in, int n_out,
                                       double pixel_scale_out, const double* wavelengths_host,
                                       double focal_length, double shift_x, double shift_y,
                                       int inverse, void* out_c64, void* stream) {
  if (batch < 0 || n_in <= 0 || n_out <= 0)
    return fail(DLX_ERR_SHAPE, "mft_forward_noalloc: batch >= 0, n_in > 0, n_out > 0 required");
  if (batch == 0) return DLX_OK;
  if (!in_c64 || !out_c64 || !wavelengths_host)
    return fail(DLX_ERR_ARG, "mft_forward_noalloc: null pointer");
  if (!(pixel_scale_in > 0) || !(pixel_scale_out > 0))
    return fail(DLX_ERR_ARG, "mft_forward_noalloc: pixel scales must be positive");
  DLX_TRY(check_focal(focal_length, "mft_forward_noalloc"));
  const size_t mat = (size_t)n_in * n_out;
  const size_t mat_bytes = (mat * sizeof(float2) + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign;
  const size_t need = 3 * mat_bytes + kNoAllocAlign;  // AxT, AyT, half-transformed field, alpha
  if (need > kNoAllocScratchBytes)
    return fail(DLX_ERR_SHAPE,
                "mft_forward_noalloc: n_in = " + std::to_string(n_in) + ", n_out = " +
                    std::to_string(n_out) + " needs " + std::to_string(need) +
                    " bytes of scratch (3 * roundup(n_in * n_out * 8, 256) + 256); the fixed "
                    "scratch holds " + std::to_string(kNoAllocScratchBytes));
  for (int b = 0; b < batch; ++b)
    if (!(wavelengths_host[b] > 0))
      return fail(DLX_ERR_ARG, "mft_forward_noalloc: wavelengths must be positive");

  void* base = nullptr;
  DLX_TRY(scratch_address(&base));
  unsigned char* s = static_cast<unsigned char*>(base);
  float2* atx = reinterpret_cast<float2*>(s);
  float2* aty = reinterpret_cast<float2*>(s + mat_bytes);
  float2* mid = reinterpret_cast<float2*>(s + 2 * mat_bytes);
  float* alpha = reinterpret_cast<float*>(s + 3 * mat_bytes);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  const dim3 block(32, 8);
  const dim3 grid(ceil_div(n_in, 32), ceil_div(n_out, 8));
  // One wavelength at a time through the same scratch (stream-ordered).
  for (int b = 0; b < batch; ++b) {
    const double wl = wavelengths_host[b];
    noalloc_dft_kernel<<<grid, block, 0, st>>>(
        axis_for(wl, n_in, pixel_scale_in, n_out, pixel_scale_out, shift_x, focal_length,
                 inverse != 0), n_out, n_in, atx);
    DLX_LAUNCH_CHECK("noalloc_dft_kernel");
    noalloc_dft_kernel<<<grid, block, 0, st>>>(
        axis_for(wl, n_in, pixel_scale_in, n_out, pixel_scale_out, shift_y, focal_length,
                 inverse != 0), n_out, n_in, aty);
    DLX_LAUNCH_CHECK("noalloc_dft_kernel");
    double out_size = n_out * pixel_scale_out;
    if (focal_length != 0) out_size /= focal_length;
    const double nf = out_size / (wl / (n_in * pixel_scale_in));
    noalloc_set_kernel<<<1, 1, 0, st>>>(alpha, (float)(nf / ((double)n_in * n_out)));
    DLX_LAUNCH_CHECK("noalloc_set_kernel");

    const float2* in_b = reinterpret_cast<const float2*>(in_c64) + (long long)b * n_in * n_in;
    float2* out_b = reinterpret_cast<float2*>(out_c64) + (long long)b * n_out * n_out;
    // D1[u][y] = sum_x AxT[u][x] E[y][x]
    GemmArgs g1{};
    g1.batch = 1; g1.M = n_out; g1.N = n_in; g1.K = n_in;
    g1.A = atx; g1.B = in_b; g1.a_batch_div = 1;
    g1.epi.kind = EPI_C64;
    g1.epi.out_c64 = mid;
    DLX_TRY(launch_gemm_fp32(g1, st));
    // F[v][u] = alpha sum_y AyT[v][y] D1[u][y]
    GemmArgs g2{};
    g2.batch = 1; g2.M = n_out; g2.N = n_out; g2.K = n_in;
    g2.A = aty; g2.B = mid; g2.a_batch_div = 1;
    g2.epi.kind = EPI_C64;
    g2.epi.alpha = alpha;
    g2.epi.out_c64 = out_b;
    DLX_TRY(launch_gemm_fp32(g2, st));
  }
  return DLX_OK;
}
