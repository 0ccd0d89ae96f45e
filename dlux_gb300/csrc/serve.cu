// serve.cu -- one serving batch as a single stream-ordered call.
//
// A serving loop answers many small PSF requests. Going through the generic
// entry points would cost the host one call per step per request (copies,
// OPD, PSF, reverse pass, basis gradient, copies back). dlx_serve_run issues
// the whole batch at once on one stream from host memory the caller keeps
// pinned, so
//   * the host side of a batch is a single call, and
//   * the batch allocates nothing and never synchronises, which makes it
//     capturable as a CUDA graph: a later batch of the same shape on the
//     same buffers is one graph launch.
// Each request's result does not depend on the other requests of its batch:
// the kernels give every object the same arithmetic and reduce in a fixed
// order.
#include <cstdint>

#include "kernels.h"

namespace dlx {
namespace {

constexpr int kServeParts = 64;  // partial sums per basis term in the coefficient gradient

size_t round256(size_t n) { return (n + 255) / 256 * 256; }

struct ServeLayout {
  size_t coeffs, weights, g_psf, opd, psf, g_opd, grad, partial, total;
};

ServeLayout serve_layout(int R, int K, int N, int M, int L) {
  const size_t r = R, k = K, n2 = (size_t)N * N, m2 = (size_t)M * M;
  ServeLayout s{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += round256(bytes);
    return at;
  };
  s.coeffs = take(r * k * 4);
  s.weights = take(r * (size_t)L * 4);
  s.g_psf = take(r * m2 * 4);
  s.opd = take(r * n2 * 4);
  s.psf = take(r * m2 * 4);
  s.g_opd = take(r * n2 * 4);
  s.grad = take(r * k * 4);
  s.partial = take(r * k * kServeParts * sizeof(double));
  s.total = off;
  return s;
}

}  // namespace
}  // namespace dlx

using namespace dlx;

extern "C" {

int dlx_serve_workspace_bytes(int max_objects, int n_coeffs, int n_in, int n_out,
                              int n_wavelengths, size_t* bytes) {
  if (!bytes) return fail(DLX_ERR_ARG, "serve_workspace_bytes: null pointer");
  if (max_objects <= 0 || n_coeffs <= 0 || n_in <= 0 || n_out <= 0 || n_wavelengths <= 0)
    return fail(DLX_ERR_SHAPE, "serve_workspace_bytes: sizes must be positive");
  *bytes = serve_layout(max_objects, n_coeffs, n_in, n_out, n_wavelengths).total;
  return DLX_OK;
}

int dlx_serve_run(dlx_poly_plan plan, const dlx_serve_batch* b, void* stream) {
  if (!plan || !b) return fail(DLX_ERR_ARG, "serve_run: null pointer");
  int L = 0, N = 0, M = 0, max_obj = 0;
  DLX_TRY(dlx_poly_plan_info(plan, &L, &N, &M, &max_obj));
  const int R = b->n_objects, G = b->n_grad, K = b->n_coeffs;
  if (R < 1 || R > max_obj)
    return fail(DLX_ERR_ARG, "serve_run: n_objects must lie in [1, " + std::to_string(max_obj) +
                                 "] for this plan");
  if (G < 0 || G > R) return fail(DLX_ERR_ARG, "serve_run: n_grad must lie in [0, n_objects]");
  if (K <= 0) return fail(DLX_ERR_SHAPE, "serve_run: n_coeffs must be positive");
  if (!b->basis || !b->amp || !b->h_coeffs || !b->h_weights || !b->h_psf || !b->d_work)
    return fail(DLX_ERR_ARG, "serve_run: null buffer");
  if (G > 0 && (!b->h_g_psf || !b->h_grad))
    return fail(DLX_ERR_ARG, "serve_run: gradient requests need h_g_psf and h_grad");
  if ((uintptr_t)b->d_work % 256 != 0)
    return fail(DLX_ERR_ARG, "serve_run: d_work must be 256-byte aligned");
  const ServeLayout lay = serve_layout(R, K, N, M, L);
  if (b->d_work_bytes < lay.total)
    return fail(DLX_ERR_SHAPE, "serve_run: d_work holds " + std::to_string(b->d_work_bytes) +
                                   " bytes, " + std::to_string(lay.total) + " needed");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(b->d_work);
  float* coeffs = reinterpret_cast<float*>(w + lay.coeffs);
  float* weights = reinterpret_cast<float*>(w + lay.weights);
  float* g_psf = reinterpret_cast<float*>(w + lay.g_psf);
  float* opd = reinterpret_cast<float*>(w + lay.opd);
  float* psf = reinterpret_cast<float*>(w + lay.psf);
  float* g_opd = reinterpret_cast<float*>(w + lay.g_opd);
  float* grad = reinterpret_cast<float*>(w + lay.grad);
  double* partial = reinterpret_cast<double*>(w + lay.partial);
  const size_t n2 = (size_t)N * N, m2 = (size_t)M * M;

  DLX_TRY_CUDA(cudaMemcpyAsync(coeffs, b->h_coeffs, sizeof(float) * R * K,
                               cudaMemcpyHostToDevice, s));
  DLX_TRY_CUDA(cudaMemcpyAsync(weights, b->h_weights, sizeof(float) * R * L,
                               cudaMemcpyHostToDevice, s));
  if (G > 0)
    DLX_TRY_CUDA(cudaMemcpyAsync(g_psf, b->h_g_psf, sizeof(float) * G * m2,
                                 cudaMemcpyHostToDevice, s));
  for (int r = 0; r < R; ++r)
    DLX_TRY(launch_basis_eval(b->basis, coeffs + (size_t)r * K, nullptr, K, (long long)n2,
                              opd + r * n2, s));

  dlx_poly_object objs[kMaxObj] = {};
  for (int r = 0; r < R; ++r) {
    objs[r].amp = b->amp;
    objs[r].amp_scale = b->amp_scale;
    objs[r].opd = opd + r * n2;
    objs[r].weights = weights + (size_t)r * L;
    objs[r].psf = psf + r * m2;
    if (r < G) {
      objs[r].g_psf = g_psf + r * m2;
      objs[r].g_opd = g_opd + r * n2;
    }
  }
  // Gradient requests (the first G) know their cotangent up front: PSF and
  // reverse pass in one sweep. The others take the forward pass only.
  if (G > 0) DLX_TRY(dlx_poly_forward_backward(plan, objs, G, s));
  if (R > G) DLX_TRY(dlx_poly_forward(plan, objs + G, R - G, nullptr, 0, s));
  if (G > 0) {
    for (int r = 0; r < G; ++r)
      DLX_TRY(launch_basis_grad(b->basis, g_opd + r * n2, K, (long long)n2, grad + (size_t)r * K,
                                partial + (size_t)r * K * kServeParts, kServeParts, s));
  }
  DLX_TRY_CUDA(cudaMemcpyAsync(b->h_psf, psf, sizeof(float) * R * m2, cudaMemcpyDeviceToHost, s));
  if (G > 0)
    DLX_TRY_CUDA(cudaMemcpyAsync(b->h_grad, grad, sizeof(float) * G * K, cudaMemcpyDeviceToHost,
                                 s));
  return DLX_OK;
}

}  // extern "C"
