// zernike.cu -- dynamic apertures with Zernike aberrations on the device
// (AberratedAperture over a Circular, Square, Rectangular or RegPoly aperture,
// layers/apertures.py:240-555 and :643-800; DynamicZernike, polynomials.py:20-51;
// utils/zernikes.py:122-419; soft edges and distances utils/geometry.py:49-91,
// 229-351, 402-579; CoordTransform coordinates.py:240-320 with
// utils/coordinates.py:23-101).
//
// Every pixel is evaluated from its coordinates, so no K x N x N basis is
// stored or read:
//   (x, y)  = pixel centre (i - (N-1)/2) * dx, transformed in dLux's order:
//             translate, shear (with dLux's transposed-plane form), compress,
//             rotate (clockwise by `rotation`)
//   T       = soft mask of the shape's distance d (circle: radius - r; square:
//             w/2 - max(|x|, |y|); rectangle: -max(|x| - w/2, |y| - h/2);
//             polygon: -max over its edges of the signed edge distance),
//             clip(d, -c, c) (negated when occulting) rescaled by the global
//             min/max of d to [0, 1]
//   opd     = sum_j c_j Z_j at (x, y) / extent (radius, sqrt(2) w, hypot(h/2,
//             w/2) or rmax), where Z_j = [rho <= 1] norm_j R_nm(rho) {cos,
//             sin}(|m| theta) for a circle, and for an n-sided shape the
//             polygon-stretched form (1 / r_a) Z_j((u, v) / r_a) with
//             r_a = cos(pi / n) / cos(u_a), u_a the angle from the nearest
//             edge normal (utils/zernikes.py:318-352).
// The radial part is Horner in t = rho^2 times rho^|m|, and rho^|m| {cos,
// sin}(|m| theta) is Re/Im of (u + i v)^|m|, so only the polygon stretch
// takes an angle.
#include <math_constants.h>

#include <atomic>
#include <cmath>
#include <string>

#include "kernels.h"

namespace dlx {
namespace {

// d of one pixel after the coordinate transformation; also returns the
// Zernike coordinates (u, v) and the factor `zs` multiplying every Zernike
// value there (1 for a circle; 1 / r_a for a polygon-stretched basis).
__device__ __forceinline__ float aperture_point(const ZernAperture& a, int i, int j, float* u,
                                                float* v, float* zs) {
  const float half = 0.5f * (float)(a.n - 1);
  const float x0 = ((float)i - half) * a.pixel_scale;
  const float y0 = ((float)j - half) * a.pixel_scale;
  float x = x0 - a.translation[0];
  float y = y0 - a.translation[1];
  // dLux shears the translated coordinate planes with their transposes; on a
  // square xy grid the transposed x plane holds y0 - tx, the transposed y
  // plane x0 - ty (each keeps its own plane's translation).
  const float xs = x + (y0 - a.translation[0]) * a.shear[0];
  const float ys = y + (x0 - a.translation[1]) * a.shear[1];
  x = xs * a.compression[0];
  y = ys * a.compression[1];
  const float xr = a.rot_c * x + a.rot_s * y;   // cos(-r) x + sin(-r) y
  const float yr = -a.rot_s * x + a.rot_c * y;  // -sin(-r) x + cos(-r) y
  float uu = xr / a.extent, vv = yr / a.extent, scale = 1.0f;
  if (a.nsides > 0) {
    // polygon stretch: the wedge of the nearest edge and its radial factor
    const float alpha = CUDART_PI_F / (float)a.nsides;
    const float phi = atan2f(vv, uu) + alpha;
    const float wedge = floorf((phi + alpha) / (2.0f * alpha));
    const float ua = phi - wedge * (2.0f * alpha);
    const float ra = cosf(alpha) / cosf(ua);
    uu /= ra;
    vv /= ra;
    scale = 1.0f / ra;
  }
  *u = uu;
  *v = vv;
  *zs = scale;
  float d;
  if (a.shape == AP_SQUARE) {
    d = a.half_w - fmaxf(fabsf(xr), fabsf(yr));
  } else if (a.shape == AP_RECTANGLE) {
    d = -fmaxf(fabsf(xr) - a.half_w, fabsf(yr) - a.half_h);
  } else if (a.shape == AP_POLYGON) {
    float e = -INFINITY;
    for (int k = 0; k < a.n_edges; ++k)
      e = fmaxf(e, fmaf(a.edge_a[k], xr, fmaf(a.edge_b[k], yr, a.edge_c[k])));
    d = -e;
  } else {
    d = a.radius - sqrtf(xr * xr + yr * yr);
  }
  if (a.occulting) d = -d;
  return fminf(fmaxf(d, -a.clip), a.clip);
}

// Z_j at (u, v): norm * R(rho) * (Re|Im)((u + i v)^|m|) inside the unit disk.
__device__ __forceinline__ float zernike_at(const ZernTable& z, int j, float u, float v) {
  const float t = u * u + v * v;
  if (sqrtf(t) > 1.0f) return 0.0f;
  const int am = z.m[j] < 0 ? -z.m[j] : z.m[j];
  // P(t) = sum_k c_k t^((n - |m|)/2 - k), c_0 the highest power
  const int nk = z.nc[j];
  float p = z.c[j][0];
  for (int k = 1; k < nk; ++k) p = fmaf(p, t, z.c[j][k]);
  float zr = 1.0f, zi = 0.0f;  // (u + i v)^|m|
  for (int q = 0; q < am; ++q) {
    const float nr = zr * u - zi * v;
    zi = zr * v + zi * u;
    zr = nr;
  }
  return z.norm[j] * p * (z.m[j] < 0 ? zi : zr);
}

__device__ __forceinline__ unsigned f2ordered(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Global min and max of the clipped distances (order-encoded atomics: exact).
__global__ void aperture_minmax_kernel(ZernAperture a, unsigned* mm) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long npix = (long long)a.n * a.n;
  float lo = INFINITY, hi = -INFINITY;
  if (p < npix) {
    float u, v, zs;
    const float d = aperture_point(a, (int)(p % a.n), (int)(p / a.n), &u, &v, &zs);
    lo = hi = d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0 && lo <= hi) {
    atomicMin(mm, f2ordered(lo));
    atomicMax(mm + 1, f2ordered(hi));
  }
}

__global__ void aperture_eval_kernel(ZernAperture a, ZernTable z, const float* __restrict__ coeffs,
                                     const unsigned* __restrict__ mm, float* __restrict__ trans,
                                     float* __restrict__ opd) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long npix = (long long)a.n * a.n;
  if (p >= npix) return;
  float u, v, zs;
  const float d = aperture_point(a, (int)(p % a.n), (int)(p / a.n), &u, &v, &zs);
  if (trans) {
    const float dmin = ordered2f(mm[0]), dmax = ordered2f(mm[1]);
    // soften(): constant support when every distance is equal, else (d - min) / (max - min)
    trans[p] = dmax == dmin ? (d > 0.0f ? 1.0f : 0.0f) : (d - dmin) / (dmax - dmin);
  }
  if (opd) {
    float acc = 0.0f;
    for (int j = 0; j < z.K; ++j) acc = fmaf(coeffs[j], zernike_at(z, j, u, v), acc);
    opd[p] = acc * zs;
  }
}

// Partial sums of sum_p Z_j(p) g[p], 8 terms per block row, float pairs per thread.
constexpr int kZernTermsPerBlock = 8;
__global__ void zernike_grad_partial_kernel(ZernAperture a, ZernTable z, const float* __restrict__ g,
                                            int nparts, double* __restrict__ partial) {
  __shared__ double smem[kZernTermsPerBlock][8];
  const long long npix = (long long)a.n * a.n;
  const long long chunk = (npix + nparts - 1) / nparts;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(npix, lo + chunk);
  const int j0 = blockIdx.y * kZernTermsPerBlock;
  float sh[kZernTermsPerBlock], sl[kZernTermsPerBlock];
#pragma unroll
  for (int t = 0; t < kZernTermsPerBlock; ++t) sh[t] = sl[t] = 0.0f;
  for (long long p = lo + threadIdx.x; p < hi; p += blockDim.x) {
    float u, v, zs;
    aperture_point(a, (int)(p % a.n), (int)(p / a.n), &u, &v, &zs);
    const float gp = g[p] * zs;
#pragma unroll
    for (int t = 0; t < kZernTermsPerBlock; ++t) {
      if (j0 + t >= z.K) break;
      const float x = zernike_at(z, j0 + t, u, v);
      const float pr = x * gp;
      const float pe = fmaf(x, gp, -pr);
      const float s = sh[t] + pr;
      const float bv = s - sh[t];
      sl[t] += ((sh[t] - (s - bv)) + (pr - bv)) + pe;
      sh[t] = s;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < kZernTermsPerBlock; ++t) {
    double w = (double)sh[t] + (double)sl[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if (lane == 0) smem[t][warp] = w;
  }
  __syncthreads();
  if (threadIdx.x < kZernTermsPerBlock && j0 + (int)threadIdx.x < z.K) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += smem[threadIdx.x][w];
    partial[(long long)(j0 + threadIdx.x) * nparts + blockIdx.x] = s;
  }
}

__global__ void zernike_grad_finish_kernel(const double* __restrict__ partial, int nparts, int K,
                                           float* __restrict__ g_coeffs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  double s = 0.0;
  for (int i = 0; i < nparts; ++i) s += partial[(long long)j * nparts + i];
  g_coeffs[j] = (float)s;
}

int validate(const ZernAperture& a, const ZernTable& z) {
  if (a.n <= 0) return fail(DLX_ERR_SHAPE, "aperture: npixels must be positive");
  if (!(a.extent > 0)) return fail(DLX_ERR_ARG, "aperture: its size must be positive");
  if (!(a.clip > 0)) return fail(DLX_ERR_ARG, "softening must be greater than 0.");
  if (z.K < 0 || z.K > kMaxZern) return fail(DLX_ERR_ARG, "aperture: too many Zernike terms");
  for (int j = 0; j < z.K; ++j)
    if (z.nc[j] < 1 || z.nc[j] > kMaxZernCoeff)
      return fail(DLX_ERR_ARG, "aperture: Zernike order too high for the device table");
  return DLX_OK;
}

}  // namespace

int launch_aperture_eval(const ZernAperture& a, const ZernTable& z, const float* coeffs,
                         unsigned* minmax_ws, float* trans, float* opd, cudaStream_t s) {
  DLX_TRY(validate(a, z));
  const long long npix = (long long)a.n * a.n;
  if (trans) {
    const unsigned init[2] = {0xffffffffu, 0u};
    DLX_TRY_CUDA(cudaMemcpyAsync(minmax_ws, init, sizeof(init), cudaMemcpyHostToDevice, s));
    aperture_minmax_kernel<<<ceil_div(npix, 256), 256, 0, s>>>(a, minmax_ws);
    DLX_LAUNCH_CHECK("aperture_minmax_kernel");
  }
  aperture_eval_kernel<<<ceil_div(npix, 256), 256, 0, s>>>(a, z, coeffs, minmax_ws, trans,
                                                           (z.K > 0 && coeffs) ? opd : nullptr);
  DLX_LAUNCH_CHECK("aperture_eval_kernel");
  return DLX_OK;
}

int launch_zernike_grad(const ZernAperture& a, const ZernTable& z, const float* g, double* partial,
                        int nparts, float* g_coeffs, cudaStream_t s) {
  DLX_TRY(validate(a, z));
  if (z.K == 0) return DLX_OK;
  dim3 grid(nparts, (z.K + kZernTermsPerBlock - 1) / kZernTermsPerBlock);
  zernike_grad_partial_kernel<<<grid, 256, 0, s>>>(a, z, g, nparts, partial);
  DLX_LAUNCH_CHECK("zernike_grad_partial_kernel");
  zernike_grad_finish_kernel<<<ceil_div(z.K, 64), 64, 0, s>>>(partial, nparts, z.K, g_coeffs);
  DLX_LAUNCH_CHECK("zernike_grad_finish_kernel");
  return DLX_OK;
}

}  // namespace dlx

using namespace dlx;

namespace {

// Noll index -> (n, m): n from the row, |m| from the position in the row
// (even n: 0, 2, 2, 4, 4, ...; odd n: 1, 1, 3, 3, ...), m < 0 (sine) for odd j.
void noll_nm(int j, int* n, int* m) {
  int nn = 0;
  while ((nn + 1) * (nn + 2) / 2 < j) ++nn;
  const int pos = j - nn * (nn + 1) / 2 - 1;
  const int am = (nn % 2 == 0) ? 2 * ((pos + 1) / 2) : 2 * (pos / 2) + 1;
  *n = nn;
  *m = (am != 0 && (j % 2 == 1)) ? -am : am;
}

double fact(int x) {
  double f = 1.0;
  for (int i = 2; i <= x; ++i) f *= i;
  return f;
}

int build_table(const int* noll, int K, ZernTable* z) {
  if (K < 0 || K > kMaxZern)
    return fail(DLX_ERR_ARG, "zernike: between 0 and " + std::to_string(kMaxZern) + " terms");
  if (K > 0 && !noll) return fail(DLX_ERR_ARG, "zernike: null Noll indices");
  *z = ZernTable{};
  z->K = K;
  for (int t = 0; t < K; ++t) {
    if (noll[t] < 1) return fail(DLX_ERR_ARG, "The Zernike index must be greater than 0.");
    int n, m;
    noll_nm(noll[t], &n, &m);
    const int am = m < 0 ? -m : m;
    const int nk = (n - am) / 2 + 1;
    if (nk > kMaxZernCoeff)
      return fail(DLX_ERR_ARG, "zernike: radial order " + std::to_string(n) +
                                   " is above the device table limit");
    z->n[t] = n;
    z->m[t] = m;
    z->nc[t] = nk;
    z->norm[t] = (float)(std::sqrt((double)n + 1.0) * (m != 0 ? std::sqrt(2.0) : 1.0));
    for (int k = 0; k < nk; ++k) {
      const double c = ((k % 2) ? -1.0 : 1.0) * fact(n - k) /
                       (fact(k) * fact((n + am) / 2 - k) * fact((n - am) / 2 - k));
      z->c[t][k] = (float)c;
    }
  }
  return DLX_OK;
}

int build_aperture(const dlx_aperture_desc* d, ZernAperture* a) {
  if (!d) return fail(DLX_ERR_ARG, "aperture: null descriptor");
  *a = ZernAperture{};
  a->n = d->npixels;
  a->pixel_scale = (float)d->pixel_scale;
  for (int i = 0; i < 2; ++i) {
    a->translation[i] = (float)d->translation[i];
    a->shear[i] = (float)d->shear[i];
    a->compression[i] = (float)d->compression[i];
  }
  a->rot_c = (float)std::cos(-d->rotation);
  a->rot_s = (float)std::sin(-d->rotation);
  a->shape = d->shape;
  a->radius = (float)d->radius;
  a->half_w = (float)(0.5 * d->width);
  a->half_h = (float)(0.5 * d->height);
  switch (d->shape) {
    case AP_CIRCLE:
      if (!(d->radius > 0)) return fail(DLX_ERR_ARG, "aperture: radius must be positive");
      a->extent = (float)d->radius;
      a->nsides = 0;
      break;
    case AP_SQUARE:
      if (!(d->width > 0)) return fail(DLX_ERR_ARG, "aperture: width must be positive");
      a->extent = (float)(std::sqrt(2.0) * d->width);
      a->nsides = 4;
      break;
    case AP_RECTANGLE:
      if (!(d->width > 0) || !(d->height > 0))
        return fail(DLX_ERR_ARG, "aperture: width and height must be positive");
      a->extent = (float)std::hypot(0.5 * d->height, 0.5 * d->width);
      a->nsides = 4;
      break;
    case AP_POLYGON: {
      const int n = d->nsides;
      if (n < 3 || n > kMaxPolySides)
        return fail(DLX_ERR_ARG, "aperture: a regular polygon needs 3 to " +
                                     std::to_string(kMaxPolySides) + " sides");
      if (!(d->radius > 0)) return fail(DLX_ERR_ARG, "aperture: rmax must be positive");
      a->extent = (float)d->radius;
      a->nsides = n;
      a->n_edges = n;
      // Edges from vertex i to i + 1, vertices at angles linspace(-pi, pi, n,
      // endpoint=False) (utils/geometry.py:519-552). Signed distance of edge
      // i as a x + b y + c (utils/geometry.py:486-516): horizontal (slope 0),
      // vertical (run exactly 0: slope inf) or general, with the sign that
      // makes the inside negative.
      const double pi = 3.14159265358979323846;
      for (int i = 0; i < n; ++i) {
        const int k = (i + 1) % n;
        const double ti = -pi + 2.0 * pi * i / n, tk = -pi + 2.0 * pi * k / n;
        const double xi = d->radius * std::cos(ti), yi = d->radius * std::sin(ti);
        const double xk = d->radius * std::cos(tk), yk = d->radius * std::sin(tk);
        const double dx = xk - xi, dy = yk - yi;
        auto sign = [](double v) { return v > 0 ? 1.0 : (v < 0 ? -1.0 : 0.0); };
        double ea, eb, ec;
        if (dx == 0) {                     // vertical: -sgn (x_i - x)
          const double sg = sign(xi);
          ea = sg; eb = 0.0; ec = -sg * xi;
        } else if (dy / dx == 0) {         // horizontal: -sgn (y_i - y)
          const double sg = sign(yi);
          ea = 0.0; eb = sg; ec = -sg * yi;
        } else {                           // -sgn (m x - y + y_i - m x_i) / sqrt(m^2 + 1)
          const double m = dy / dx;
          const double sg = sign(yi - m * xi), s = std::sqrt(m * m + 1.0);
          ea = -sg * m / s; eb = sg / s; ec = -sg * (yi - m * xi) / s;
        }
        a->edge_a[i] = (float)ea;
        a->edge_b[i] = (float)eb;
        a->edge_c[i] = (float)ec;
      }
      break;
    }
    default:
      return fail(DLX_ERR_ARG, "aperture: unknown shape " + std::to_string(d->shape));
  }
  if (!(d->softening > 0)) return fail(DLX_ERR_ARG, "softening must be greater than 0.");
  a->clip = (float)(d->pixel_scale * d->softening / 2.0);
  a->occulting = d->occulting ? 1 : 0;
  return DLX_OK;
}

}  // namespace

extern "C" {

int dlx_zernike_table(const int* noll, int n_terms, int* n_out, int* m_out, float* c_out) {
  ZernTable z;
  DLX_TRY(build_table(noll, n_terms, &z));
  for (int t = 0; t < n_terms; ++t) {
    if (n_out) n_out[t] = z.n[t];
    if (m_out) m_out[t] = z.m[t];
    if (c_out)
      for (int k = 0; k < kMaxZernCoeff; ++k) c_out[t * kMaxZernCoeff + k] = k < z.nc[t] ? z.c[t][k] : 0.f;
  }
  return DLX_OK;
}

int dlx_aberrated_aperture(const dlx_aperture_desc* desc, const int* noll, int n_terms,
                           const float* coeffs, float* transmission, float* opd, void* stream) {
  ZernAperture a;
  ZernTable z;
  DLX_TRY(build_aperture(desc, &a));
  DLX_TRY(build_table(noll, n_terms, &z));
  if (!transmission && !opd) return DLX_OK;
  if (opd && n_terms > 0 && !coeffs) return fail(DLX_ERR_ARG, "aberrated_aperture: null coefficients");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned* mm = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&mm, 2 * sizeof(unsigned), s));
  const int st = launch_aperture_eval(a, z, coeffs, mm, transmission, opd, s);
  cudaFreeAsync(mm, s);
  if (opd && n_terms == 0)
    DLX_TRY_CUDA(cudaMemsetAsync(opd, 0, sizeof(float) * (size_t)a.n * a.n, s));
  return st;
}

int dlx_aberrated_aperture_grad(const dlx_aperture_desc* desc, const int* noll, int n_terms,
                                const float* g_opd, float* g_coeffs, void* stream) {
  ZernAperture a;
  ZernTable z;
  DLX_TRY(build_aperture(desc, &a));
  DLX_TRY(build_table(noll, n_terms, &z));
  if (n_terms == 0) return DLX_OK;
  if (!g_opd || !g_coeffs) return fail(DLX_ERR_ARG, "aberrated_aperture_grad: null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nparts = 128;
  double* partial = nullptr;
  DLX_TRY_CUDA(cudaMallocAsync((void**)&partial, sizeof(double) * nparts * n_terms, s));
  const int st = launch_zernike_grad(a, z, g_opd, partial, nparts, g_coeffs, s);
  cudaFreeAsync(partial, s);
  return st;
}

}  // extern "C"
