// Shared device helpers of the mom25d sweep engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include <string>

#ifndef M25_PI
#define M25_PI 3.141592653589793
#endif

namespace m25 {

constexpr double kPi = 3.141592653589793;
constexpr double kC0 = 299792458.0;
constexpr double kMu0 = 4e-7 * kPi;
// 1 / (mu0 c0^2) evaluated in the same order as the host constants
__host__ __device__ inline double eps0() { return 1.0 / (kMu0 * kC0 * kC0); }

// ------------------------------------------------------------------ complex
template <class T>
struct cx {
  T re, im;
  __host__ __device__ cx() : re(0), im(0) {}
  __host__ __device__ cx(T r, T i = 0) : re(r), im(i) {}
  template <class U>
  __host__ __device__ explicit cx(const cx<U>& o) : re(T(o.re)), im(T(o.im)) {}
};
using zd = cx<double>;
using zf = cx<float>;

template <class T> __host__ __device__ inline cx<T> operator+(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> __host__ __device__ inline cx<T> operator-(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> __host__ __device__ inline cx<T> operator-(cx<T> a) { return {-a.re, -a.im}; }
template <class T> __host__ __device__ inline cx<T> operator*(cx<T> a, cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T> __host__ __device__ inline cx<T> operator*(cx<T> a, T s) { return {a.re * s, a.im * s}; }
template <class T> __host__ __device__ inline cx<T> operator*(T s, cx<T> a) { return {a.re * s, a.im * s}; }
template <class T> __host__ __device__ inline cx<T>& operator+=(cx<T>& a, cx<T> b) { a.re += b.re; a.im += b.im; return a; }
template <class T> __host__ __device__ inline cx<T>& operator-=(cx<T>& a, cx<T> b) { a.re -= b.re; a.im -= b.im; return a; }
template <class T> __host__ __device__ inline cx<T> conj(cx<T> a) { return {a.re, -a.im}; }
template <class T> __host__ __device__ inline T norm2(cx<T> a) { return a.re * a.re + a.im * a.im; }
template <class T> __host__ __device__ inline T cabs1(cx<T> a) { return fabs(a.re) + fabs(a.im); }

// Smith's algorithm for complex division.
template <class T> __host__ __device__ inline cx<T> operator/(cx<T> a, cx<T> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    T r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  T r = b.re / b.im, d = b.re * r + b.im;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
template <class T> __host__ __device__ inline cx<T> operator/(cx<T> a, T s) { return {a.re / s, a.im / s}; }

__host__ __device__ inline double cabs(zd z) { return hypot(z.re, z.im); }

// Principal square root (Re >= 0; the sign of Im follows Im z, incl. -0).
__host__ __device__ inline zd csqrt(zd z) {
  double x = z.re, y = z.im;
  if (x == 0.0 && y == 0.0) return {0.0, y};
  double r = hypot(x, y);
  if (x >= 0.0) {
    double t = sqrt(0.5 * (r + x));
    return {t, y / (2.0 * t)};
  }
  double t = sqrt(0.5 * (r - x));
  return {fabs(y) / (2.0 * t), copysign(t, y)};
}

__host__ __device__ inline zd cexp(zd z) {
  double e = exp(z.re), s, c;
  sincos(z.im, &s, &c);
  return {e * c, e * s};
}

// e^z - 1 without cancellation for small |z|: expm1(a) cos b - 2 sin^2(b/2) + i e^a sin b.
__host__ __device__ inline zd cexpm1(zd z) {
  double s, c, sh = sin(0.5 * z.im);
  sincos(z.im, &s, &c);
  return {expm1(z.re) * c - 2.0 * sh * sh, exp(z.re) * s};
}

// --------------------------------------------------------- error reporting
void set_error(const std::string& msg);
const char* last_error();

}  // namespace m25

#define M25_CUDA(call)                                                             \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      m25::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));          \
      return M25_ERR_CUDA;                                                         \
    }                                                                              \
  } while (0)

#define M25_CHECK_LAUNCH()                                                         \
  do {                                                                             \
    cudaError_t e_ = cudaGetLastError();                                           \
    if (e_ != cudaSuccess) {                                                       \
      m25::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_));     \
      return M25_ERR_CUDA;                                                         \
    }                                                                              \
  } while (0)
