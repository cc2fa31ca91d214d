// aero_dual.cuh -- forward-mode dual numbers for the discrete adjoint: a value and N
// directional derivatives, propagated exactly through +, -, *, /, sqrt, |.|, and the
// max/min/clamp selections of aero_numerics.cuh (a selection passes the derivative of the
// branch it takes, so the result is the derivative of the arithmetic actually executed).
//
// The numerics are templates on their real type, so evaluating them with Dual<N> gives the
// local Jacobian of a face flux with respect to N seeded inputs without a second copy of the
// flux code. The functions live in aero::ad and are found by argument-dependent lookup (the
// numerics' sabs / ssqrt / sfinite call fabs / sqrt / isfinite unqualified), so they never
// hide the double overloads used elsewhere in namespace aero.
#pragma once

#include "aero_numerics.cuh"

namespace aero {
namespace ad {

template <int N>
struct Dual {
  double v;
  double d[N];
  __host__ __device__ constexpr Dual() : v(0.0), d{} {}
  __host__ __device__ constexpr Dual(double x) : v(x), d{} {}  // NOLINT: constants convert
};

template <int N>
__host__ __device__ __forceinline__ Dual<N> seed(double x, int k) {
  Dual<N> r(x);
  r.d[k] = 1.0;
  return r;
}

#define AERO_DUAL_LOOP for (int i = 0; i < N; ++i)

template <int N>
__host__ __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
  AERO_DUAL_LOOP r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
  AERO_DUAL_LOOP r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
  AERO_DUAL_LOOP r.d[i] = -a.d[i];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
  AERO_DUAL_LOOP r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  const double inv = 1.0 / b.v;
  r.v = a.v * inv;
  AERO_DUAL_LOOP r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) {
  a = a + b;
  return a;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) {
  a = a - b;
  return a;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) {
  a = a * b;
  return a;
}
// mixed with plain doubles (the constants of the numerics)
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
  AERO_DUAL_LOOP r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N>
__host__ __device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }

// comparisons act on the value
template <int N>
__host__ __device__ __forceinline__ bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator==(const Dual<N>& a, const Dual<N>& b) { return a.v == b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator!=(const Dual<N>& a, const Dual<N>& b) { return a.v != b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N>
__host__ __device__ __forceinline__ bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N>
__host__ __device__ __forceinline__ bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }
template <int N>
__host__ __device__ __forceinline__ bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }
template <int N>
__host__ __device__ __forceinline__ bool operator<(double a, const Dual<N>& b) { return a < b.v; }
template <int N>
__host__ __device__ __forceinline__ bool operator>(double a, const Dual<N>& b) { return a > b.v; }

template <int N>
__host__ __device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double h = r.v > 0.0 ? 0.5 / r.v : 0.0;  // sqrt is only taken of clamped, non-negative values
  AERO_DUAL_LOOP r.d[i] = a.d[i] * h;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) {
  return a.v < 0.0 ? -a : a;
}
template <int N>
__host__ __device__ __forceinline__ bool isfinite(const Dual<N>& a) {
  return ::isfinite(a.v);
}

// The numerics' floors (Kn<T>) stay plain doubles for duals: a class-type static constant
// has no device storage. These overloads take them where the numerics mix them with T.
template <int N>
__host__ __device__ __forceinline__ Dual<N> smax(const Dual<N>& a, double b) {
  return ::aero::smax(a, Dual<N>(b));
}
template <int N>
__host__ __device__ __forceinline__ Dual<N> sclamp(const Dual<N>& v, double lo, const Dual<N>& hi) {
  return ::aero::sclamp(v, Dual<N>(lo), hi);
}

#undef AERO_DUAL_LOOP

}  // namespace ad

template <int N>
struct Kn<ad::Dual<N>> {
  static constexpr double rho_floor = Kn<double>::rho_floor;
  static constexpr double p_floor = Kn<double>::p_floor;
  static constexpr double wave_floor = Kn<double>::wave_floor;
  static constexpr double low_mach_min = Kn<double>::low_mach_min;
  static constexpr double all_speed_floor = Kn<double>::all_speed_floor;
  static constexpr double smooth_eps = Kn<double>::smooth_eps;
  static constexpr double vol_floor = Kn<double>::vol_floor;
};

}  // namespace aero
