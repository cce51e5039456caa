// Forward-mode dual numbers for the residual's Jacobian-vector product.
//
// A Dual carries a value and one directional derivative.  The residual
// kernels are templates on their state scalar (double for the residual,
// Dual for the tangent): every branch (limiter selections, flux switches,
// min/max) is decided on the value, and the derivative follows the branch
// taken, i.e. the exact derivative of the piecewise-smooth discrete
// residual wherever it is differentiable.
#pragma once

#include <cuda_runtime.h>

namespace ics {

struct Dual {
  double v, d;
  Dual() = default;
  __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}
  __host__ __device__ constexpr Dual(double x, double dx) : v(x), d(dx) {}
};

__host__ __device__ __forceinline__ double val(double x) { return x; }
__host__ __device__ __forceinline__ double val(const Dual& x) { return x.v; }
__host__ __device__ __forceinline__ double tan_of(double) { return 0.0; }
__host__ __device__ __forceinline__ double tan_of(const Dual& x) { return x.d; }

__host__ __device__ __forceinline__ Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
__host__ __device__ __forceinline__ Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
__host__ __device__ __forceinline__ Dual operator+(const Dual& a, double b) { return Dual(a.v + b, a.d); }
__host__ __device__ __forceinline__ Dual operator+(double a, const Dual& b) { return Dual(a + b.v, b.d); }
__host__ __device__ __forceinline__ Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
__host__ __device__ __forceinline__ Dual operator-(const Dual& a, double b) { return Dual(a.v - b, a.d); }
__host__ __device__ __forceinline__ Dual operator-(double a, const Dual& b) { return Dual(a - b.v, -b.d); }
__host__ __device__ __forceinline__ Dual operator*(const Dual& a, const Dual& b) {
  return Dual(a.v * b.v, a.d * b.v + a.v * b.d);
}
__host__ __device__ __forceinline__ Dual operator*(const Dual& a, double b) { return Dual(a.v * b, a.d * b); }
__host__ __device__ __forceinline__ Dual operator*(double a, const Dual& b) { return Dual(a * b.v, a * b.d); }
__host__ __device__ __forceinline__ Dual operator/(const Dual& a, const Dual& b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__host__ __device__ __forceinline__ Dual operator/(const Dual& a, double b) { return Dual(a.v / b, a.d / b); }
__host__ __device__ __forceinline__ Dual operator/(double a, const Dual& b) {
  const double q = a / b.v;
  return Dual(q, -q * b.d / b.v);
}
__host__ __device__ __forceinline__ Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
__host__ __device__ __forceinline__ Dual& operator-=(Dual& a, const Dual& b) { return a = a - b; }
__host__ __device__ __forceinline__ Dual& operator*=(Dual& a, const Dual& b) { return a = a * b; }
__host__ __device__ __forceinline__ Dual& operator/=(Dual& a, const Dual& b) { return a = a / b; }

#define ICS_DUAL_CMP(op)                                                                                   \
  __host__ __device__ __forceinline__ bool operator op(const Dual& a, const Dual& b) { return a.v op b.v; } \
  __host__ __device__ __forceinline__ bool operator op(const Dual& a, double b) { return a.v op b; }        \
  __host__ __device__ __forceinline__ bool operator op(double a, const Dual& b) { return a op b.v; }
ICS_DUAL_CMP(<)
ICS_DUAL_CMP(>)
ICS_DUAL_CMP(<=)
ICS_DUAL_CMP(>=)
ICS_DUAL_CMP(==)
ICS_DUAL_CMP(!=)
#undef ICS_DUAL_CMP

// The Dual overloads below hide the global functions inside namespace ics;
// these forward the plain double and float calls to them.
__host__ __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
__host__ __device__ __forceinline__ double fabs(double x) { return ::fabs(x); }
__host__ __device__ __forceinline__ double fmax(double a, double b) { return ::fmax(a, b); }
__host__ __device__ __forceinline__ double fmin(double a, double b) { return ::fmin(a, b); }
__host__ __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
__host__ __device__ __forceinline__ float fabs(float x) { return ::fabsf(x); }
__host__ __device__ __forceinline__ float fmax(float a, float b) { return ::fmaxf(a, b); }
__host__ __device__ __forceinline__ float fmin(float a, float b) { return ::fminf(a, b); }

__host__ __device__ __forceinline__ Dual sqrt(const Dual& a) {
  const double s = ::sqrt(a.v);
  return Dual(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
}
__host__ __device__ __forceinline__ Dual fabs(const Dual& a) { return a.v >= 0.0 ? a : -a; }
__host__ __device__ __forceinline__ Dual fmax(const Dual& a, const Dual& b) { return a.v >= b.v ? a : b; }
__host__ __device__ __forceinline__ Dual fmax(const Dual& a, double b) { return a.v >= b ? a : Dual(b); }
__host__ __device__ __forceinline__ Dual fmax(double a, const Dual& b) { return a >= b.v ? Dual(a) : b; }
__host__ __device__ __forceinline__ Dual fmin(const Dual& a, const Dual& b) { return a.v <= b.v ? a : b; }
__host__ __device__ __forceinline__ Dual fmin(const Dual& a, double b) { return a.v <= b ? a : Dual(b); }
__host__ __device__ __forceinline__ Dual fmin(double a, const Dual& b) { return a <= b.v ? Dual(a) : b; }

// Order-preserving integer image of a double: key(a) < key(b) exactly when
// a < b for finite values (and -0 < +0).  Comparisons, min and max of doubles
// through it run on the integer pipes, which on GB300 issue many times faster
// than the FP64 pipe that DSETP / DMNMX would occupy; the selected operand is
// returned unchanged.  The Dual forms decide on the value and keep the chosen
// operand's derivative, as fmax / fmin above do.
__device__ __forceinline__ long long okey(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ long long okey(const Dual& x) { return okey(x.v); }
template <typename Real>
__device__ __forceinline__ Real omax(const Real& a, const Real& b) {
  return okey(a) >= okey(b) ? a : b;
}
template <typename Real>
__device__ __forceinline__ Real omin(const Real& a, const Real& b) {
  return okey(a) <= okey(b) ? a : b;
}
// x > c and x < c for a constant c
template <typename Real>
__device__ __forceinline__ bool ogt(const Real& x, double c) {
  return okey(x) > okey(c);
}
template <typename Real>
__device__ __forceinline__ bool olt(const Real& x, double c) {
  return okey(x) < okey(c);
}

}  // namespace ics
