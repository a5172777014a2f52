// Forward-mode dual numbers for the run-time compiled DG forms.
//
// Dual<T> carries a value and one directional derivative.  T is float,
// double or itself a Dual: the form kernels evaluate the user's pointwise
// functions on Dual<R> to get the Jacobian-vector product of the whole
// discrete operator, and the generated SIPG face terms need the derivative
// of the flux with respect to the gradient inside that, i.e. Dual<Dual<R>>.
// Every function below works at any nesting depth: the value comes from the
// CUDA math function at the innermost level and the derivative from the
// chain rule.
#pragma once
#include <type_traits>

namespace gbfem {
namespace form {

template <typename S>
using Scalar = typename std::enable_if<std::is_arithmetic<S>::value>::type;

// innermost-level math: CUDA's functions for float and double
#define GBFEM_FORM_UNARY(name, fname)                                  \
  __device__ __forceinline__ double name(double a) { return ::name(a); } \
  __device__ __forceinline__ float name(float a) { return ::fname(a); }
GBFEM_FORM_UNARY(exp, expf)
GBFEM_FORM_UNARY(log, logf)
GBFEM_FORM_UNARY(sqrt, sqrtf)
GBFEM_FORM_UNARY(sin, sinf)
GBFEM_FORM_UNARY(cos, cosf)
GBFEM_FORM_UNARY(tan, tanf)
GBFEM_FORM_UNARY(tanh, tanhf)
GBFEM_FORM_UNARY(sinh, sinhf)
GBFEM_FORM_UNARY(cosh, coshf)
GBFEM_FORM_UNARY(atan, atanf)
GBFEM_FORM_UNARY(fabs, fabsf)
#undef GBFEM_FORM_UNARY
__device__ __forceinline__ double pow(double a, double b) { return ::pow(a, b); }
__device__ __forceinline__ float pow(float a, float b) { return ::powf(a, b); }
__device__ __forceinline__ double value(double a) { return a; }
__device__ __forceinline__ float value(float a) { return a; }

template <typename T>
struct Dual {
  T v, d;
  __device__ Dual() : v(0), d(0) {}
  __device__ Dual(const T& a, const T& b) : v(a), d(b) {}
  __device__ Dual(const T& a) : v(a), d(0) {}
  template <typename S, typename = Scalar<S>>
  __device__ Dual(S a) : v(T(a)), d(0) {}
};

// the value at the innermost level (for comparisons and selections)
template <typename T>
__device__ __forceinline__ auto value(const Dual<T>& a) -> decltype(value(a.v)) {
  return value(a.v);
}

template <typename T> __device__ __forceinline__ Dual<T> operator+(const Dual<T>& a) { return a; }
template <typename T> __device__ __forceinline__ Dual<T> operator-(const Dual<T>& a) { return Dual<T>(-a.v, -a.d); }
template <typename T> __device__ __forceinline__ Dual<T> operator+(const Dual<T>& a, const Dual<T>& b) {
  return Dual<T>(a.v + b.v, a.d + b.d);
}
template <typename T> __device__ __forceinline__ Dual<T> operator-(const Dual<T>& a, const Dual<T>& b) {
  return Dual<T>(a.v - b.v, a.d - b.d);
}
template <typename T> __device__ __forceinline__ Dual<T> operator*(const Dual<T>& a, const Dual<T>& b) {
  return Dual<T>(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <typename T> __device__ __forceinline__ Dual<T> operator/(const Dual<T>& a, const Dual<T>& b) {
  const T q = a.v / b.v;
  return Dual<T>(q, (a.d - q * b.d) / b.v);
}
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator+(const Dual<T>& a, S b) { return Dual<T>(a.v + b, a.d); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator+(S a, const Dual<T>& b) { return Dual<T>(a + b.v, b.d); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator-(const Dual<T>& a, S b) { return Dual<T>(a.v - b, a.d); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator-(S a, const Dual<T>& b) { return Dual<T>(a - b.v, -b.d); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator*(const Dual<T>& a, S b) { return Dual<T>(a.v * b, a.d * b); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator*(S a, const Dual<T>& b) { return Dual<T>(a * b.v, a * b.d); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator/(const Dual<T>& a, S b) { return Dual<T>(a.v / b, a.d / b); }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> operator/(S a, const Dual<T>& b) { return Dual<T>(a) / b; }

template <typename T, typename U> __device__ __forceinline__ Dual<T>& operator+=(Dual<T>& a, const U& b) { return a = a + b; }
template <typename T, typename U> __device__ __forceinline__ Dual<T>& operator-=(Dual<T>& a, const U& b) { return a = a - b; }
template <typename T, typename U> __device__ __forceinline__ Dual<T>& operator*=(Dual<T>& a, const U& b) { return a = a * b; }
template <typename T, typename U> __device__ __forceinline__ Dual<T>& operator/=(Dual<T>& a, const U& b) { return a = a / b; }

// comparisons look at the value only
#define GBFEM_FORM_CMP(op)                                                                            \
  template <typename T> __device__ __forceinline__ bool operator op(const Dual<T>& a, const Dual<T>& b) { \
    return value(a) op value(b);                                                                      \
  }                                                                                                   \
  template <typename T, typename S, typename = Scalar<S>>                                             \
  __device__ __forceinline__ bool operator op(const Dual<T>& a, S b) { return value(a) op b; }          \
  template <typename T, typename S, typename = Scalar<S>>                                             \
  __device__ __forceinline__ bool operator op(S a, const Dual<T>& b) { return a op value(b); }
GBFEM_FORM_CMP(<)
GBFEM_FORM_CMP(<=)
GBFEM_FORM_CMP(>)
GBFEM_FORM_CMP(>=)
#undef GBFEM_FORM_CMP

// elementary functions, recursively (T may itself be a Dual)
template <typename T> __device__ __forceinline__ Dual<T> exp(const Dual<T>& a) {
  const T e = exp(a.v);
  return Dual<T>(e, a.d * e);
}
template <typename T> __device__ __forceinline__ Dual<T> log(const Dual<T>& a) { return Dual<T>(log(a.v), a.d / a.v); }
template <typename T> __device__ __forceinline__ Dual<T> sqrt(const Dual<T>& a) {
  const T r = sqrt(a.v);
  return Dual<T>(r, a.d / (r * 2.0f));
}
template <typename T> __device__ __forceinline__ Dual<T> sin(const Dual<T>& a) { return Dual<T>(sin(a.v), a.d * cos(a.v)); }
template <typename T> __device__ __forceinline__ Dual<T> cos(const Dual<T>& a) { return Dual<T>(cos(a.v), -(a.d * sin(a.v))); }
template <typename T> __device__ __forceinline__ Dual<T> tan(const Dual<T>& a) {
  const T t = tan(a.v);
  return Dual<T>(t, a.d * (t * t + 1.0f));
}
template <typename T> __device__ __forceinline__ Dual<T> tanh(const Dual<T>& a) {
  const T t = tanh(a.v);
  return Dual<T>(t, a.d * (1.0f - t * t));
}
template <typename T> __device__ __forceinline__ Dual<T> sinh(const Dual<T>& a) { return Dual<T>(sinh(a.v), a.d * cosh(a.v)); }
template <typename T> __device__ __forceinline__ Dual<T> cosh(const Dual<T>& a) { return Dual<T>(cosh(a.v), a.d * sinh(a.v)); }
template <typename T> __device__ __forceinline__ Dual<T> atan(const Dual<T>& a) {
  return Dual<T>(atan(a.v), a.d / (a.v * a.v + 1.0f));
}
template <typename T> __device__ __forceinline__ Dual<T> fabs(const Dual<T>& a) { return value(a) < 0 ? -a : a; }
template <typename T, typename S, typename = Scalar<S>>
__device__ __forceinline__ Dual<T> pow(const Dual<T>& a, S p) {
  using R = decltype(value(a));
  const R pr = R(p);
  return Dual<T>(pow(a.v, pr), a.d * (pow(a.v, pr - R(1)) * pr));
}
template <typename T> __device__ __forceinline__ Dual<T> pow(const Dual<T>& a, const Dual<T>& b) { return exp(b * log(a)); }
// integer powers by repeated multiplication (any type)
template <int P, typename T> __device__ __forceinline__ T ipow(const T& a) {
  T r = a;
  for (int i = 1; i < P; ++i) r = r * a;
  return r;
}
template <typename T> __device__ __forceinline__ T max(const T& a, const T& b) { return value(a) >= value(b) ? a : b; }
template <typename T> __device__ __forceinline__ T min(const T& a, const T& b) { return value(a) <= value(b) ? a : b; }

// fma of a real table entry with a value of the kernel's type
__device__ __forceinline__ double vfma(double m, double x, double acc) { return ::fma(m, x, acc); }
__device__ __forceinline__ float vfma(float m, float x, float acc) { return ::fmaf(m, x, acc); }
template <typename R, typename T> __device__ __forceinline__ Dual<T> vfma(R m, const Dual<T>& x, const Dual<T>& acc) {
  return Dual<T>(vfma(m, x.v, acc.v), vfma(m, x.d, acc.d));
}
// the derivative part of a first-level dual (0 for a plain value)
__device__ __forceinline__ double tangent(double) { return 0.0; }
__device__ __forceinline__ float tangent(float) { return 0.0f; }
template <typename R> __device__ __forceinline__ R tangent(const Dual<R>& a) { return a.d; }

}  // namespace form
}  // namespace gbfem
