// Support for user-defined pointwise reaction terms compiled at run time.
//
// The counterpart of the reference's UFL code generation for an integrand
// r(u, x) v dx (python/dune/models/integrands/ufl.py generates the C++ of the
// integrand; schemes/galerkin.hh:332-410 integrates it and its linearisation).
// Here the user writes r as a CUDA C++ expression in u, x, y, z; the
// integrands module of the Python package wraps it in a functor, instantiates
// the reaction kernel of reaction_kernel.cuh for the operator's precision,
// order and quadrature, and compiles it with nvcc into an sm_103a cubin that
// gbfem_dg_nonlinear_operator_create_jit loads.  The derivative r'(u) needed
// by the Jacobian comes from forward-mode dual numbers: the expression is
// evaluated once with u = (u, 1) and coordinates (x, 0).
#pragma once
#include <type_traits>

#include "reaction_kernel.cuh"

namespace gbfem {
namespace jit {

template <typename T>
struct Dual {
  T v, d;
  __device__ Dual() : v(T(0)), d(T(0)) {}
  __device__ Dual(T a, T b = T(0)) : v(a), d(b) {}
};

template <typename S>
using Scalar = typename std::enable_if<std::is_arithmetic<S>::value>::type;

template <typename T> __device__ Dual<T> operator+(Dual<T> a) { return a; }
template <typename T> __device__ Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }
template <typename T> __device__ Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <typename T> __device__ Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <typename T> __device__ Dual<T> operator*(Dual<T> a, Dual<T> b) {
  return Dual<T>(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <typename T> __device__ Dual<T> operator/(Dual<T> a, Dual<T> b) {
  return Dual<T>(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v));
}
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator+(Dual<T> a, S b) { return a + Dual<T>(T(b)); }
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator+(S a, Dual<T> b) { return Dual<T>(T(a)) + b; }
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator-(Dual<T> a, S b) { return a - Dual<T>(T(b)); }
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator-(S a, Dual<T> b) { return Dual<T>(T(a)) - b; }
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator*(Dual<T> a, S b) {
  return Dual<T>(a.v * T(b), a.d * T(b));
}
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator*(S a, Dual<T> b) {
  return Dual<T>(T(a) * b.v, T(a) * b.d);
}
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator/(Dual<T> a, S b) {
  return Dual<T>(a.v / T(b), a.d / T(b));
}
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> operator/(S a, Dual<T> b) {
  return Dual<T>(T(a)) / b;
}

// elementary functions: value from CUDA's function, derivative by the chain rule
template <typename T> __device__ Dual<T> exp(Dual<T> a) { const T e = ::exp(a.v); return Dual<T>(e, a.d * e); }
template <typename T> __device__ Dual<T> log(Dual<T> a) { return Dual<T>(::log(a.v), a.d / a.v); }
template <typename T> __device__ Dual<T> sqrt(Dual<T> a) { const T r = ::sqrt(a.v); return Dual<T>(r, a.d / (T(2) * r)); }
template <typename T> __device__ Dual<T> sin(Dual<T> a) { return Dual<T>(::sin(a.v), a.d * ::cos(a.v)); }
template <typename T> __device__ Dual<T> cos(Dual<T> a) { return Dual<T>(::cos(a.v), -a.d * ::sin(a.v)); }
template <typename T> __device__ Dual<T> tanh(Dual<T> a) { const T t = ::tanh(a.v); return Dual<T>(t, a.d * (T(1) - t * t)); }
template <typename T> __device__ Dual<T> sinh(Dual<T> a) { return Dual<T>(::sinh(a.v), a.d * ::cosh(a.v)); }
template <typename T> __device__ Dual<T> cosh(Dual<T> a) { return Dual<T>(::cosh(a.v), a.d * ::sinh(a.v)); }
template <typename T> __device__ Dual<T> atan(Dual<T> a) { return Dual<T>(::atan(a.v), a.d / (T(1) + a.v * a.v)); }
template <typename T> __device__ Dual<T> fabs(Dual<T> a) { return a.v < T(0) ? -a : a; }
template <typename T, typename S, typename = Scalar<S>> __device__ Dual<T> pow(Dual<T> a, S p) {
  const T e = T(p);
  return Dual<T>(::pow(a.v, e), a.d * e * ::pow(a.v, e - T(1)));
}
// integer powers by repeated multiplication (exact derivative, no pow call)
template <int P, typename T> __device__ Dual<T> ipow(Dual<T> a) {
  Dual<T> r(T(1));
  for (int i = 0; i < P; ++i) r = r * a;
  return r;
}

// Wraps a user functor F (template <class D> D operator()(D u, D x, D y, D z))
// as the pointwise function of dg_reaction_body.
template <class F>
struct UserReaction {
  static constexpr bool kCoordinates = true;
  template <typename T>
  __device__ static T value(const ReactTabsT<T>&, T u, T x, T y, T z) {
    return F()(Dual<T>(u), Dual<T>(x), Dual<T>(y), Dual<T>(z)).v;
  }
  template <typename T>
  __device__ static T derivative(const ReactTabsT<T>&, T u, T x, T y, T z) {
    return F()(Dual<T>(u, T(1)), Dual<T>(x), Dual<T>(y), Dual<T>(z)).d;
  }
};

}  // namespace jit
}  // namespace gbfem
