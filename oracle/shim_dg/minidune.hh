// A minimal grid / discrete-function-space layer of our own, just large
// enough to compile dune-fem's DGEllipticOperator (dune/fem/schemes/
// dgelliptic.hh), LegendreShapeFunctionSet (dune/fem/space/shapefunctionset/
// legendre.hh), TimeProvider (solver/timeprovider.hh),
// ExplicitRungeKuttaSolver (solver/rungekutta/explicit.hh),
// NewtonInverseOperator (solver/newtoninverseoperator.hh),
// FemPreconditioning (solver/fempreconditioning.hh) and SparseRowMatrix
// (operator/matrix/spmatrix.hh) unmodified,
// standing in for dune-common, dune-geometry and dune-grid and the parts of
// dune-fem those headers pull in, which are absent here.  Test
// infrastructure only: built by oracle/make_ref_golden.sh into oracle/_ref/,
// never used by the product.
//
// What it provides, and the reference behaviour each piece restates:
//  - DUNE_THROW and the exception types; DynamicVector / DynamicMatrix;
//    a serial MPIManager; no-op persistence hooks; a ParameterReader over
//    string values with getEnum, and LocalParameter; declarations of the
//    matrix-object templates spmatrix.hh names but these drivers never
//    instantiate;
//    the SpaceOperatorInterface the Runge-Kutta solver calls (operator(),
//    space(), setTime(), timeStepEstimate());
//  - FieldVector / FieldMatrix with the dense operations the two headers call
//    (umv, mmv, usmv, mv, mtv, two_norm, scalar assignment);
//  - an axis-aligned Cartesian grid of N0 x N1 x N2 cells on a box, cells
//    numbered x fastest (YaspGrid's lexicographic order), optionally periodic
//    per direction; a periodic boundary face is a neighbour intersection, as
//    in YaspGrid; intersections of a cell in the order -x,+x,-y,+y,-z,+z;
//  - affine cell geometry: integrationElement = |K|, J^{-T} = diag(1/h);
//  - intersection geometry: |F| as volume and integration element, and
//    integrationOuterNormal = |F| n (face reference element [0,1]^2, whose
//    two coordinates are the cell's other two axes in increasing order);
//  - tensor Gauss quadratures built from the reference's compiled GaussPts:
//    m = the first rule whose order reaches the requested one (order <= 0
//    taken as 1), point index with the first coordinate fastest
//    (quadrature/femquadratures_inline.hh:33-90);
//  - local functions over the Legendre set: values sum dof * phi, gradients
//    are summed in reference coordinates and then mapped by J^{-T}, and axpy
//    adds value * phi + (J^{-1} * factor) . grad_ref phi
//    (space/basisfunctionset/default.hh:225-246, 451-459).
#ifndef GBFEM_SHIM_DG_MINIDUNE_HH
#define GBFEM_SHIM_DG_MINIDUNE_HH

#include <array>
#include <cmath>
#include <cstddef>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include <dune/common/ftraits.hh>
#include <dune/fem/quadrature/gausspoints.hh>

// exceptions (dune/common/exceptions.hh)
#define DUNE_THROW(E, m)                 \
  do {                                   \
    std::ostringstream dune_throw_msg_;  \
    dune_throw_msg_ << m;                \
    throw E(dune_throw_msg_.str());      \
  } while (0)

namespace Dune {

struct Exception : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct InvalidStateException : Exception {
  using Exception::Exception;
};
struct NotImplemented : Exception {
  using Exception::Exception;
};

// dense containers of run-time size (dune/common/dynvector.hh, dynmatrix.hh)
template <class K>
class DynamicVector {
 public:
  DynamicVector() {}
  explicit DynamicVector(std::size_t n, const K& v = K(0)) : d_(n, v) {}
  K& operator[](std::size_t i) { return d_[i]; }
  const K& operator[](std::size_t i) const { return d_[i]; }
  std::size_t size() const { return d_.size(); }
  typename std::vector<K>::iterator begin() { return d_.begin(); }
  typename std::vector<K>::iterator end() { return d_.end(); }
  typename std::vector<K>::const_iterator begin() const { return d_.begin(); }
  typename std::vector<K>::const_iterator end() const { return d_.end(); }

 private:
  std::vector<K> d_;
};

template <class K>
class DynamicMatrix {
 public:
  DynamicMatrix() {}
  DynamicMatrix(std::size_t m, std::size_t n, const K& v = K(0)) : rows_(m, DynamicVector<K>(n, v)) {}
  DynamicVector<K>& operator[](std::size_t i) { return rows_[i]; }
  const DynamicVector<K>& operator[](std::size_t i) const { return rows_[i]; }
  std::size_t rows() const { return rows_.size(); }

 private:
  std::vector<DynamicVector<K>> rows_;
};

template <class K, int n>
class FieldVector {
 public:
  typedef K value_type;
  typedef K field_type;
  static constexpr int dimension = n;
  FieldVector() { for (int i = 0; i < n; ++i) d_[i] = K(0); }
  FieldVector(const K& v) { for (int i = 0; i < n; ++i) d_[i] = v; }
  K& operator[](int i) { return d_[i]; }
  const K& operator[](int i) const { return d_[i]; }
  static constexpr int size() { return n; }
  FieldVector& operator+=(const FieldVector& o) { for (int i = 0; i < n; ++i) d_[i] += o.d_[i]; return *this; }
  FieldVector& operator-=(const FieldVector& o) { for (int i = 0; i < n; ++i) d_[i] -= o.d_[i]; return *this; }
  FieldVector& operator*=(const K& s) { for (int i = 0; i < n; ++i) d_[i] *= s; return *this; }
  FieldVector& operator/=(const K& s) { for (int i = 0; i < n; ++i) d_[i] /= s; return *this; }
  FieldVector operator+(const FieldVector& o) const { FieldVector r(*this); r += o; return r; }
  FieldVector operator-(const FieldVector& o) const { FieldVector r(*this); r -= o; return r; }
  FieldVector operator-() const { FieldVector r(*this); r *= K(-1); return r; }
  FieldVector& axpy(const K& a, const FieldVector& y) { for (int i = 0; i < n; ++i) d_[i] += a * y.d_[i]; return *this; }
  K operator*(const FieldVector& o) const { K s(0); for (int i = 0; i < n; ++i) s += d_[i] * o.d_[i]; return s; }
  K two_norm() const { K s(0); for (int i = 0; i < n; ++i) s += d_[i] * d_[i]; return std::sqrt(s); }

 private:
  K d_[n];
};

template <class K, int r, int c>
class FieldMatrix {
 public:
  typedef FieldVector<K, c> row_type;
  typedef row_type value_type;
  typedef K field_type;
  static constexpr int rows = r;
  static constexpr int cols = c;
  FieldMatrix() {}
  FieldMatrix(const K& v) { for (int i = 0; i < r; ++i) m_[i] = row_type(v); }
  row_type& operator[](int i) { return m_[i]; }
  const row_type& operator[](int i) const { return m_[i]; }
  FieldMatrix& operator+=(const FieldMatrix& o) { for (int i = 0; i < r; ++i) m_[i] += o.m_[i]; return *this; }
  FieldMatrix& operator-=(const FieldMatrix& o) { for (int i = 0; i < r; ++i) m_[i] -= o.m_[i]; return *this; }
  FieldMatrix& operator*=(const K& s) { for (int i = 0; i < r; ++i) m_[i] *= s; return *this; }
  // y = A x
  template <class X, class Y>
  void mv(const X& x, Y& y) const { for (int i = 0; i < r; ++i) { y[i] = K(0); for (int j = 0; j < c; ++j) y[i] += m_[i][j] * x[j]; } }
  // y = A^T x
  template <class X, class Y>
  void mtv(const X& x, Y& y) const { for (int j = 0; j < c; ++j) { y[j] = K(0); for (int i = 0; i < r; ++i) y[j] += m_[i][j] * x[i]; } }
  // y += A x
  template <class X, class Y>
  void umv(const X& x, Y& y) const { for (int i = 0; i < r; ++i) for (int j = 0; j < c; ++j) y[i] += m_[i][j] * x[j]; }
  // y -= A x
  template <class X, class Y>
  void mmv(const X& x, Y& y) const { for (int i = 0; i < r; ++i) for (int j = 0; j < c; ++j) y[i] -= m_[i][j] * x[j]; }
  // y += alpha A x
  template <class X, class Y>
  void usmv(const K& alpha, const X& x, Y& y) const { for (int i = 0; i < r; ++i) for (int j = 0; j < c; ++j) y[i] += alpha * m_[i][j] * x[j]; }

 private:
  row_type m_[r];
};

namespace Fem {

// parameters (dune/fem/io/parameter.hh): string values by key, converted on
// read; getEnum returns the position of the value in a table of names
class ParameterReader {
 public:
  bool exists(const std::string& key) const { return values_.count(key) != 0; }
  template <class T>
  T getValue(const std::string& key, const T& fallback) const {
    auto it = values_.find(key);
    return it == values_.end() ? fallback : convert<T>(it->second);
  }
  template <class T>
  T getValue(const std::string& key) const {
    auto it = values_.find(key);
    if (it == values_.end()) throw std::invalid_argument("missing parameter " + key);
    return convert<T>(it->second);
  }
  template <class T, class Validator>
  T getValidValue(const std::string& key, const T& fallback, const Validator& valid) const {
    const T v = getValue<T>(key, fallback);
    if (!valid(v)) throw std::invalid_argument("invalid value for parameter " + key);
    return v;
  }
  template <class T, class Validator>
  T getValidValue(const std::string& key, const Validator& valid) const {
    const T v = getValue<T>(key);
    if (!valid(v)) throw std::invalid_argument("invalid value for parameter " + key);
    return v;
  }
  template <class Names>
  int getEnum(const std::string& key, const Names& names, int fallback) const {
    auto it = values_.find(key);
    if (it == values_.end()) return fallback;
    for (std::size_t i = 0; i < names.size(); ++i)
      if (names[i] == it->second) return int(i);
    throw std::invalid_argument("parameter " + key + ": unknown value " + it->second);
  }
  void set(const std::string& key, double v) {
    std::ostringstream os;
    os.precision(17);
    os << v;
    values_[key] = os.str();
  }
  void set(const std::string& key, const std::string& v) { values_[key] = v; }

 private:
  template <class T>
  static T convert(const std::string& s) {
    if (std::is_same<T, bool>::value) return T(s == "true" || s == "1");
    std::istringstream is(s);
    double v = 0;
    is >> v;
    return T(v);
  }
  std::map<std::string, std::string> values_;
};
struct Parameter {
  static const int solverStatistics = 1;
  static const int extendedStatistics = 2;
  static ParameterReader& container() { static ParameterReader r; return r; }
  static void append(const std::string& key, const std::string& value, bool = false) { container().set(key, value); }
  static bool verbose(int = 0) { return false; }
};

// parameter classes with a clone() (dune/fem/io/parameter.hh: LocalParameter)
template <class ParamDefault, class ParamImpl>
struct LocalParameter : public ParamDefault {
  virtual ~LocalParameter() {}
  virtual ParamDefault* clone() const { return new ParamImpl(static_cast<const ParamImpl&>(*this)); }
  template <class... Args>
  LocalParameter(Args... args) : ParamDefault(args...) {}
};
template <class ParamDefault>
struct LocalParameter<ParamDefault, ParamDefault> {
  virtual ~LocalParameter() {}
  virtual ParamDefault* clone() const { return new ParamDefault(static_cast<const ParamDefault&>(*this)); }
};

// a serial run (dune/fem/misc/mpimanager.hh)
struct SerialCommunication {
  template <class T>
  T min(const T& x) const { return x; }
  template <class T>
  T max(const T& x) const { return x; }
  template <class T>
  T sum(const T& x) const { return x; }
};
struct MPIManager {
  typedef SerialCommunication Communication;
  static const Communication& comm() { static Communication c; return c; }
  static int thread() { return 0; }
  static int numThreads() { return 1; }
  template <class F>
  static void run(F&& f) { f(); }
};
struct SingleThreadModeError : Exception {
  using Exception::Exception;
};

// checkpointing hooks (dune/fem/io/file/persistencemanager.hh): no-ops here
struct AutoPersistentObject {
  virtual ~AutoPersistentObject() {}
  virtual void backup() const {}
  virtual void restore() {}
};
struct PersistenceManager {
  template <class T>
  static void backupValue(const std::string&, const T&) {}
  template <class T>
  static void restoreValue(const std::string&, T&) {}
};

template <class Grid>
class DofManager;

// the right-hand side of an ODE u' = L(u) (operator/common/spaceoperatorif.hh)
template <class DestinationImp>
struct SpaceOperatorInterface {
  typedef DestinationImp DestinationType;
  typedef typename DestinationImp::DiscreteFunctionSpaceType SpaceType;
  virtual ~SpaceOperatorInterface() {}
  virtual void operator()(const DestinationType& u, DestinationType& w) const = 0;
  virtual const SpaceType& space() const = 0;
  virtual void setTime(const double) {}
  virtual double timeStepEstimate() const { return std::numeric_limits<double>::max(); }
};

// -- operator interfaces (operator/common/operator.hh:55,
//    differentiableoperator.hh:54) ------------------------------------------
template <class DomainFunction, class RangeFunction = DomainFunction>
struct Operator {
  typedef DomainFunction DomainFunctionType;
  typedef RangeFunction RangeFunctionType;
  typedef double DomainFieldType;
  typedef double RangeFieldType;
  virtual ~Operator() {}
  virtual void operator()(const DomainFunction& u, RangeFunction& w) const = 0;
  virtual bool nonlinear() const { return true; }
};
template <class JacobianOperator>
struct DifferentiableOperator
    : public virtual Operator<typename JacobianOperator::DomainFunctionType,
                              typename JacobianOperator::RangeFunctionType> {
  virtual void jacobian(const typename JacobianOperator::DomainFunctionType& u, JacobianOperator& jOp) const = 0;
};

// an operator that holds an assembled matrix (operator/common/operator.hh)
template <class DomainFunction, class RangeFunction = DomainFunction>
struct AssembledOperator : public virtual Operator<DomainFunction, RangeFunction> {};

// declared so that the reference's matrix header parses; not instantiated
template <class Factory>
class ObjectStack;
template <class BlockMapper, int blockSize>
class NonBlockMapper;
template <class Stack>
class LocalMatrixWrapper;
template <class Object>
class ColumnObject;
template <class Traits>
class LocalMatrix;
template <class Traits>
class LocalMatrixDefault;
template <class DomainSpace, class RangeSpace, class Set>
struct StencilWrapper;

// defined in dgspace.hh
template <class DomainSpace, class RangeSpace>
class TemporaryLocalMatrix;
template <class DomainSpace, class RangeSpace>
class DiagonalAndNeighborStencil;

// -- function spaces -------------------------------------------------------
template <int dim>
struct ScalarFunctionSpace {
  static const int dimDomain = dim;
  static const int dimRange = 1;
  typedef double DomainFieldType;
  typedef double RangeFieldType;
  typedef FieldVector<double, dim> DomainType;
  typedef FieldVector<double, 1> RangeType;
  typedef FieldMatrix<double, 1, dim> JacobianRangeType;
  typedef FieldVector<FieldMatrix<double, dim, dim>, 1> HessianRangeType;
};
typedef ScalarFunctionSpace<3> ScalarFunctionSpace3;

// -- grid ------------------------------------------------------------------
struct CartesianGrid {
  int N[3];
  double lower[3], h[3];
  int periodic[3];
  long long ncells() const { return (long long)N[0] * N[1] * N[2]; }
  void coords(long long c, int* x) const {
    x[0] = int(c % N[0]);
    x[1] = int((c / N[0]) % N[1]);
    x[2] = int(c / ((long long)N[0] * N[1]));
  }
  long long index(const int* x) const { return x[0] + (long long)N[0] * (x[1] + (long long)N[1] * x[2]); }
  // neighbour of cell c through face f (-x,+x,-y,+y,-z,+z); -1 on a domain boundary
  long long neighbour(long long c, int f) const {
    int x[3];
    coords(c, x);
    const int dir = f / 2;
    x[dir] += (f % 2) ? 1 : -1;
    if (x[dir] < 0 || x[dir] >= N[dir]) {
      if (!periodic[dir]) return -1;
      x[dir] = (x[dir] + N[dir]) % N[dir];
    }
    return index(x);
  }
  double volume() const { return h[0] * h[1] * h[2]; }
};

class CellGeometry {
 public:
  typedef FieldMatrix<double, 3, 3> JacobianInverseTransposed;
  explicit CellGeometry(const CartesianGrid* g) : g_(g) {}
  double volume() const { return g_->volume(); }
  template <class X>
  double integrationElement(const X&) const { return g_->volume(); }
  template <class X>
  JacobianInverseTransposed jacobianInverseTransposed(const X&) const {
    JacobianInverseTransposed j(0.0);
    for (int k = 0; k < 3; ++k) j[k][k] = 1.0 / g_->h[k];
    return j;
  }

 private:
  const CartesianGrid* g_;
};

class Cell {
 public:
  typedef CellGeometry Geometry;
  Cell() : g_(nullptr), idx_(-1) {}
  Cell(const CartesianGrid* g, long long idx) : g_(g), idx_(idx) {}
  Geometry geometry() const { return Geometry(g_); }
  long long index() const { return idx_; }
  const CartesianGrid* grid() const { return g_; }

 private:
  const CartesianGrid* g_;
  long long idx_;
};

class FaceGeometry {
 public:
  FaceGeometry(const CartesianGrid* g, int dir) : area_(g->volume() / g->h[dir]) {}
  double volume() const { return area_; }
  template <class X>
  double integrationElement(const X&) const { return area_; }

 private:
  double area_;
};

class Face {
 public:
  typedef FaceGeometry Geometry;
  Face(const CartesianGrid* g, long long in, int f) : g_(g), in_(in), f_(f), out_(g->neighbour(in, f)) {}
  bool neighbor() const { return out_ >= 0; }
  bool boundary() const {
    // YaspGrid: a face on the domain boundary is a boundary intersection,
    // periodic or not
    int x[3];
    g_->coords(in_, x);
    const int dir = f_ / 2;
    return (f_ % 2) ? x[dir] == g_->N[dir] - 1 : x[dir] == 0;
  }
  Cell inside() const { return Cell(g_, in_); }
  Cell outside() const { return Cell(g_, out_); }
  Geometry geometry() const { return Geometry(g_, f_ / 2); }
  int indexInInside() const { return f_; }
  int indexInOutside() const { return f_ ^ 1; }
  template <class X>
  FieldVector<double, 3> unitOuterNormal(const X&) const {
    FieldVector<double, 3> n(0.0);
    n[f_ / 2] = (f_ % 2) ? 1.0 : -1.0;
    return n;
  }
  template <class X>
  FieldVector<double, 3> integrationOuterNormal(const X& x) const {
    FieldVector<double, 3> n = unitOuterNormal(x);
    n *= geometry().volume();
    return n;
  }
  const CartesianGrid* grid() const { return g_; }

 private:
  const CartesianGrid* g_;
  long long in_;
  int f_;
  long long out_;
};

class FaceIterator {
 public:
  typedef Face Intersection;
  FaceIterator(const CartesianGrid* g, long long c, int f) : g_(g), c_(c), f_(f) {}
  Face operator*() const { return Face(g_, c_, f_); }
  FaceIterator& operator++() { ++f_; return *this; }
  bool operator!=(const FaceIterator& o) const { return f_ != o.f_ || c_ != o.c_; }
  bool operator==(const FaceIterator& o) const { return !(*this != o); }

 private:
  const CartesianGrid* g_;
  long long c_;
  int f_;
};

class CellIterator {
 public:
  typedef Cell Entity;
  CellIterator(const CartesianGrid* g, long long c) : g_(g), c_(c) {}
  Cell operator*() const { return Cell(g_, c_); }
  CellIterator& operator++() { ++c_; return *this; }
  bool operator!=(const CellIterator& o) const { return c_ != o.c_; }
  bool operator==(const CellIterator& o) const { return c_ == o.c_; }

 private:
  const CartesianGrid* g_;
  long long c_;
};

class GridPart {
 public:
  typedef FaceIterator IntersectionIteratorType;
  typedef Face IntersectionType;
  explicit GridPart(const CartesianGrid* g) : g_(g) {}
  FaceIterator ibegin(const Cell& e) const { return FaceIterator(g_, e.index(), 0); }
  FaceIterator iend(const Cell& e) const { return FaceIterator(g_, e.index(), 6); }
  const CartesianGrid* grid() const { return g_; }

 private:
  const CartesianGrid* g_;
};

// -- quadratures -----------------------------------------------------------
// A quadrature point as handed to local functions and models: the position
// in the reference cell of the element it is evaluated on.
struct ElementPoint {
  FieldVector<double, 3> x;
};
inline const FieldVector<double, 3>& coordinate(const ElementPoint& p) { return p.x; }
template <class K, int d>
inline const FieldVector<K, d>& coordinate(const FieldVector<K, d>& x) { return x; }

inline int gauss_points_for_order(int order) {
  static const GaussPts gp;
  if (order <= 0) order = 1;
  for (int i = 0; i <= GaussPts::MAXP; ++i)
    if (gp.order(i) >= order) return i;
  return -1;
}
inline const GaussPts& gauss_rules() {
  static const GaussPts gp;
  return gp;
}

template <class GridPartT, int codim>
class CachingQuadrature;

template <class GridPartT>
class CachingQuadrature<GridPartT, 0> {
 public:
  typedef FieldVector<double, 3> CoordinateType;
  typedef ElementPoint QuadraturePointWrapperType;
  CachingQuadrature(const Cell&, int order) {
    const int m = gauss_points_for_order(order);
    const GaussPts& gp = gauss_rules();
    for (int i = 0; i < m * m * m; ++i) {
      int z = i;
      ElementPoint p;
      double w = 1.0;
      for (int k = 0; k < 3; ++k) {
        const int xk = z % m;
        z /= m;
        p.x[k] = gp.point(m, xk);
        w *= gp.weight(m, xk);
      }
      pts_.push_back(p);
      wts_.push_back(w);
    }
  }
  std::size_t nop() const { return pts_.size(); }
  const CoordinateType& point(std::size_t i) const { return pts_[i].x; }
  double weight(std::size_t i) const { return wts_[i]; }
  const ElementPoint& operator[](std::size_t i) const { return pts_[i]; }

 private:
  std::vector<ElementPoint> pts_;
  std::vector<double> wts_;
};

template <class GridPartT, int codim>
class ElementQuadrature;

template <class GridPartT>
class ElementQuadrature<GridPartT, 1> {
 public:
  enum Side { INSIDE, OUTSIDE };
  typedef FieldVector<double, 2> LocalCoordinateType;
  typedef FieldVector<double, 3> CoordinateType;
  ElementQuadrature(const GridPartT&, const Face& face, int order, Side side) {
    const int m = gauss_points_for_order(order);
    const GaussPts& gp = gauss_rules();
    const int f = side == INSIDE ? face.indexInInside() : face.indexInOutside();
    const int dir = f / 2;
    int axes[2], a = 0;
    for (int k = 0; k < 3; ++k)
      if (k != dir) axes[a++] = k;
    for (int i = 0; i < m * m; ++i) {
      const int s = i % m, t = i / m;
      LocalCoordinateType xl;
      xl[0] = gp.point(m, s);
      xl[1] = gp.point(m, t);
      ElementPoint p;
      p.x[dir] = (f % 2) ? 1.0 : 0.0;
      p.x[axes[0]] = xl[0];
      p.x[axes[1]] = xl[1];
      local_.push_back(xl);
      pts_.push_back(p);
      wts_.push_back(gp.weight(m, s) * gp.weight(m, t));
    }
  }
  std::size_t nop() const { return pts_.size(); }
  const LocalCoordinateType& localPoint(std::size_t i) const { return local_[i]; }
  const CoordinateType& point(std::size_t i) const { return pts_[i].x; }
  double weight(std::size_t i) const { return wts_[i]; }
  const ElementPoint& operator[](std::size_t i) const { return pts_[i]; }

 private:
  std::vector<LocalCoordinateType> local_;
  std::vector<ElementPoint> pts_;
  std::vector<double> wts_;
};

}  // namespace Fem
}  // namespace Dune

#endif
