// The DG space, discrete function and local-function classes of the shim
// layer (see minidune.hh): a scalar discontinuous space over the reference's
// own LegendreShapeFunctionSet (legendre.hh, non-hierarchical ordering),
// dofs stored cell by cell (dof = cell * size + local), as the reference's
// DG block mapper lays them out.  Test infrastructure only.
#ifndef GBFEM_SHIM_DG_DGSPACE_HH
#define GBFEM_SHIM_DG_DGSPACE_HH

#include <algorithm>
#include <string>
#include <vector>

#include "minidune.hh"
#include <dune/fem/space/shapefunctionset/legendre.hh>

namespace Dune {
namespace Fem {

class LegendreDGSpace;

// The basis of one cell (DefaultBasisFunctionSet): values and gradients of
// all shape functions at a point, gradients mapped by J^{-T}
// (space/basisfunctionset/default.hh:276-330, 361-372).
class LegendreBasisFunctionSet {
 public:
  typedef ScalarFunctionSpace3::RangeType RangeType;
  typedef ScalarFunctionSpace3::JacobianRangeType JacobianRangeType;
  LegendreBasisFunctionSet() : space_(nullptr) {}
  LegendreBasisFunctionSet(const LegendreDGSpace* s, const Cell& c) : space_(s), cell_(c) {}
  inline std::size_t size() const;
  template <class Point>
  void evaluateAll(const Point& x, std::vector<RangeType>& phi) const;
  template <class Point>
  void jacobianAll(const Point& x, std::vector<JacobianRangeType>& dphi) const;

 private:
  const LegendreDGSpace* space_;
  Cell cell_;
};

struct BlockMapper {
  std::size_t n;
  std::size_t maxNumDofs() const { return n; }
};

class LegendreDGSpace {
 public:
  typedef ScalarFunctionSpace3 FunctionSpaceType;
  typedef FunctionSpaceType::DomainType DomainType;
  typedef FunctionSpaceType::RangeType RangeType;
  typedef FunctionSpaceType::JacobianRangeType JacobianRangeType;
  typedef GridPart GridPartType;
  typedef CellIterator IteratorType;
  typedef LegendreShapeFunctionSet<FunctionSpaceType, false> ShapeFunctionSetType;
  typedef LegendreBasisFunctionSet BasisFunctionSetType;
  static const int localBlockSize = 1;

  // reported_order: the polynomial order that local functions report to the
  // operator, which chooses its quadrature from it (order() of u plus order()
  // of w); it is the space's order unless a finer rule is wanted
  LegendreDGSpace(const CartesianGrid& g, int order, int reported_order)
      : grid_(g), gridPart_(&grid_), shapes_(order), order_(order), reported_(reported_order) {}
  IteratorType begin() const { return IteratorType(&grid_, 0); }
  IteratorType end() const { return IteratorType(&grid_, grid_.ncells()); }
  const GridPartType& gridPart() const { return gridPart_; }
  bool continuous() const { return false; }
  int order() const { return order_; }
  int reportedOrder() const { return reported_; }
  std::size_t localSize() const { return shapes_.size(); }
  std::size_t size() const { return shapes_.size() * grid_.ncells(); }
  const ShapeFunctionSetType& shapeFunctionSet() const { return shapes_; }
  BasisFunctionSetType basisFunctionSet(const Cell& c) const { return BasisFunctionSetType(this, c); }
  BlockMapper blockMapper() const { return BlockMapper{shapes_.size()}; }
  const CartesianGrid& grid() const { return grid_; }

 private:
  CartesianGrid grid_;
  GridPart gridPart_;
  ShapeFunctionSetType shapes_;
  int order_, reported_;
};

inline std::size_t LegendreBasisFunctionSet::size() const { return space_->localSize(); }
template <class Point>
void LegendreBasisFunctionSet::evaluateAll(const Point& x, std::vector<RangeType>& phi) const {
  space_->shapeFunctionSet().evaluateEach(x, [&](std::size_t i, const RangeType& v) { phi[i] = v; });
}
template <class Point>
void LegendreBasisFunctionSet::jacobianAll(const Point& x, std::vector<JacobianRangeType>& dphi) const {
  const auto jit = cell_.geometry().jacobianInverseTransposed(coordinate(x));
  space_->shapeFunctionSet().jacobianEach(x, [&](std::size_t i, const JacobianRangeType& d) {
    jit.mv(d[0], dphi[i][0]);
  });
}

struct LocalFunctionTraits {
  typedef LegendreDGSpace::RangeType RangeType;
  typedef LegendreDGSpace::JacobianRangeType JacobianRangeType;
  typedef double RangeFieldType;
  static const int dimDomain = 3;
  static const int dimRange = 1;
};

// The dof vector as the reference's block vectors present it (blocks of
// one dof): find(i) gives an iterator at dof i, [i][0] the dof.
class DofBlockView {
 public:
  explicit DofBlockView(double* d) : d_(d) {}
  double* find(std::size_t i) const { return d_ + i; }
  double* operator[](std::size_t i) const { return d_ + i; }

 private:
  double* d_;
};

class DGFunction {
 public:
  typedef LegendreDGSpace DiscreteFunctionSpaceType;
  typedef LocalFunctionTraits LocalFunctionType;
  typedef double DofType;
  typedef double* DofIteratorType;
  typedef const double* ConstDofIteratorType;
  explicit DGFunction(const LegendreDGSpace& s) : space_(&s), dofs_(s.size(), 0.0) {}
  DGFunction(const std::string&, const LegendreDGSpace& s) : DGFunction(s) {}
  const LegendreDGSpace& space() const { return *space_; }
  void clear() { std::fill(dofs_.begin(), dofs_.end(), 0.0); }
  void assign(const DGFunction& o) { dofs_ = o.dofs_; }
  DGFunction& operator-=(const DGFunction& o) {
    for (std::size_t i = 0; i < dofs_.size(); ++i) dofs_[i] -= o.dofs_[i];
    return *this;
  }
  double scalarProductDofs(const DGFunction& o) const {
    double s = 0.0;
    for (std::size_t i = 0; i < dofs_.size(); ++i) s += dofs_[i] * o.dofs_[i];
    return s;
  }
  void axpy(double a, const DGFunction& x) {
    for (std::size_t i = 0; i < dofs_.size(); ++i) dofs_[i] += a * x.dofs_[i];
  }
  void communicate() {}
  DofIteratorType dbegin() { return dofs_.data(); }
  DofIteratorType dend() { return dofs_.data() + dofs_.size(); }
  ConstDofIteratorType dbegin() const { return dofs_.data(); }
  ConstDofIteratorType dend() const { return dofs_.data() + dofs_.size(); }
  DofBlockView dofVector() const { return DofBlockView(const_cast<double*>(dofs_.data())); }
  std::vector<double>& dofs() { return dofs_; }
  const std::vector<double>& dofs() const { return dofs_; }

 private:
  const LegendreDGSpace* space_;
  std::vector<double> dofs_;
};

// Evaluation of a discrete function on one cell (ConstLocalFunction).
template <class GF>
class ConstLocalFunction {
 public:
  typedef LocalFunctionTraits::RangeType RangeType;
  typedef LocalFunctionTraits::JacobianRangeType JacobianRangeType;
  explicit ConstLocalFunction(const GF& f) : f_(&f) {}
  void bind(const Cell& e) { cell_ = e; }
  void unbind() { cell_ = Cell(); }
  int order() const { return f_->space().reportedOrder(); }
  template <class Point>
  void evaluate(const Point& x, RangeType& value) const {
    const double* u = dofs();
    value = RangeType(0.0);
    f_->space().shapeFunctionSet().evaluateEach(x, [&](std::size_t i, const RangeType& phi) {
      value[0] += u[i] * phi[0];
    });
  }
  template <class Point>
  void jacobian(const Point& x, JacobianRangeType& jac) const {
    const double* u = dofs();
    JacobianRangeType ref(0.0);
    f_->space().shapeFunctionSet().jacobianEach(x, [&](std::size_t i, const JacobianRangeType& dphi) {
      for (int k = 0; k < 3; ++k) ref[0][k] += u[i] * dphi[0][k];
    });
    const auto jit = cell_.geometry().jacobianInverseTransposed(coordinate(x));
    jit.mv(ref[0], jac[0]);
  }

 private:
  const double* dofs() const { return f_->dofs().data() + cell_.index() * f_->space().localSize(); }
  const GF* f_;
  Cell cell_;
};

// Accumulation into a discrete function on one cell (AddLocalContribution):
// contributions are gathered locally and added to the global vector on
// unbind.
template <class DF>
class AddLocalContribution {
 public:
  typedef LocalFunctionTraits::RangeType RangeType;
  typedef LocalFunctionTraits::JacobianRangeType JacobianRangeType;
  explicit AddLocalContribution(DF& f) : f_(&f), local_(f.space().localSize(), 0.0) {}
  void bind(const Cell& e) {
    cell_ = e;
    std::fill(local_.begin(), local_.end(), 0.0);
  }
  void unbind() {
    double* w = f_->dofs().data() + cell_.index() * f_->space().localSize();
    for (std::size_t i = 0; i < local_.size(); ++i) w[i] += local_[i];
    cell_ = Cell();
  }
  int order() const { return f_->space().reportedOrder(); }
  template <class Point>
  void axpy(const Point& x, const RangeType& value, const JacobianRangeType& dvalue) {
    f_->space().shapeFunctionSet().evaluateEach(x, [&](std::size_t i, const RangeType& phi) {
      local_[i] += value[0] * phi[0];
    });
    const auto jit = cell_.geometry().jacobianInverseTransposed(coordinate(x));
    FieldVector<double, 3> t;
    jit.mtv(dvalue[0], t);
    f_->space().shapeFunctionSet().jacobianEach(x, [&](std::size_t i, const JacobianRangeType& dphi) {
      local_[i] += t * dphi[0];
    });
  }

 private:
  DF* f_;
  Cell cell_;
  std::vector<double> local_;
};

// A dense local matrix between the basis of a domain cell (columns) and of a
// range cell (rows), with the column axpy of operator/common/localmatrix.hh:
// 545-566: a_ij += weight (factor phi_i + jacobianFactor : dphi_i).
template <class DomainSpace, class RangeSpace>
class TemporaryLocalMatrix {
 public:
  class Column {
   public:
    Column(TemporaryLocalMatrix* m, int c) : m_(m), c_(c) {}
    template <class RangeVector, class JacobianVector, class R, class J>
    void axpy(const RangeVector& phi, const JacobianVector& dphi, const R& factor, const J& jacobianFactor,
              double weight) {
      for (int row = 0; row < m_->rows(); ++row) {
        double value = factor * phi[row];
        for (int k = 0; k < J::rows; ++k) value += jacobianFactor[k] * dphi[row][k];
        m_->a_[std::size_t(row) * m_->cols() + c_] += weight * value;
      }
    }

   private:
    TemporaryLocalMatrix* m_;
    int c_;
  };
  TemporaryLocalMatrix(const DomainSpace& d, const RangeSpace& r) : domain_(&d), range_(&r) {}
  void bind(const Cell& domainEntity, const Cell& rangeEntity) {
    de_ = domainEntity;
    re_ = rangeEntity;
    a_.assign(std::size_t(rows()) * cols(), 0.0);
  }
  void unbind() {}
  void clear() { std::fill(a_.begin(), a_.end(), 0.0); }
  int rows() const { return int(range_->localSize()); }
  int cols() const { return int(domain_->localSize()); }
  double get(int i, int j) const { return a_[std::size_t(i) * cols() + j]; }
  LegendreBasisFunctionSet domainBasisFunctionSet() const { return domain_->basisFunctionSet(de_); }
  LegendreBasisFunctionSet rangeBasisFunctionSet() const { return range_->basisFunctionSet(re_); }
  Column column(int c) { return Column(this, c); }
  const Cell& domainEntity() const { return de_; }
  const Cell& rangeEntity() const { return re_; }

 private:
  const DomainSpace* domain_;
  const RangeSpace* range_;
  Cell de_, re_;
  std::vector<double> a_;
};

template <class DomainSpace, class RangeSpace>
class DiagonalAndNeighborStencil {
 public:
  DiagonalAndNeighborStencil(const DomainSpace&, const RangeSpace&) {}
};

// The assembled Jacobian as a dense matrix (rows: range dofs, columns: domain
// dofs), filled by addLocalMatrix like the reference's sparse-row operator.
class DenseLinearOperator {
 public:
  typedef DGFunction DomainFunctionType;
  typedef DGFunction RangeFunctionType;
  explicit DenseLinearOperator(const LegendreDGSpace& s) : space_(&s), n_(s.size()), a_(n_ * n_, 0.0) {}
  template <class SolverParam>
  DenseLinearOperator(const std::string&, const LegendreDGSpace& domain, const LegendreDGSpace&, const SolverParam&)
      : DenseLinearOperator(domain) {}
  const LegendreDGSpace& domainSpace() const { return *space_; }
  const LegendreDGSpace& rangeSpace() const { return *space_; }
  template <class Stencil>
  void reserve(const Stencil&) {}
  void clear() { std::fill(a_.begin(), a_.end(), 0.0); }
  template <class Local>
  void addLocalMatrix(const Cell& domainEntity, const Cell& rangeEntity, const Local& m) {
    const std::size_t nl = space_->localSize();
    for (int i = 0; i < m.rows(); ++i)
      for (int j = 0; j < m.cols(); ++j)
        a_[(rangeEntity.index() * nl + i) * n_ + domainEntity.index() * nl + j] += m.get(i, j);
  }
  void flushAssembly() {}
  double operator()(std::size_t i, std::size_t j) const { return a_[i * n_ + j]; }
  std::size_t size() const { return n_; }

 private:
  const LegendreDGSpace* space_;
  std::size_t n_;
  std::vector<double> a_;
};

template <class LF>
struct BindGuard {
  LF* lf;
  ~BindGuard() { if (lf) lf->unbind(); }
};
template <class LF>
BindGuard<LF> bindGuard(LF& lf, const Cell& e) {
  lf.bind(e);
  return BindGuard<LF>{&lf};
}

}  // namespace Fem
}  // namespace Dune

#endif
