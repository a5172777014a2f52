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

class LegendreDGSpace {
 public:
  typedef ScalarFunctionSpace3 FunctionSpaceType;
  typedef FunctionSpaceType::DomainType DomainType;
  typedef FunctionSpaceType::RangeType RangeType;
  typedef FunctionSpaceType::JacobianRangeType JacobianRangeType;
  typedef GridPart GridPartType;
  typedef CellIterator IteratorType;
  typedef LegendreShapeFunctionSet<FunctionSpaceType, false> ShapeFunctionSetType;

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
  const CartesianGrid& grid() const { return grid_; }

 private:
  CartesianGrid grid_;
  GridPart gridPart_;
  ShapeFunctionSetType shapes_;
  int order_, reported_;
};

struct LocalFunctionTraits {
  typedef LegendreDGSpace::RangeType RangeType;
  typedef LegendreDGSpace::JacobianRangeType JacobianRangeType;
  typedef double RangeFieldType;
  static const int dimDomain = 3;
  static const int dimRange = 1;
};

class DGFunction {
 public:
  typedef LegendreDGSpace DiscreteFunctionSpaceType;
  typedef LocalFunctionTraits LocalFunctionType;
  typedef double DofType;
  explicit DGFunction(const LegendreDGSpace& s) : space_(&s), dofs_(s.size(), 0.0) {}
  DGFunction(const std::string&, const LegendreDGSpace& s) : DGFunction(s) {}
  const LegendreDGSpace& space() const { return *space_; }
  void clear() { std::fill(dofs_.begin(), dofs_.end(), 0.0); }
  void assign(const DGFunction& o) { dofs_ = o.dofs_; }
  void axpy(double a, const DGFunction& x) {
    for (std::size_t i = 0; i < dofs_.size(); ++i) dofs_[i] += a * x.dofs_[i];
  }
  void communicate() {}
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
