"""User-defined pointwise integrands, compiled at run time.

The counterpart of dune-fem's UFL integrand generation
(python/dune/models/integrands/ufl.py turns a UFL form into the C++ of an
integrands class, compiled when the scheme is built): here the user writes the
reaction r(u, x, y, z) of the volume term r v dx as a CUDA C++ expression.
This module wraps it in a functor (reaction_jit.cuh), instantiates the
sum-factorised reaction kernel for the operator's precision, order and
quadrature, and compiles it with nvcc into an sm_103a cubin, which the
library loads (gbfem_dg_nonlinear_operator_create_jit).  The Jacobian needs
r'(u): it comes from the same expression evaluated on dual numbers.

The expression may use u, x, y, z, arithmetic with numbers, and exp, log,
sqrt, sin, cos, tanh, sinh, cosh, atan, fabs, pow(u, p) and ipow<P>(u).
Cubins are cached under _jit/ by a hash of the generated source.
"""
import ctypes as C
import hashlib
import os
import re
import subprocess

import gbfem

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CACHE = os.path.join(HERE, "_jit")

_ALLOWED = re.compile(r"^[\w\s\.\+\-\*/\(\),<>]*$")


def reaction_source(expr, precision, order, quad_points=0):
    """The CUDA source of the reaction kernel for r(u, x, y, z) = expr."""
    if not _ALLOWED.match(expr):
        raise ValueError("reaction expression: only identifiers, numbers, + - * / ( ) , < > are allowed")
    n = order + 1
    q = quad_points or order + 2
    real = "double" if precision == gbfem.F64 else "float"
    tag = "f64" if precision == gbfem.F64 else "f32"
    return """// generated by integrands.py: r(u, x, y, z) = %(expr)s
#include "reaction_jit.cuh"

namespace {
struct UserFunction {
  template <class D>
  __device__ D operator()(D u, D x, D y, D z) const {
    using namespace gbfem::jit;
    (void)x; (void)y; (void)z;
    return D(%(expr)s);
  }
};
}  // namespace

extern "C" __global__ void __launch_bounds__(128)
gbfem_user_reaction_%(tag)s_n%(n)d_q%(q)d(int mode, const %(real)s* __restrict__ u, %(real)s* __restrict__ w,
                                          %(real)s* __restrict__ pts, long long cell_begin, long long count,
                                          const __grid_constant__ gbfem::ReactTabsT<%(real)s> tb) {
  gbfem::dg_reaction_body<%(real)s, %(n)d, %(q)d, 4, gbfem::jit::UserReaction<UserFunction>>(
      mode, u, w, pts, cell_begin, count, tb);
}
""" % dict(expr=expr, tag=tag, n=n, q=q, real=real)


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def compile_reaction(expr, precision, order, quad_points=0, cache_dir=CACHE):
    """Compiles r(u, x, y, z) = expr for (precision, order, quad_points);
    returns the path of the sm_103a cubin (cached by source hash)."""
    src = reaction_source(expr, precision, order, quad_points)
    key = hashlib.sha256(src.encode()).hexdigest()[:20]
    os.makedirs(cache_dir, exist_ok=True)
    cubin = os.path.join(cache_dir, "reaction_%s.cubin" % key)
    if os.path.exists(cubin):
        return cubin
    cu = os.path.join(cache_dir, "reaction_%s.cu" % key)
    with open(cu, "w") as f:
        f.write(src)
    cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE, "-o", cubin + ".tmp", cu]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reaction expression did not compile:\n%s" % r.stderr)
    os.replace(cubin + ".tmp", cubin)
    return cubin


class UserNonlinearDGOperator(gbfem.DGOperator):
    """S(u) = A u + int r(u, x) v with r given as a CUDA expression (see the
    module docstring); A the SIPG / upwind / mass operator (DGOperator's
    arguments).  jacobian(u), Newton and the Krylov solvers take it as they
    take NonlinearDGOperator."""

    def __init__(self, cells, order, reaction, quad_points=0, precision=gbfem.F64, diffusion=1.0, penalty=None,
                 mass=0.0, velocity=(0.0, 0.0, 0.0), weak_dirichlet=True, periodic=(0, 0, 0),
                 lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0), kappa=None, algorithm=0):
        q = quad_points or order + 2
        self.cubin = compile_reaction(reaction, precision, order, q)
        d = gbfem.DgDesc()
        d.grid = gbfem.grid_desc(cells, lower, upper, periodic)
        d.order = order
        d.quad_points = q
        d.precision = precision
        d.diffusion = diffusion
        d.penalty = 10.0 * (order + 1) ** 2 if penalty is None else penalty
        d.mass = mass
        for k in range(3):
            d.velocity[k] = velocity[k]
        d.weak_dirichlet = 1 if weak_dirichlet else 0
        self.kappa = kappa
        d.kappa = kappa.ptr if kappa is not None else None
        d.algorithm = algorithm
        L = gbfem.lib()
        L.gbfem_dg_nonlinear_operator_create_jit.argtypes = [C.POINTER(gbfem.DgDesc), C.c_char_p,
                                                             C.POINTER(C.c_void_p)]
        h = C.c_void_p()
        gbfem.check(L.gbfem_dg_nonlinear_operator_create_jit(C.byref(d), self.cubin.encode(), C.byref(h)))
        self.desc = d
        self.reaction = reaction
        self.order = order
        self.nloc = (order + 1) ** 3
        gbfem.Operator.__init__(self, h, precision)


def load_vector(cells, order, expr, quad_points=0, precision=gbfem.F64, lower=(0.0, 0.0, 0.0),
                upper=(1.0, 1.0, 1.0)):
    """b_l = int f phi_l for f(x, y, z) = expr (a CUDA expression in x, y, z), by
    the Gauss rule with quad_points per direction (0: order + 2): the reaction
    kernel with r = f applied to u = 0.  A DeviceArray in the DG dof layout."""
    op = UserNonlinearDGOperator(cells, order, expr, quad_points=quad_points, precision=precision, diffusion=0.0,
                                 penalty=0.0, weak_dirichlet=False, lower=lower, upper=upper)
    zero = gbfem.DeviceArray(op.size, precision)
    zero.clear()
    b = gbfem.DeviceArray(op.size, precision)
    op(zero, b)
    return b


def project(cells, order, expr, quad_points=0, precision=gbfem.F64, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
    """L2 projection of f(x, y, z) = expr onto DG Q_order (space.interpolate of a
    UFL expression): the load vector divided by |K|, the orthonormal basis
    making the mass matrix |K| I."""
    b = load_vector(cells, order, expr, quad_points, precision, lower, upper)
    vol = 1.0
    for k in range(3):
        vol *= (upper[k] - lower[k]) / cells[k]
    gbfem.check(gbfem.lib().gbfem_scal(precision, b.n, 1.0 / vol, b.ptr, None))
    return b
