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
        d.weak_dirichlet = gbfem.weak_dirichlet_flag(weak_dirichlet)
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


# ---- general forms -----------------------------------------------------------

_STMT_ALLOWED = re.compile(r"^[\w\s\.\+\-\*/\(\),<>\[\]=;:{}?!&|%]*$")


def _body(code, what):
    code = code or ""
    if not _STMT_ALLOWED.match(code):
        raise ValueError("%s: only identifiers, numbers, operators, brackets and ; are allowed" % what)
    return code


class Form:
    """A DG form for `components` solution components, written as CUDA C++
    statements that are compiled at run time (csrc/form_kernel.cuh): the
    counterpart of a UFL form that dune-fem turns into an integrands class
    (python/dune/models/integrands/ufl.py).

    Interior-penalty form (the default), from pointwise pieces; in every piece
    x[3] is the physical point, u[m] the solution, g[m][k] = du_m/dx_k, and the
    statements assign the outputs (zero-initialised):

      flux       F[m][k]   diffusive flux:    int_K F : grad v
      source     s[m]                         int_K s . v
      advection  Fa[m][k]  convective flux:  -int_K Fa : grad v + numerical flux
      wavespeed  an expression in x, u, n: bound of |dFa/du . n|
                 (local Lax-Friedrichs flux; for Fa = b u it is fabs(b.n), the upwind flux)
      dirichlet  gD[m] from x: weak boundary values on non-periodic boundaries
                 (None: natural boundary, zero diffusive flux)

    and the face terms of the symmetric (symmetry=1), incomplete (0) or
    non-symmetric (-1) interior penalty method,
      int_F sigma [u][v] - {F}.n [v] - symmetry [u] {A^T n}.grad v,
    sigma = penalty / h_F, A = dF/d(grad u) from dual numbers.  For
    F = kappa grad u, source = c u, Fa = b u this is the SIPG / upwind / mass
    operator of DGOperator (with penalty = diffusion * beta).

    Raw form: interior, skeleton and boundary statement bodies that assign
    s[m] and F[m][k] given (x, u, g), (x, n, sigma, uL, gL, uR, gR) and
    (x, n, sigma, u, g): the own side's test coefficients (see
    csrc/form_kernel.cuh).

    Expressions may use arithmetic, comparisons, ?:, exp, log, sqrt, sin, cos,
    tan, tanh, sinh, cosh, atan, fabs, pow, ipow<P>(.), max and min; they are
    generic in the value type, which is a dual number in the Jacobian.
    """

    def __init__(self, components=1, flux=None, source=None, advection=None, wavespeed=None, dirichlet=None,
                 symmetry=1, interior=None, skeleton=None, boundary=None):
        if not 1 <= components <= 4:
            raise ValueError("Form: 1..4 components")
        self.components = components
        self.raw = interior is not None or skeleton is not None or boundary is not None
        if self.raw and (flux or source or advection or dirichlet):
            raise ValueError("Form: give either the interior-penalty pieces or raw interior/skeleton/boundary bodies")
        if advection and not wavespeed:
            raise ValueError("Form: advection needs a wavespeed expression")
        if symmetry not in (-1, 0, 1):
            raise ValueError("Form: symmetry is 1, 0 or -1")
        self.pieces = dict(flux=_body(flux, "flux"), source=_body(source, "source"),
                           advection=_body(advection, "advection"), wavespeed=_body(wavespeed, "wavespeed"),
                           dirichlet=_body(dirichlet, "dirichlet"), interior=_body(interior, "interior"),
                           skeleton=_body(skeleton, "skeleton"), boundary=_body(boundary, "boundary"))
        self.flags = dict(flux=bool(flux), source=bool(source), advection=bool(advection),
                          dirichlet=dirichlet is not None)
        self.symmetry = symmetry

    def _integrand(self):
        p = self.pieces
        M = self.components
        if self.raw:
            return """struct Integrand {
  static constexpr int M = %(M)d;
  template <class D, class R>
  __device__ static void interior(const R* x, const D* u, D (*g)[3], D* s, D (*F)[3]) {
    (void)x; (void)u; (void)g; (void)s; (void)F;
    %(interior)s
  }
  template <class D, class R>
  __device__ static void skeleton(const R* x, const R* n, R sigma, const D* uL, D (*gL)[3], const D* uR,
                                  D (*gR)[3], D* s, D (*F)[3]) {
    (void)x; (void)n; (void)sigma; (void)uL; (void)gL; (void)uR; (void)gR; (void)s; (void)F;
    %(skeleton)s
  }
  template <class D, class R>
  __device__ static void boundary(const R* x, const R* n, R sigma, const D* u, D (*g)[3], D* s, D (*F)[3]) {
    (void)x; (void)n; (void)sigma; (void)u; (void)g; (void)s; (void)F;
    %(boundary)s
  }
};""" % dict(M=M, **p)
        f = self.flags
        return """struct Pieces {
  static constexpr int M = %(M)d;
  static constexpr bool kFlux = %(kf)s, kSource = %(ks)s, kAdvection = %(ka)s, kDirichlet = %(kd)s;
  template <class D, class R>
  __device__ static void flux(const R* x, const D* u, D (*g)[3], D (*F)[3]) {
    (void)x; (void)u; (void)g; (void)F;
    %(flux)s
  }
  template <class D, class R>
  __device__ static void source(const R* x, const D* u, D (*g)[3], D* s) {
    (void)x; (void)u; (void)g; (void)s;
    %(source)s
  }
  template <class D, class R>
  __device__ static void advection(const R* x, const D* u, D (*Fa)[3]) {
    (void)x; (void)u; (void)Fa;
    %(advection)s
  }
  template <class D, class R>
  __device__ static D wavespeed(const R* x, const D* u, const R* n) {
    (void)x; (void)u; (void)n;
    return D(%(wavespeed)s);
  }
  template <class R>
  __device__ static void dirichlet(const R* x, R* gD) {
    (void)x; (void)gD;
    %(dirichlet)s
  }
};
using Integrand = Sipg<Pieces, %(theta)d>;""" % dict(M=M, kf=str(f["flux"]).lower(), ks=str(f["source"]).lower(),
                                                     ka=str(f["advection"]).lower(), kd=str(f["dirichlet"]).lower(),
                                                     theta=self.symmetry, wavespeed=p["wavespeed"] or "0", **{
                                                         k: p[k] for k in ("flux", "source", "advection",
                                                                           "dirichlet")})

    def source_code(self, precision, order, quad_points=0):
        """The CUDA source of the form's two kernels for (precision, order, q)."""
        n = order + 1
        q = quad_points or order + 2
        real = "double" if precision == gbfem.F64 else "float"
        tag = "f64" if precision == gbfem.F64 else "f32"
        name = "gbfem_form_%s_n%d_q%d_m%d" % (tag, n, q, self.components)
        kern = """extern "C" __global__ void __launch_bounds__(128)
%(name)s_%(suffix)s(const __grid_constant__ gbfem::form::FormArgs<%(real)s> a,
     const __grid_constant__ gbfem::DgTablesT<%(real)s> t) {
  gbfem::form::form_body<gbfem::form::generated::Integrand, %(real)s, %(vt)s, %(n)d, %(q)d, %(M)d>(a, t);
}
"""
        return ("// generated by integrands.py\n#include \"form_kernel.cuh\"\n\n"
                "namespace gbfem {\nnamespace form {\nnamespace generated {\n\n%s\n\n}  // namespace generated\n"
                "}  // namespace form\n}  // namespace gbfem\n\n" % self._integrand()
                + kern % dict(name=name, suffix="val", real=real, vt=real, n=n, q=q, M=self.components)
                + kern % dict(name=name, suffix="lin", real=real, vt="gbfem::form::Dual<%s>" % real, n=n, q=q,
                              M=self.components))

    def compile(self, precision, order, quad_points=0, cache_dir=CACHE):
        """Compiles the form for (precision, order, q); returns the sm_103a
        cubin's path (cached by source hash)."""
        src = self.source_code(precision, order, quad_points)
        key = hashlib.sha256(src.encode()).hexdigest()[:20]
        os.makedirs(cache_dir, exist_ok=True)
        cubin = os.path.join(cache_dir, "form_%s.cubin" % key)
        if os.path.exists(cubin):
            return cubin
        cu = os.path.join(cache_dir, "form_%s.cu" % key)
        with open(cu, "w") as f:
            f.write(src)
        cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
               "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE, "-o", cubin + ".%d.tmp" % os.getpid(), cu]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("form did not compile:\n%s" % r.stderr)
        os.replace(cubin + ".%d.tmp" % os.getpid(), cubin)
        return cubin


class FormOperator(gbfem.Operator):
    """S(u) for a Form on a structured grid of DG Q_order (dof = cell *
    M (p+1)^3 + i * M + m).  A nonlinear operator: jacobian(u) is exact, and
    Newton, the Krylov solvers, the preconditioners of the Jacobian, Scheme
    and RK3 take it like NonlinearDGOperator.  penalty is the beta of
    sigma = beta / h_F (default 10 (p+1)^2)."""

    def __init__(self, form, cells, order, quad_points=0, precision=gbfem.F64, penalty=None, periodic=(0, 0, 0),
                 lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
        if getattr(form, "unit_penalty", False):
            # a UFL form with FacetSize() reads h_F as 1 / sigma
            if penalty not in (None, 1.0):
                raise ValueError("FormOperator: this form uses the facet size; its penalty is fixed at 1")
            penalty = 1.0
        q = quad_points or order + 2
        self.cubin = form.compile(precision, order, q)
        d = gbfem.DgDesc()
        d.grid = gbfem.grid_desc(cells, lower, upper, periodic)
        d.order = order
        d.quad_points = q
        d.precision = precision
        d.penalty = 10.0 * (order + 1) ** 2 if penalty is None else penalty
        L = gbfem.lib()
        L.gbfem_form_operator_create.argtypes = [C.POINTER(gbfem.DgDesc), C.c_int, C.c_char_p, C.POINTER(C.c_void_p)]
        h = C.c_void_p()
        gbfem.check(L.gbfem_form_operator_create(C.byref(d), form.components, self.cubin.encode(), C.byref(h)))
        self.desc = d
        self.form = form
        self.order = order
        self.components = form.components
        self.nloc = form.components * (order + 1) ** 3
        gbfem.Operator.__init__(self, h, precision)
