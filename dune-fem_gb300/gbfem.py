"""Python binding of libgbfem's C-ABI (include/gbfem.h) through ctypes.

It mirrors the reference's Python surface for this path: an operator object
called as ``op(u, w)`` (dune/fempy/py/operator.hh:49,215), solvers called as
``solver(f, u)`` (InverseOperator::operator(), solver/inverseoperatorinterface.hh:81-84).
Dof vectors are DeviceArray objects resident in GPU memory.

There is no CPU fallback: if libgbfem.so is missing, loading raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgbfem.so")

F64, F32 = 0, 1
F16 = 2  # block-Jacobi storage only (scaled FP16 blocks, FP32 vectors)
ALGO_AUTO, ALGO_QUADRATURE, ALGO_TRACE_PASS = 0, 1, 2
_DTYPES = {F64: np.float64, F32: np.float32}


class GbfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gbfem error %d: %s" % (code, msg))
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("cells", C.c_int * 3), ("lower", C.c_double * 3),
                ("upper", C.c_double * 3), ("periodic", C.c_int * 3)]


class DgDesc(C.Structure):
    _fields_ = [("grid", GridDesc), ("order", C.c_int), ("quad_points", C.c_int), ("precision", C.c_int),
                ("diffusion", C.c_double), ("penalty", C.c_double), ("mass", C.c_double),
                ("velocity", C.c_double * 3), ("weak_dirichlet", C.c_int), ("kappa", C.c_void_p),
                ("algorithm", C.c_int), ("kappa_cell", C.c_void_p)]


class SolverParams(C.Structure):
    _fields_ = [("method", C.c_int), ("tolerance", C.c_double), ("error_measure", C.c_int),
                ("max_iterations", C.c_int), ("restart", C.c_int), ("verbose", C.c_int), ("graph_chunk", C.c_int)]


class SolverInfo(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int), ("residual", C.c_double),
                ("time_ms", C.c_double), ("operator_applies", C.c_int), ("preconditioner_applies", C.c_int),
                ("status", C.c_int), ("fallbacks", C.c_int), ("outer_iterations", C.c_int),
                ("stagnated", C.c_int)]


class IRParams(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("max_outer", C.c_int), ("inner", SolverParams),
                ("outer_method", C.c_int), ("outer_restart", C.c_int)]


class Reaction(C.Structure):
    _fields_ = [("linear", C.c_double), ("cubic", C.c_double), ("exponential", C.c_double)]


class NewtonParams(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("max_iterations", C.c_int), ("max_linear_iterations", C.c_int),
                ("max_line_search_iterations", C.c_int), ("line_search", C.c_int), ("forcing", C.c_int),
                ("eta_max", C.c_double), ("gamma", C.c_double), ("simplified", C.c_int),
                ("preconditioner", C.c_int), ("verbose", C.c_int), ("linear", SolverParams), ("assembled", C.c_int)]


class NewtonInfo(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int), ("linear_iterations", C.c_int),
                ("residual", C.c_double), ("failure", C.c_int), ("time_ms", C.c_double)]


PC_NONE, PC_DIAGONAL, PC_BLOCK_JACOBI = 0, 1, 2
NEWTON_FAILURES = {0: "Success", 1: "InvalidResidual", 4: "LineSearchFailed", 5: "TooManyIterations",
                   6: "TooManyLinearIterations", 7: "LinearSolverFailed"}

CG, GMRES, BICGSTAB, FCG, FGMRES = 0, 1, 2, 3, 4
ABSOLUTE, RELATIVE, RESIDUAL_REDUCTION, RELATIVE_RESIDUAL = 0, 1, 2, 3
METHODS = {"cg": CG, "gmres": GMRES, "bicgstab": BICGSTAB, "fcg": FCG, "fgmres": FGMRES}

_lib = None


def lib():
    """Loads libgbfem.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbfem.so not built: run __graft_entry__.build() (%s)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        L.gbfem_last_error.restype = C.c_char_p
        L.gbfem_dot.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
        L.gbfem_axpy.argtypes = [C.c_int, C.c_int64, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_scal.argtypes = [C.c_int, C.c_int64, C.c_double, C.c_void_p, C.c_void_p]
        L.gbfem_copy.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_convert.argtypes = [C.c_int64, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.gbfem_malloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        L.gbfem_free.argtypes = [C.c_void_p]
        L.gbfem_memcpy_h2d.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.gbfem_memcpy_d2h.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.gbfem_memset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
        L.gbfem_operator_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_operator_apply_host.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_operator_set_host_chunks.argtypes = [C.c_void_p, C.c_int]
        L.gbfem_operator_set_host_transfer.argtypes = [C.c_void_p, C.c_int]
        L.gbfem_operator_update_coefficients.argtypes = [C.c_void_p]
        L.gbfem_operator_diagonal.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_operator_block_diagonal.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_operator_destroy.argtypes = [C.c_void_p]
        L.gbfem_operator_size.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        L.gbfem_dg_operator_create.argtypes = [C.POINTER(DgDesc), C.POINTER(C.c_void_p)]
        L.gbfem_q1_operator_create.argtypes = [C.POINTER(GridDesc), C.c_int, C.c_double, C.c_double,
                                               C.POINTER(C.c_void_p)]
        L.gbfem_operator_assemble.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.gbfem_fourier_modes.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.gbfem_dg_project.argtypes = [C.POINTER(GridDesc), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.gbfem_rk3_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.gbfem_rk3_step.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
        L.gbfem_rk3_destroy.argtypes = [C.c_void_p]
        L.gbfem_dg_time_step_estimate.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.POINTER(C.c_double),
                                                  C.POINTER(C.c_double)]
        L.gbfem_cnn_create.argtypes = [C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]
        L.gbfem_cnn_destroy.argtypes = [C.c_void_p]
        L.gbfem_cnn_set_kappa.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.gbfem_cnn_set_output_scale.argtypes = [C.c_void_p, C.c_double]
        L.gbfem_cnn_set_coarse.argtypes = [C.c_void_p, C.c_int]
        L.gbfem_cnn_get_output_scale.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.gbfem_cnn_forward.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.gbfem_cnn_loss_grad.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                          C.c_void_p]
        L.gbfem_cnn_train_step.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                           C.POINTER(C.c_double), C.c_void_p]
        L.gbfem_cnn_num_params.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        L.gbfem_cnn_train_step_grad.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                                C.c_void_p]
        L.gbfem_cnn_get_params.argtypes = [C.c_void_p, C.c_void_p]
        L.gbfem_cnn_set_params.argtypes = [C.c_void_p, C.c_void_p]
        L.gbfem_cnn_get_grads.argtypes = [C.c_void_p, C.c_void_p]
        L.gbfem_cnn_save.argtypes = [C.c_void_p, C.c_char_p]
        L.gbfem_cnn_load.argtypes = [C.c_void_p, C.c_char_p]
        L.gbfem_preconditioner_learned_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]
        L.gbfem_preconditioner_diagonal_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.gbfem_preconditioner_block_jacobi_create.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.gbfem_preconditioner_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_preconditioner_sor_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double,
                                                      C.POINTER(C.c_void_p)]
        L.gbfem_preconditioner_scaled_block_jacobi_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.gbfem_preconditioner_scaled_block_jacobi_create_engine.argtypes = [C.c_void_p, C.c_int,
                                                                             C.POINTER(C.c_void_p)]
        L.gbfem_preconditioner_status.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.gbfem_preconditioner_destroy.argtypes = [C.c_void_p]
        L.gbfem_solver_params_default.argtypes = [C.POINTER(SolverParams)]
        L.gbfem_solve.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(SolverParams), C.c_void_p, C.c_void_p,
                                  C.POINTER(SolverInfo)]
        L.gbfem_solve_mixed.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(IRParams), C.c_void_p,
                                        C.c_void_p, C.POINTER(SolverInfo)]
        L.gbfem_dg_nonlinear_operator_create.argtypes = [C.POINTER(DgDesc), C.POINTER(Reaction),
                                                         C.POINTER(C.c_void_p)]
        L.gbfem_operator_nonlinear.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.gbfem_operator_jacobian_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.gbfem_operator_jacobian.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_newton_params_default.argtypes = [C.POINTER(NewtonParams)]
        L.gbfem_legendre_hierarchical_permutation.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.gbfem_dg_permute.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_dg_cell_means.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbfem_newton_solve.argtypes = [C.c_void_p, C.POINTER(NewtonParams), C.c_void_p, C.c_void_p,
                                         C.POINTER(NewtonInfo)]
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        raise GbfemError(rc, lib().gbfem_last_error().decode())
    return rc


class DeviceArray:
    """A dof vector in GPU memory (the storage of an AdaptiveDiscreteFunction)."""

    def __init__(self, n, precision=F64):
        self.n = int(n)
        self.precision = precision
        self.itemsize = 8 if precision == F64 else 4
        self.ptr = C.c_void_p()
        check(lib().gbfem_malloc(C.byref(self.ptr), self.n * self.itemsize))

    @classmethod
    def from_numpy(cls, a, precision=None):
        a = np.ascontiguousarray(a)
        if precision is None:
            precision = F32 if a.dtype == np.float32 else F64
        a = np.ascontiguousarray(a, dtype=_DTYPES[precision])
        d = cls(a.size, precision)
        check(lib().gbfem_memcpy_h2d(d.ptr, a.ctypes.data, a.nbytes))
        return d

    def numpy(self):
        out = np.empty(self.n, dtype=_DTYPES[self.precision])
        check(lib().gbfem_memcpy_d2h(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def clear(self):
        check(lib().gbfem_memset(self.ptr, 0, self.n * self.itemsize))

    @property
    def __cuda_array_interface__(self):
        """Zero-copy view of the dofs for GPU array libraries (the CUDA Array
        Interface, version 3): torch.as_tensor(a, device="cuda"), cupy, numba
        see the same device memory, no copy.  (numpy() copies to the host.)"""
        return {"shape": (self.n,), "typestr": "<f8" if self.precision == F64 else "<f4",
                "data": (int(self.ptr.value or 0), False), "version": 3, "strides": None}

    def as_tensor(self):
        """The dofs as a torch tensor on the GPU sharing this memory (no copy);
        the DeviceArray must outlive it."""
        import torch
        return torch.as_tensor(self, device="cuda")

    def free(self):
        if self.ptr:
            lib().gbfem_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def grid_desc(cells, lower=None, upper=None, periodic=None):
    dim = len(cells)
    g = GridDesc()
    g.dim = dim
    for k in range(3):
        g.cells[k] = int(cells[k]) if k < dim else 1
        g.lower[k] = (lower[k] if lower is not None else 0.0) if k < dim else 0.0
        g.upper[k] = (upper[k] if upper is not None else 1.0) if k < dim else 1.0
        g.periodic[k] = int(periodic[k]) if (periodic is not None and k < dim) else 0
    return g


class Operator:
    """w = op(u): dune-fem's Operator::operator()(u, w) (operator/common/operator.hh:55)."""

    def __init__(self, handle, precision):
        self.handle = handle
        self.precision = precision
        n = C.c_int64()
        check(lib().gbfem_operator_size(self.handle, C.byref(n)))
        self.size = n.value

    def __call__(self, u, w, stream=None):
        check(lib().gbfem_operator_apply(self.handle, u.ptr, w.ptr, stream))

    def apply_host(self, u, w):
        """Host-buffer apply: copies u in, applies, copies w out (synchronous)."""
        check(lib().gbfem_operator_apply_host(self.handle, u.ctypes.data, w.ctypes.data))

    def update_coefficients(self):
        """Re-evaluates a variable kappa at the Gauss points after its vector changed."""
        check(lib().gbfem_operator_update_coefficients(self.handle))

    def set_host_transfer(self, in_place):
        """True: the kernels read u and write w in page-locked host memory over
        NVLink-C2C; False (default): the slab copy pipeline."""
        check(lib().gbfem_operator_set_host_transfer(self.handle, 1 if in_place else 0))

    def set_host_chunks(self, nchunks):
        """Slabs of the pipelined host-buffer apply of a DG operator (0 = automatic)."""
        check(lib().gbfem_operator_set_host_chunks(self.handle, nchunks))

    def diagonal(self):
        d = DeviceArray(self.size, self.precision)
        check(lib().gbfem_operator_diagonal(self.handle, d.ptr, None))
        return d

    def assemble(self):
        """The assembled (block-sparse) copy of this operator, as an Operator."""
        h = C.c_void_p()
        check(lib().gbfem_operator_assemble(self.handle, C.byref(h)))
        a = Operator(h, self.precision)
        a.nloc = getattr(self, "nloc", None)
        return a

    def block_diagonal(self, nloc):
        b = DeviceArray(self.size * nloc, self.precision)
        check(lib().gbfem_operator_block_diagonal(self.handle, b.ptr, None))
        return b

    def nonlinear(self):
        v = C.c_int()
        check(lib().gbfem_operator_nonlinear(self.handle, C.byref(v)))
        return bool(v.value)

    def jacobian(self, u, jac=None):
        """The Jacobian at u as a linear Operator (jacobian(u, jOp),
        operator/common/differentiableoperator.hh:54); pass jac to update one."""
        if jac is None:
            h = C.c_void_p()
            check(lib().gbfem_operator_jacobian_create(self.handle, C.byref(h)))
            jac = Operator(h, self.precision)
            jac.nloc = getattr(self, "nloc", None)
            jac._base = self
        check(lib().gbfem_operator_jacobian(self.handle, u.ptr, jac.handle, None))
        return jac

    def __del__(self):
        try:
            if self.handle:
                lib().gbfem_operator_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def weak_dirichlet_flag(weak_dirichlet):
    """The descriptor's weak_dirichlet field: 1 for the symmetric interior-
    penalty boundary (the full -u kappa grad v . n term), 0 for none.  The
    boundary of dune-fem's DGEllipticOperator, which halves that term, is a
    different form; it is available as an integrands.Form, not here."""
    if weak_dirichlet in (True, False, 0, 1):
        return 1 if weak_dirichlet else 0
    raise ValueError("weak_dirichlet must be True or False (got %r); write other boundary forms "
                     "with integrands.Form" % (weak_dirichlet,))


class DGOperator(Operator):
    """SIPG / upwind / mass DG operator on a structured hexahedral grid."""

    def __init__(self, cells, order, quad_points=0, precision=F64, diffusion=1.0, penalty=None, mass=0.0,
                 velocity=(0.0, 0.0, 0.0), weak_dirichlet=True, periodic=(0, 0, 0), lower=(0.0, 0.0, 0.0),
                 upper=(1.0, 1.0, 1.0), kappa=None, algorithm=0, kappa_cell=None):
        d = DgDesc()
        self.kappa_cell = kappa_cell
        d.kappa_cell = kappa_cell.ptr if kappa_cell is not None else None
        d.grid = grid_desc(cells, lower, upper, periodic)
        d.order = order
        d.quad_points = quad_points
        d.precision = precision
        d.diffusion = diffusion
        d.penalty = 10.0 * (order + 1) ** 2 if penalty is None else penalty
        d.mass = mass
        for k in range(3):
            d.velocity[k] = velocity[k]
        d.weak_dirichlet = weak_dirichlet_flag(weak_dirichlet)
        self.kappa = kappa  # keep the device array alive
        d.kappa = kappa.ptr if kappa is not None else None
        d.algorithm = algorithm
        h = C.c_void_p()
        check(lib().gbfem_dg_operator_create(C.byref(d), C.byref(h)))
        self.desc = d
        self.order = order
        self.nloc = (order + 1) ** 3
        super().__init__(h, precision)


class NonlinearDGOperator(DGOperator):
    """S(u) = A u + int r(u) v, r(u) = linear u + cubic u^3 + exponential e^u,
    A the SIPG / upwind / mass DG operator (same arguments as DGOperator)."""

    def __init__(self, cells, order, reaction=(0.0, 0.0, 0.0), quad_points=0, precision=F64, diffusion=1.0,
                 penalty=None, mass=0.0, velocity=(0.0, 0.0, 0.0), weak_dirichlet=True, periodic=(0, 0, 0),
                 lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0), kappa=None, algorithm=0):
        d = DgDesc()
        d.grid = grid_desc(cells, lower, upper, periodic)
        d.order = order
        d.quad_points = quad_points
        d.precision = precision
        d.diffusion = diffusion
        d.penalty = 10.0 * (order + 1) ** 2 if penalty is None else penalty
        d.mass = mass
        for k in range(3):
            d.velocity[k] = velocity[k]
        d.weak_dirichlet = weak_dirichlet_flag(weak_dirichlet)
        self.kappa = kappa
        d.kappa = kappa.ptr if kappa is not None else None
        d.algorithm = algorithm
        r = Reaction(*reaction)
        h = C.c_void_p()
        check(lib().gbfem_dg_nonlinear_operator_create(C.byref(d), C.byref(r), C.byref(h)))
        self.desc = d
        self.reaction = tuple(reaction)
        self.order = order
        self.nloc = (order + 1) ** 3
        Operator.__init__(self, h, precision)


class NewtonInverseOperator:
    """w = S^{-1}(rhs) by Newton's method: NewtonInverseOperator
    (solver/newtoninverseoperator.hh:484-790): bind(op), __call__(rhs, w) with
    w the initial guess, iterations(), linearIterations(), info().

    linear: a KrylovInverseOperator-style parameter set (method, tolerance,
    error_measure, max_iterations, restart); preconditioner: PC_* of each
    Jacobian; line_search "none" | "simple"; forcing "none" | "eisenstatwalker";
    assembled: solve with each Jacobian assembled into the block-sparse matrix
    (the reference's matrix-based Newton) instead of matrix-free."""

    def __init__(self, tolerance=1e-6, max_iterations=None, max_linear_iterations=None, line_search="none",
                 forcing="none", eta_max=0.99, gamma=0.1, simplified=False, preconditioner=PC_BLOCK_JACOBI,
                 linear_method="cg", linear_tolerance=1e-8, linear_error_measure=RELATIVE,
                 linear_max_iterations=None, linear_restart=20, max_line_search_iterations=None, verbose=False,
                 assembled=False):
        p = NewtonParams()
        check(lib().gbfem_newton_params_default(C.byref(p)))
        p.tolerance = tolerance
        if max_iterations is not None:
            p.max_iterations = max_iterations
        if max_line_search_iterations is not None:
            p.max_line_search_iterations = max_line_search_iterations
        p.line_search = {"none": 0, "simple": 1}[line_search]
        p.forcing = {"none": 0, "eisenstatwalker": 1}[forcing]
        p.eta_max, p.gamma = eta_max, gamma
        p.simplified = 1 if simplified else 0
        p.preconditioner = preconditioner
        p.verbose = 1 if verbose else 0
        p.assembled = 1 if assembled else 0
        p.linear = solver_params(linear_method, linear_tolerance, linear_error_measure, linear_max_iterations,
                                 linear_restart)
        p.max_linear_iterations = p.linear.max_iterations if max_linear_iterations is None else max_linear_iterations
        self.params = p
        self.op = None
        self._info = NewtonInfo()

    def bind(self, op):
        self.op = op

    def unbind(self):
        self.op = None

    def __call__(self, rhs, w):
        if self.op is None:
            raise GbfemError(-1, "NewtonInverseOperator: no operator bound")
        check(lib().gbfem_newton_solve(self.op.handle, C.byref(self.params), rhs.ptr, w.ptr, C.byref(self._info)))
        return self._info

    def iterations(self):
        return self._info.iterations

    def linearIterations(self):
        return self._info.linear_iterations

    def info(self):
        i = self._info
        return {"converged": bool(i.converged), "iterations": i.iterations, "linear_iterations": i.linear_iterations,
                "residual": i.residual, "failure": NEWTON_FAILURES.get(i.failure, str(i.failure)),
                "time_ms": i.time_ms}


class Space:
    """The discrete space a scheme acts on: its size and precision, and the
    zero vector (scheme.space.zero)."""

    def __init__(self, size, precision):
        self.size = size
        self.precision = precision

    @property
    def zero(self):
        z = DeviceArray(self.size, self.precision)
        z.clear()
        return z

    def function(self, name=None):
        """A new discrete function (dof vector) of this space, set to zero."""
        return self.zero


_PRECONDITIONING = ("none", "jacobi", "blockjacobi", "sor", "ssor", "gauss-seidel")


class Scheme:
    """A Galerkin scheme over one of the library's operators, in the shape of
    dune.fem's schemes (python/dune/fem/scheme/__init__.py:17-45,
    dune/fempy/py/scheme.hh:112-190): scheme(u, w) applies the operator,
    scheme.solve(target, rightHandSide=...) solves S(target) = rightHandSide
    from the initial guess in target and returns the info dictionary
    {converged, iterations, linear_iterations, timing}.

    parameters: the fem.solver keys without the prefix, as dune.fem takes
    them: "linear.method" (cg, gmres, bicgstab, fcg, fgmres),
    "linear.tolerance", "linear.errormeasure" (absolute, relative,
    residualreduction), "linear.maxiterations", "linear.gmres.restart",
    "linear.preconditioning.method" (none, jacobi, blockjacobi, sor, ssor,
    gauss-seidel), "linear.verbose"; for a nonlinear operator
    "nonlinear.tolerance", "nonlinear.maxiterations",
    "nonlinear.linesearch" (none, simple), "nonlinear.forcing" (none,
    eisenstatwalker).  The deprecated "newton." prefix is accepted, as in
    dune.fem."""

    _MEASURES = {"absolute": ABSOLUTE, "relative": RELATIVE, "residualreduction": RESIDUAL_REDUCTION}

    def __init__(self, op, parameters=None):
        self.op = op
        self.space = Space(op.size, op.precision)
        prm = {}
        for k, v in (parameters or {}).items():
            prm[k[len("newton."):] if k.startswith("newton.") else k] = v
        self.parameters = prm
        pre = prm.get("linear.preconditioning.method", "none")
        if pre not in _PRECONDITIONING:
            raise GbfemError(-1, "Scheme: unknown preconditioning method %r" % (pre,))
        self._pc = None

    def __call__(self, u, w):
        """w = S(u): the operator's apply (GalerkinOperator::operator())."""
        self.op(u, w)

    def linear(self):
        """The linear operator of a linear scheme, the Jacobian at 0 of a nonlinear one."""
        if not self.op.nonlinear():
            return self.op
        return self.op.jacobian(self.space.zero)

    def _preconditioner(self, op):
        pre = self.parameters.get("linear.preconditioning.method", "none")
        if pre == "none":
            return None
        if pre == "jacobi":
            return Preconditioner.diagonal(op)
        if pre == "blockjacobi":
            return Preconditioner.block_jacobi(op)
        return Preconditioner.sor(op.assemble(), method=pre,
                                  iterations=int(self.parameters.get("linear.preconditioning.iterations", 1)),
                                  relaxation=float(self.parameters.get("linear.preconditioning.relaxation", 1.0)))

    def inverseLinearOperator(self, parameters=None):
        """A KrylovInverseOperator bound to the linear operator, with this
        scheme's parameters (updated by `parameters`)."""
        prm = dict(self.parameters)
        prm.update(parameters or {})
        inv = KrylovInverseOperator(prm.get("linear.method", "cg"), tolerance=float(prm.get("linear.tolerance", 1e-8)),
                                    error_measure=self._MEASURES[prm.get("linear.errormeasure", "absolute")],
                                    max_iterations=prm.get("linear.maxiterations"),
                                    restart=int(prm.get("linear.gmres.restart", 20)),
                                    verbose=bool(prm.get("linear.verbose", False)))
        op = self.linear()
        inv.bind(op, self._preconditioner(op))
        return inv

    def solve(self, target, rightHandSide=None):
        """target = S^{-1}(rightHandSide) (rightHandSide None: zero), target
        on entry the initial guess.  Linear: the Krylov inverse operator;
        nonlinear: Newton with that linear solver."""
        rhs = rightHandSide if rightHandSide is not None else self.space.zero
        prm = self.parameters
        if not self.op.nonlinear():
            inv = self.inverseLinearOperator()
            inv(rhs, target)
            i = inv.info()
            return {"converged": i["converged"], "iterations": 0, "linear_iterations": i["iterations"],
                    "timing": [i["time_ms"] * 1e-3]}
        pre = prm.get("linear.preconditioning.method", "none")
        pcs = {"none": PC_NONE, "jacobi": PC_DIAGONAL, "blockjacobi": PC_BLOCK_JACOBI}
        if pre not in pcs:
            raise GbfemError(-1, "Scheme: a nonlinear scheme takes none, jacobi or blockjacobi preconditioning")
        newton = NewtonInverseOperator(
            tolerance=float(prm.get("nonlinear.tolerance", 1e-6)), max_iterations=prm.get("nonlinear.maxiterations"),
            line_search=prm.get("nonlinear.linesearch", "none"), forcing=prm.get("nonlinear.forcing", "none"),
            preconditioner=pcs[pre], linear_method=prm.get("linear.method", "cg"),
            linear_tolerance=float(prm.get("linear.tolerance", 1e-8)),
            linear_error_measure=self._MEASURES[prm.get("linear.errormeasure", "relative")],
            linear_max_iterations=prm.get("linear.maxiterations"),
            linear_restart=int(prm.get("linear.gmres.restart", 20)))
        newton.bind(self.op)
        newton(rhs, target)
        i = newton.info()
        return {"converged": i["converged"], "iterations": i["iterations"], "linear_iterations": i["linear_iterations"],
                "timing": [i["time_ms"] * 1e-3]}


class Q1Operator(Operator):
    """Continuous Lagrange Q1 on a 2-D grid with strong homogeneous Dirichlet rows."""

    def __init__(self, cells, precision=F64, diffusion=1.0, mass=0.0, lower=(0.0, 0.0), upper=(1.0, 1.0)):
        g = grid_desc(cells, lower, upper)
        h = C.c_void_p()
        check(lib().gbfem_q1_operator_create(C.byref(g), precision, diffusion, mass, C.byref(h)))
        super().__init__(h, precision)


def dot(x, y, stream=None):
    r = C.c_double()
    check(lib().gbfem_dot(x.precision, x.n, x.ptr, y.ptr, C.byref(r), stream))
    return r.value


def axpy(alpha, x, y, stream=None):
    check(lib().gbfem_axpy(x.precision, x.n, alpha, x.ptr, y.ptr, stream))


class Preconditioner:
    """z = P(r) (any Operator<D,D> in the reference, krylovinverseoperators.hh:36)."""

    def __init__(self, handle, precision, keep=None):
        self.handle = handle
        self.precision = precision
        self._keep = keep

    @classmethod
    def diagonal(cls, op):
        h = C.c_void_p()
        check(lib().gbfem_preconditioner_diagonal_create(op.handle, C.byref(h)))
        return cls(h, op.precision, op)

    @classmethod
    def block_jacobi(cls, op, precision=None):
        precision = op.precision if precision is None else precision
        h = C.c_void_p()
        check(lib().gbfem_preconditioner_block_jacobi_create(op.handle, precision, C.byref(h)))
        return cls(h, F32 if precision == F16 else precision, op)

    @classmethod
    def scaled_block_jacobi(cls, op, engine="tensor"):
        """For an FP32 operator with kappa_cell (no mass): z_c = H_t^-1 r_c / kappa_c
        with the shared kappa = 1 blocks H_t of the cell's boundary type.
        engine: "tensor" (tcgen05, 3xTF32) or "fma" for the tile products."""
        h = C.c_void_p()
        eng = {"tensor": 0, "fma": 1}[engine]
        check(lib().gbfem_preconditioner_scaled_block_jacobi_create_engine(op.handle, eng, C.byref(h)))
        return cls(h, F32, op)

    def status(self):
        """0, or 1 if a bounded wait in the tensor-core kernel gave up."""
        st = C.c_int()
        check(lib().gbfem_preconditioner_status(self.handle, C.byref(st)))
        return st.value

    SMOOTHERS = {"ssor": 2, "sor": 3, "gauss-seidel": 5, "jacobi": 6}

    @classmethod
    def sor(cls, assembled, method="ssor", iterations=1, relaxation=1.0):
        """Jacobi / Gauss-Seidel / SOR / SSOR sweeps of an assembled operator
        (Operator.assemble()), fem.solver.preconditioning.method."""
        h = C.c_void_p()
        check(lib().gbfem_preconditioner_sor_create(assembled.handle, cls.SMOOTHERS[method], iterations, relaxation,
                                                    C.byref(h)))
        return cls(h, assembled.precision, assembled)

    def __call__(self, r, z, stream=None):
        check(lib().gbfem_preconditioner_apply(self.handle, r.ptr, z.ptr, stream))

    def __del__(self):
        try:
            if self.handle:
                lib().gbfem_preconditioner_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def solver_params(method="cg", tolerance=1e-8, error_measure=RELATIVE, max_iterations=None, restart=20,
                  verbose=False, graph_chunk=0):
    p = SolverParams()
    check(lib().gbfem_solver_params_default(C.byref(p)))
    p.method = METHODS[method] if isinstance(method, str) else method
    p.tolerance = tolerance
    p.error_measure = error_measure
    if max_iterations is not None:
        p.max_iterations = max_iterations
    p.restart = restart
    p.verbose = 1 if verbose else 0
    p.graph_chunk = graph_chunk
    return p


class KrylovInverseOperator:
    """u = op^{-1}(f): the shape of dune-fem's KrylovInverseOperator
    (solver/krylovinverseoperators.hh:46-274, inverseoperatorinterface.hh:81-146):
    bind(op[, precond]), __call__(f, u), iterations(), info()."""

    def __init__(self, method="cg", tolerance=1e-8, error_measure=RELATIVE, max_iterations=None, restart=20,
                 verbose=False, graph_chunk=0):
        self.params = solver_params(method, tolerance, error_measure, max_iterations, restart, verbose, graph_chunk)
        self.op = None
        self.precond = None
        self._info = SolverInfo()

    def bind(self, op, precond=None):
        self.op = op
        self.precond = precond

    def unbind(self):
        self.op = None
        self.precond = None

    def __call__(self, f, u):
        if self.op is None:
            raise GbfemError(-1, "KrylovInverseOperator: no operator bound")
        pc = self.precond.handle if self.precond is not None else None
        check(lib().gbfem_solve(self.op.handle, pc, C.byref(self.params), f.ptr, u.ptr, C.byref(self._info)))
        return self._info

    def iterations(self):
        return self._info.iterations

    def info(self):
        i = self._info
        return {"converged": bool(i.converged), "iterations": i.iterations, "residual": i.residual,
                "time_ms": i.time_ms, "operator_applies": i.operator_applies,
                "preconditioner_applies": i.preconditioner_applies, "status": i.status,
                "fallbacks": i.fallbacks}


def solve_mixed(op64, op32, pc32, f, u, tolerance=1e-10, max_outer=50, inner_method="cg", inner_tolerance=1e-4,
                inner_max_iterations=100000, inner_restart=20, verbose=False, graph_chunk=0, outer="refinement",
                outer_restart=20):
    """FP64 outer iteration around an FP32 inner Krylov solve: outer =
    "refinement" (iterative refinement), "fgmres" or "fcg" (flexible FP64
    Krylov with the inner solve as preconditioner)."""
    p = IRParams()
    p.tolerance = tolerance
    p.max_outer = max_outer
    p.inner = solver_params(inner_method, inner_tolerance, RELATIVE, inner_max_iterations, inner_restart, verbose,
                            graph_chunk)
    p.outer_method = {"refinement": 0, "fgmres": FGMRES, "fcg": FCG}[outer]
    p.outer_restart = outer_restart
    info = SolverInfo()
    check(lib().gbfem_solve_mixed(op64.handle, op32.handle, pc32.handle if pc32 is not None else None,
                                  C.byref(p), f.ptr, u.ptr, C.byref(info)))
    return info


FN_EXP_FOURIER, FN_GAUSSIAN, FN_CONSTANT = 0, 1, 2


def fourier_modes(seed, nmodes=256, corr_length=0.1, stddev=1.0):
    """Seeded random Fourier modes of a log-Gaussian field: array [nmodes, 5]."""
    m = np.zeros(5 * nmodes)
    check(lib().gbfem_fourier_modes(seed, nmodes, corr_length, stddev, m.ctypes.data_as(C.POINTER(C.c_double))))
    return m.reshape(nmodes, 5)


def project(cells, order, kind, params=None, modes=None, quad_points=0, scale_by_volume=False, precision=F64,
            lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
    """L2 projection of a closed-form function onto DG Q_order: a DeviceArray."""
    g = grid_desc(cells, lower, upper)
    n = int(np.prod(cells)) * (order + 1) ** 3
    out = DeviceArray(n, precision)
    pr = np.zeros(8) if params is None else np.array(params, dtype=np.float64)
    md = np.ascontiguousarray(modes, dtype=np.float64).ravel() if modes is not None else None
    check(lib().gbfem_dg_project(C.byref(g), order, quad_points, kind, pr.ctypes.data_as(C.POINTER(C.c_double)),
                                 md.ctypes.data_as(C.POINTER(C.c_double)) if md is not None else None,
                                 0 if md is None else md.size // 5, 1 if scale_by_volume else 0, precision,
                                 out.ptr, None))
    return out


class RK3:
    """Explicit SSP-RK3 for u' = -M^{-1} A(u) (ExplicitRungeKuttaSolver + TVD3)."""

    def __init__(self, op):
        self.op = op
        self.handle = C.c_void_p()
        check(lib().gbfem_rk3_create(op.handle, C.byref(self.handle)))

    def step(self, u, dt, stream=None):
        check(lib().gbfem_rk3_step(self.handle, u.ptr, dt, stream))

    def __del__(self):
        try:
            if self.handle:
                lib().gbfem_rk3_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def hierarchical_permutation(order, dim=3):
    """perm[h] = non-hierarchical local index of the h-th hierarchical Legendre shape function."""
    perm = (C.c_int * ((order + 1) ** dim))()
    check(lib().gbfem_legendre_hierarchical_permutation(order, dim, perm))
    return np.array(perm[:], dtype=np.int64)


def cell_means(u, order):
    """The cell means of a DG field (one value per cell, a new DeviceArray)."""
    nc = u.n // (order + 1) ** 3
    out = DeviceArray(nc, u.precision)
    check(lib().gbfem_dg_cell_means(u.precision, nc, order, u.ptr, out.ptr, None))
    return out


def to_hierarchical(u, order):
    """The dof vector u (library order) in the hierarchical local order (a new DeviceArray)."""
    out = DeviceArray(u.n, u.precision)
    check(lib().gbfem_dg_permute(u.precision, u.n // (order + 1) ** 3, order, 1, u.ptr, out.ptr, None))
    return out


def from_hierarchical(u, order):
    """The inverse of to_hierarchical."""
    out = DeviceArray(u.n, u.precision)
    check(lib().gbfem_dg_permute(u.precision, u.n // (order + 1) ** 3, order, 0, u.ptr, out.ptr, None))
    return out


def time_step_estimate(op, power_iterations=30, seed=0):
    """(dt_estimate, dt_upper_bound) of a DG operator: the advective CFL-1 step
    h_min / (|b| (2p+1)) and 2 / rho(M^{-1} A) from the power method (inf when
    not applicable)."""
    est, ub = C.c_double(), C.c_double()
    check(lib().gbfem_dg_time_step_estimate(op.handle, power_iterations, seed, C.byref(est), C.byref(ub)))
    big = np.finfo(np.float64).max
    return (np.inf if est.value >= big else est.value), (np.inf if ub.value >= big else ub.value)


class TimeProvider:
    """Time, step counter and step size of an explicit time loop, as
    dune-fem's TimeProvider (solver/timeprovider.hh:35-200, 403-592):

        tp = TimeProvider(cfl=0.2)
        ode.initialize(u)                  # provides the operator's estimate
        tp.init()
        while tp.time() < end_time:
            ode.solve(u)                   # uses tp.deltaT(), provides the next estimate
            tp.next()

    deltaT = min(cfl * estimate, upper bound), both the minimum of what was
    provided since the step was fixed; a step with deltaT <= 0 is invalid and
    does not advance the time."""

    def __init__(self, start_time=0.0, cfl=1.0, update_step=1):
        self._time = float(start_time)
        self._step = 0
        self._cfl = float(cfl)
        self._update_step = int(update_step)
        self._counter = self._update_step  # the first initTimeStep fixes dt
        self._dt = 0.0
        self._valid = False
        self._init_estimate()

    def _init_estimate(self):
        self._dt_estimate = np.finfo(np.float64).max
        self._dt_upper = np.finfo(np.float64).max
        self._estimate_valid = False

    def _init_time_step(self, dt_estimate):
        self._counter += 1
        if self._counter >= self._update_step:
            self._dt = min(self._cfl * dt_estimate, self._dt_upper)
            self._valid = self._dt > 0.0
            self._counter = 0
        self._init_estimate()

    def _advance(self):
        if self._valid:
            self._time += self._dt
            self._step += 1

    def init(self, time_step=None):
        self._init_time_step(self._dt_estimate if time_step is None else time_step)

    def next(self, time_step=None):
        if time_step is None and not self._estimate_valid:
            raise RuntimeError("TimeProvider.next: no time step estimate was provided")
        self._advance()
        self._init_time_step(self._dt_estimate if time_step is None else time_step)

    def time(self):
        return self._time

    def timeStep(self):
        if not self._valid:
            raise RuntimeError("TimeProvider: the time step is not valid")
        return self._step

    def deltaT(self):
        if not self._valid:
            raise RuntimeError("TimeProvider: the time step is not valid")
        return self._dt

    def inverseDeltaT(self):
        return 1.0 / self.deltaT()

    def factor(self):
        return self._cfl

    def timeStepEstimate(self):
        return self._dt_estimate

    def provideTimeStepEstimate(self, dt_estimate):
        self._dt_estimate = min(self._dt_estimate, dt_estimate)
        self._estimate_valid = True

    def provideTimeStepUpperBound(self, upper_bound):
        self._dt_upper = min(self._dt_upper, upper_bound)
        self._estimate_valid = True

    def invalidateTimeStep(self):
        self._valid = False

    def timeStepValid(self):
        return self._valid


class ExplicitRungeKuttaSolver:
    """SSP-RK3 driven by a TimeProvider, as dune-fem's ExplicitRungeKuttaSolver
    (solver/rungekutta/explicit.hh:145-215): initialize() provides the
    operator's time-step estimate, solve(u) makes one step of tp.deltaT() and
    provides the estimate for the next one.  The estimate of the linear DG
    operator does not depend on u, so it is computed once (advective CFL-1
    step as the estimate, 2/rho(M^{-1}A) as the upper bound)."""

    def __init__(self, op, tp, power_iterations=30, seed=0, estimate=None):
        """estimate: a precomputed (dt_estimate, dt_upper_bound) pair, e.g. the
        FP64 operator's for an FP32 run, instead of computing it on op."""
        self.op, self.tp = op, tp
        self.rk = RK3(op)
        self.dt_estimate, self.dt_upper_bound = (time_step_estimate(op, power_iterations, seed)
                                                 if estimate is None else estimate)
        self.initialized = False

    def _provide(self):
        if np.isfinite(self.dt_estimate):
            self.tp.provideTimeStepEstimate(self.dt_estimate)
        if np.isfinite(self.dt_upper_bound):
            self.tp.provideTimeStepUpperBound(self.dt_upper_bound)
        if not (np.isfinite(self.dt_estimate) or np.isfinite(self.dt_upper_bound)):
            raise RuntimeError("ExplicitRungeKuttaSolver: the operator gives no time-step bound")

    def initialize(self, u):
        if not self.initialized:
            self._provide()
            self.initialized = True

    def solve(self, u, stream=None):
        if not self.initialized:
            raise RuntimeError("ExplicitRungeKuttaSolver wasn't initialized before first call!")
        self.rk.step(u, self.tp.deltaT(), stream)
        self._provide()

    def stages(self):
        return 3

    def order(self):
        return 3


class CNN:
    """The learned preconditioner's network on a cells^3 grid of DG Q_order."""

    def __init__(self, order, cells, seed=0):
        self.order = order
        self.cells = cells
        self.nloc = (order + 1) ** 3
        self.handle = C.c_void_p()
        check(lib().gbfem_cnn_create(order, cells, seed, C.byref(self.handle)))
        n = C.c_int64()
        check(lib().gbfem_cnn_num_params(self.handle, C.byref(n)))
        self.num_params = n.value

    def set_kappa(self, kappa):
        check(lib().gbfem_cnn_set_kappa(self.handle, kappa.precision if kappa is not None else F64,
                                        kappa.ptr if kappa is not None else None, None))

    @property
    def scale(self):
        v = C.c_double()
        check(lib().gbfem_cnn_get_output_scale(self.handle, C.byref(v)))
        return v.value

    @scale.setter
    def scale(self, v):
        check(lib().gbfem_cnn_set_output_scale(self.handle, float(v)))

    def set_conv_engine(self, engine):
        """"tensor" (default): the 3x3x3 convolutions as tcgen05 implicit
        GEMMs with TMA loads; "mma": warp-level mma.sync."""
        check(lib().gbfem_cnn_set_conv_engine(self.handle, {"tensor": 0, "mma": 1}[engine]))

    def status(self):
        """0, or 1 if a tensor-core convolution gave up on a bounded wait."""
        v = C.c_int()
        check(lib().gbfem_cnn_status(self.handle, C.byref(v)))
        return v.value

    def set_coarse(self, coarse=True):
        """Learned coarse-grid correction: cell means in, cell means out."""
        check(lib().gbfem_cnn_set_coarse(self.handle, 1 if coarse else 0))

    def forward(self, r, z, accumulate=False):
        check(lib().gbfem_cnn_forward(self.handle, r.precision, r.ptr, z.ptr, 1 if accumulate else 0, None))

    def loss_grad(self, r, target):
        l = C.c_double()
        check(lib().gbfem_cnn_loss_grad(self.handle, r.precision, r.ptr, target.ptr, C.byref(l), None))
        return l.value

    def train_step(self, r, target, lr=1e-3):
        l = C.c_double()
        check(lib().gbfem_cnn_train_step(self.handle, r.precision, r.ptr, target.ptr, lr, C.byref(l), None))
        return l.value

    def train_step_grad(self, r, grad_z, lr=1e-3):
        """Adam step for a caller-supplied gradient dL/dz of the dof-space output."""
        check(lib().gbfem_cnn_train_step_grad(self.handle, r.precision, r.ptr, grad_z.ptr, lr, None))

    def params(self):
        a = np.zeros(self.num_params, dtype=np.float32)
        check(lib().gbfem_cnn_get_params(self.handle, a.ctypes.data))
        return a

    def set_params(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        check(lib().gbfem_cnn_set_params(self.handle, a.ctypes.data))

    def grads(self):
        a = np.zeros(self.num_params, dtype=np.float32)
        check(lib().gbfem_cnn_get_grads(self.handle, a.ctypes.data))
        return a

    def save(self, path):
        check(lib().gbfem_cnn_save(self.handle, path.encode()))

    def load(self, path):
        check(lib().gbfem_cnn_load(self.handle, path.encode()))

    def preconditioner(self, bj, op=None):
        """op None: z = bj(r) + NN(r); op given: z = NN(r), z += bj(r - op(z)).
        bj is the fallback of flexible solvers."""
        h = C.c_void_p()
        check(lib().gbfem_preconditioner_learned_create(self.handle, bj.handle if bj is not None else None,
                                                        op.handle if op is not None else None, C.byref(h)))
        return Preconditioner(h, bj.precision if bj is not None else F64, (self, bj, op))

    def __del__(self):
        try:
            if self.handle:
                lib().gbfem_cnn_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def convert(x, precision):
    """A copy of the dof vector x in the given precision."""
    y = DeviceArray(x.n, precision)
    check(lib().gbfem_convert(x.n, x.precision, x.ptr, precision, y.ptr, None))
    return y


def copy(x):
    y = DeviceArray(x.n, x.precision)
    check(lib().gbfem_copy(x.precision, x.n, x.ptr, y.ptr, None))
    return y
