"""ctypes wrapper of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None
OPFN = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double))


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "oracle.cpp")):
            build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.oracle_gauss.argtypes = [C.c_int, dp, dp]
        L.oracle_legendre.argtypes = [C.c_int, C.c_double]
        L.oracle_legendre.restype = C.c_double
        L.oracle_legendre_d.argtypes = [C.c_int, C.c_double]
        L.oracle_legendre_d.restype = C.c_double
        dg_args = [ip, dp, dp, ip, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, C.c_int, dp]
        L.oracle_dg_apply.argtypes = dg_args + [dp, dp, C.c_int]
        L.oracle_dg_block_diagonal.argtypes = dg_args + [dp, C.c_int]
        L.oracle_dg_apply_cells.argtypes = dg_args + [dp, dp, C.c_longlong, C.c_longlong, C.c_int]
        L.oracle_dg_project.argtypes = [ip, dp, dp, C.c_int, C.c_int, C.c_int, dp, dp, C.c_int, C.c_int, dp]
        L.oracle_dg_rk3_step.argtypes = dg_args + [dp, C.c_double, C.c_int]
        L.oracle_dg_rk3_step_planes.argtypes = dg_args + [dp, C.c_double, C.c_int, C.c_int, C.c_int]
        L.oracle_q1_apply.argtypes = [ip, dp, dp, C.c_double, C.c_double, dp, dp, C.c_int]
        L.oracle_cg.argtypes = [C.c_longlong, OPFN, C.c_void_p, OPFN, C.c_void_p, dp, dp, C.c_double, C.c_int,
                                C.c_int, dp]
        L.oracle_gmres.argtypes = [C.c_longlong, OPFN, C.c_void_p, OPFN, C.c_void_p, dp, dp, C.c_int, C.c_double,
                                   C.c_int, C.c_int, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def gauss(m):
    p = np.zeros(m)
    w = np.zeros(m)
    lib().oracle_gauss(m, _dp(p), _dp(w))
    return p, w


def legendre(k, x):
    return lib().oracle_legendre(k, float(x))


def legendre_d(k, x):
    return lib().oracle_legendre_d(k, float(x))


class DGProblem:
    """Parameters of the DG operator, as passed to the oracle."""

    def __init__(self, cells, order, quad_points=0, diffusion=1.0, penalty=None, mass=0.0, velocity=(0, 0, 0),
                 weak_dirichlet=True, periodic=(0, 0, 0), lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
        self.cells = np.array(cells, dtype=np.int32)
        self.lower = np.array(lower, dtype=np.float64)
        self.upper = np.array(upper, dtype=np.float64)
        self.periodic = np.array(periodic, dtype=np.int32)
        self.order = order
        self.quad = quad_points if quad_points else order + 2
        self.diffusion = diffusion
        self.penalty = 10.0 * (order + 1) ** 2 if penalty is None else penalty
        self.mass = mass
        self.velocity = np.array(velocity, dtype=np.float64)
        # True: symmetric SIPG on the boundary; "dgelliptic": the boundary of
        # dune-fem's DGEllipticOperator (symmetry term weighted by 1/2)
        self.weak_dirichlet = 2 if weak_dirichlet == "dgelliptic" else (1 if weak_dirichlet else 0)
        self.nloc = (order + 1) ** 3
        self.ncells = int(np.prod(self.cells))
        self.ndofs = self.ncells * self.nloc

    def _args(self, kappa):
        k = _dp(kappa) if kappa is not None else None
        return [_ip(self.cells), _dp(self.lower), _dp(self.upper), _ip(self.periodic), self.order, self.quad,
                self.diffusion, self.penalty, self.mass, _dp(self.velocity), self.weak_dirichlet, k]

    def apply(self, u, kappa=None, nthreads=1):
        u = np.ascontiguousarray(u, dtype=np.float64)
        w = np.zeros(self.ndofs)
        if kappa is not None:
            kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        lib().oracle_dg_apply(*self._args(kappa), _dp(u), _dp(w), nthreads)
        return w

    def apply_cells(self, u, w, c0, c1, kappa=None, nthreads=1):
        """Adds the contributions of cells [c0, c1) to w (a bounded sample of an apply)."""
        lib().oracle_dg_apply_cells(*self._args(kappa), _dp(u), _dp(w), int(c0), int(c1), nthreads)

    def rk3_step_planes(self, u, dt, z0, z1, kappa=None, nthreads=1):
        """One SSP-RK3 step evaluated only where the z-planes [z0, z1) depend
        on it; returns a copy of u with those planes advanced (the other
        planes unchanged)."""
        u = np.array(u, dtype=np.float64)
        if kappa is not None:
            kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        rc = lib().oracle_dg_rk3_step_planes(*self._args(kappa), _dp(u), dt, int(z0), int(z1), nthreads)
        if rc != 0:
            raise ValueError("rk3_step_planes: bad plane range")
        return u

    def rk3_step(self, u, dt, kappa=None, nthreads=1):
        """One SSP-RK3 step of u' = -A(u)/|K| (in place on a copy; returns it)."""
        u = np.array(u, dtype=np.float64)
        if kappa is not None:
            kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        lib().oracle_dg_rk3_step(*self._args(kappa), _dp(u), dt, nthreads)
        return u

    def project(self, kind, params=None, modes=None, scale_by_volume=False):
        """L2 projection of a closed-form function (0 exp-Fourier, 1 Gaussian, 2 constant)."""
        out = np.zeros(self.ndofs)
        pr = np.zeros(8) if params is None else np.array(params, dtype=np.float64)
        md = np.zeros(5) if modes is None else np.ascontiguousarray(modes, dtype=np.float64)
        nm = 0 if modes is None else md.size // 5
        lib().oracle_dg_project(_ip(self.cells), _dp(self.lower), _dp(self.upper), self.order, self.quad, kind,
                                _dp(pr), _dp(md), nm, 1 if scale_by_volume else 0, _dp(out))
        return out

    def block_diagonal(self, kappa=None, nthreads=1):
        b = np.zeros(self.ncells * self.nloc * self.nloc)
        if kappa is not None:
            kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        lib().oracle_dg_block_diagonal(*self._args(kappa), _dp(b), nthreads)
        return b.reshape(self.ncells, self.nloc, self.nloc)


def q1_apply(cells, u, diffusion=1.0, mass=0.0, lower=(0.0, 0.0), upper=(1.0, 1.0), diag_only=False):
    cells = np.array(cells, dtype=np.int32)
    lo = np.array(lower, dtype=np.float64)
    up = np.array(upper, dtype=np.float64)
    n = (cells[0] + 1) * (cells[1] + 1)
    u = np.zeros(n) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    w = np.zeros(n)
    lib().oracle_q1_apply(_ip(cells), _dp(lo), _dp(up), diffusion, mass, _dp(u), _dp(w), 1 if diag_only else 0)
    return w


def _wrap(fn):
    if fn is None:
        return OPFN(), None

    def cb(ctx, x, y, _fn=fn):
        n = cb.n
        xa = np.ctypeslib.as_array(x, shape=(n,))
        ya = np.ctypeslib.as_array(y, shape=(n,))
        ya[:] = _fn(xa.copy())

    c = OPFN(cb)
    return c, cb


def cg(op, b, x0=None, prec=None, epsilon=1e-10, max_iter=1000, criterion=1):
    """LinearSolver::cg restated; op/prec are python callables on numpy arrays."""
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    fop, cbo = _wrap(op)
    cbo.n = n
    fpr, cbp = _wrap(prec)
    if cbp is not None:
        cbp.n = n
    res = C.c_double()
    it = lib().oracle_cg(n, fop, None, fpr, None, _dp(x), _dp(b), epsilon, max_iter, criterion, C.byref(res))
    return it, x, res.value


def gmres(op, b, restart, x0=None, prec=None, tolerance=1e-10, max_iter=1000, criterion=1):
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    fop, cbo = _wrap(op)
    cbo.n = n
    fpr, cbp = _wrap(prec)
    if cbp is not None:
        cbp.n = n
    res = C.c_double()
    it = lib().oracle_gmres(n, fop, None, fpr, None, _dp(x), _dp(b), restart, tolerance, max_iter, criterion,
                            C.byref(res))
    return it, x, res.value
