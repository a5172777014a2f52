"""CPU (numpy) restatement of a general DG form's residual, for checking the
run-time compiled form kernels (dune-fem_gb300/csrc/form_kernel.cuh).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker; the product
never imports it.

What it computes is dune-fem's GalerkinOperator over an integrands object
(dune/fem/schemes/galerkin.hh): per cell the interior integrand at the tensor
Gauss points (addInteriorIntegral, galerkin.hh:332-360), on every face of the
cell the own side's part of the skeleton integrand with the neighbour's traces
(addSkeletonIntegral, :475-537; the neighbour's part is the same function
seen from the neighbour), and the boundary integrand on non-periodic boundary
faces (addBoundaryIntegral, :414-435).  Gauss rules and the orthonormal
Legendre shape functions come from oracle.py, which are pinned against the
reference's own tables.  Values are evaluated directly by einsum over the
tensor tables (no sum factorisation, no shared code with the kernels).

The integrands are numpy callables over P points at once:
  interior(x[P,3], u[P,M], g[P,M,3])                          -> s[P,M], F[P,M,3]
  skeleton(x, n[3], sigma, uL, gL, uR, gR)                    -> s, F   (own side)
  boundary(x, n[3], sigma, u, g)                              -> s, F
sipg() builds them from a flux, a source, a convective flux with its wave
speed and Dirichlet data as the form's definition states, with A^T n
(A = dF/d grad u) by the complex step, exact to rounding for analytic fluxes.
"""
import numpy as np

import oracle


def tables(n, q):
    x, w = oracle.gauss(q)
    B = np.array([[oracle.legendre(i, xa) for i in range(n)] for xa in x])
    D = np.array([[oracle.legendre_d(i, xa) for i in range(n)] for xa in x])
    tr = np.array([[oracle.legendre(i, s) for i in range(n)] for s in (0.0, 1.0)])
    dtr = np.array([[oracle.legendre_d(i, s) for i in range(n)] for s in (0.0, 1.0)])
    return x, w, B, D, tr, dtr


class FormSpec:
    """Grid, space and integrands of a form."""

    def __init__(self, cells, order, components, interior, skeleton, boundary, quad_points=0, penalty=None,
                 periodic=(0, 0, 0), lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
        self.cells = tuple(int(c) for c in cells)
        self.order = order
        self.n = order + 1
        self.q = quad_points or order + 2
        self.M = components
        self.interior, self.skeleton, self.boundary = interior, skeleton, boundary
        self.penalty = 10.0 * (order + 1) ** 2 if penalty is None else penalty
        self.periodic = tuple(periodic)
        self.lower = np.array(lower, dtype=np.float64)
        self.upper = np.array(upper, dtype=np.float64)
        self.h = (self.upper - self.lower) / np.array(self.cells)
        self.ncells = int(np.prod(self.cells))
        self.nloc = self.M * self.n ** 3
        self.ndofs = self.ncells * self.nloc
        self.tabs = tables(self.n, self.q)


def _interp(Uc, T0, T1, T2):
    return np.einsum("ai,bj,ck,ijkm->abcm", T0, T1, T2, Uc)


def _test(Rq, T0, T1, T2):
    return np.einsum("ai,bj,ck,abcm->ijkm", T0, T1, T2, Rq)


def residual(spec, u):
    """S(u) as a dof vector (float64 or complex, as u)."""
    n, M = spec.n, spec.M
    xg, wg, B, D, tr, dtr = spec.tabs
    nc = spec.cells
    U = np.asarray(u).reshape(nc[2], nc[1], nc[0], n, n, n, M)
    out = np.zeros(U.shape, dtype=np.result_type(U.dtype, np.float64))
    vol = float(np.prod(spec.h))
    invh = 1.0 / spec.h

    def cell_of(cx, cy, cz):
        return U[cz, cy, cx]

    def evaluate(Uc, vals, ders):
        """u [P0,P1,P2,M] and g [P0,P1,P2,M,3] for per-axis value / derivative tables."""
        uq = _interp(Uc, *vals)
        g = np.stack([_interp(Uc, *[ders[k] if a == k else vals[a] for a in range(3)]) * invh[k]
                      for k in range(3)], axis=-1)
        return uq, g

    def add_test(r, s, F, W, vals, ders):
        r += _test(s * W[..., None], *vals)
        for k in range(3):
            r += _test(F[..., k] * W[..., None] * invh[k], *[ders[k] if a == k else vals[a] for a in range(3)])

    for cz in range(nc[2]):
        for cy in range(nc[1]):
            for cx in range(nc[0]):
                c = (cx, cy, cz)
                Uc = cell_of(*c)
                r = out[cz, cy, cx]
                # ---- volume
                vals, ders = (B, B, B), (D, D, D)
                uq, g = evaluate(Uc, vals, ders)
                P = uq.shape[:3]
                x = np.stack(np.meshgrid(*[spec.lower[k] + (c[k] + xg) * spec.h[k] for k in range(3)],
                                         indexing="ij"), axis=-1)
                s, F = spec.interior(x.reshape(-1, 3), uq.reshape(-1, M), g.reshape(-1, M, 3))
                W = np.einsum("a,b,c->abc", wg, wg, wg) * vol
                add_test(r, s.reshape(*P, M), F.reshape(*P, M, 3), W, vals, ders)
                # ---- faces
                for d in range(3):
                    area = vol / spec.h[d]
                    sigma = spec.penalty / spec.h[d]
                    for side in (0, 1):
                        nb = list(c)
                        nb[d] += 1 if side else -1
                        boundary = False
                        if nb[d] < 0 or nb[d] >= nc[d]:
                            if spec.periodic[d]:
                                nb[d] %= nc[d]
                            else:
                                boundary = True
                        own_v = [tr[side][None, :] if a == d else B for a in range(3)]
                        own_d = [dtr[side][None, :] if a == d else D for a in range(3)]
                        uL, gL = evaluate(Uc, own_v, own_d)
                        P = uL.shape[:3]
                        coords = [np.array([c[k] + side], float) if k == d else c[k] + xg for k in range(3)]
                        x = np.stack(np.meshgrid(*[spec.lower[k] + coords[k] * spec.h[k] for k in range(3)],
                                                 indexing="ij"), axis=-1).reshape(-1, 3)
                        nvec = np.zeros(3)
                        nvec[d] = 1.0 if side else -1.0
                        wv = [np.ones(1) if a == d else wg for a in range(3)]
                        W = np.einsum("a,b,c->abc", *wv) * area
                        if boundary:
                            s, F = spec.boundary(x, nvec, sigma, uL.reshape(-1, M), gL.reshape(-1, M, 3))
                        else:
                            nb_v = [tr[1 - side][None, :] if a == d else B for a in range(3)]
                            nb_d = [dtr[1 - side][None, :] if a == d else D for a in range(3)]
                            uR, gR = evaluate(cell_of(*nb), nb_v, nb_d)
                            s, F = spec.skeleton(x, nvec, sigma, uL.reshape(-1, M), gL.reshape(-1, M, 3),
                                                 uR.reshape(-1, M), gR.reshape(-1, M, 3))
                        add_test(r, s.reshape(*P, M), F.reshape(*P, M, 3), W, own_v, own_d)
    return out.reshape(-1)


def linearize(spec, u, du, h=1e-3):
    """S'(u) du by Richardson-extrapolated central differences (O(h^4))."""
    def central(t):
        return (residual(spec, u + t * du) - residual(spec, u - t * du)) / (2 * t)
    return (4.0 * central(h / 2) - central(h)) / 3.0


def sipg(M, flux=None, source=None, advection=None, wavespeed=None, dirichlet=None, symmetry=1):
    """interior, skeleton, boundary callables of the interior-penalty form:
    volume F:grad v + s.v - Fa:grad v; faces sigma [u][v] - {F}.n [v]
    - symmetry [u] {A^T n}.grad v + Lax-Friedrichs 1/2 (Fa(uL) + Fa(uR)).n
    + 1/2 lambda [u]; weak Dirichlet by the same terms against gD, natural
    boundary (dirichlet None): only the convective flux Fa(u).n."""

    def zeros(u):
        P = u.shape[0]
        return np.zeros((P, M), dtype=u.dtype), np.zeros((P, M, 3), dtype=u.dtype)

    def flux_transpose(x, u, g, jump, n):
        step = 1e-30
        c = np.zeros(g.shape, dtype=np.result_type(g.dtype, jump.dtype))
        for m in range(M):
            for k in range(3):
                gg = g.astype(np.complex128)
                gg[:, m, k] += 1j * step
                dF = flux(x, u.astype(np.complex128), gg).imag / step  # [P, M', 3]
                c[:, m, k] = np.einsum("pm,pmj,j->p", jump, dF, n)
        return c

    def interior(x, u, g):
        s, F = zeros(u)
        if flux:
            F = F + flux(x, u, g)
        if source:
            s = s + source(x, u, g)
        if advection:
            F = F - advection(x, u)
        return s, F

    def lax_friedrichs(x, n, uL, uR):
        fn = np.einsum("pmk,k->pm", advection(x, uL) + advection(x, uR), n)
        lam = np.maximum(wavespeed(x, uL, n), wavespeed(x, uR, n))
        return 0.5 * (fn + lam[:, None] * (uL - uR))

    def skeleton(x, n, sigma, uL, gL, uR, gR):
        s, F = zeros(uL)
        if flux:
            jump = uL - uR
            fn = np.einsum("pmk,k->pm", flux(x, uL, gL) + flux(x, uR, gR), n)
            s = s + sigma * jump - 0.5 * fn
            if symmetry:
                F = F - 0.5 * symmetry * flux_transpose(x, uL, gL, jump, n)
        if advection:
            s = s + lax_friedrichs(x, n, uL, uR)
        return s, F

    def boundary(x, n, sigma, u, g):
        s, F = zeros(u)
        if dirichlet is not None:
            gd = dirichlet(x)
            jump = u - gd
            if flux:
                s = s + sigma * jump - np.einsum("pmk,k->pm", flux(x, u, g), n)
                if symmetry:
                    F = F - symmetry * flux_transpose(x, u, g, jump, n)
            if advection:
                s = s + lax_friedrichs(x, n, u, gd.astype(u.dtype))
        elif advection:
            s = s + np.einsum("pmk,k->pm", advection(x, u), n)
        return s, F

    return interior, skeleton, boundary
