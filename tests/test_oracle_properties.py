"""Properties of the CPU oracle itself (no GPU): the invariants the reference's
own tests rely on (apply = assembled Jacobian . vector,
dune/fempy/test/testoperator.py:33-71; symmetry of SIPG; thread-count
invariance)."""
import numpy as np
import pytest

from conftest import relmax


@pytest.mark.parametrize("order", [1, 2, 3])
def test_sipg_is_symmetric(orc, order):
    prob = orc.DGProblem((3, 2, 2), order, mass=0.3)
    rng = np.random.default_rng(order)
    u, v = rng.uniform(-1, 1, prob.ndofs), rng.uniform(-1, 1, prob.ndofs)
    a, b = prob.apply(u) @ v, u @ prob.apply(v)
    assert abs(a - b) < 1e-12 * (abs(a) + abs(b))


def test_sipg_is_positive_definite_on_random_vectors(orc):
    prob = orc.DGProblem((2, 2, 2), 2)
    rng = np.random.default_rng(0)
    for _ in range(5):
        u = rng.uniform(-1, 1, prob.ndofs)
        assert u @ prob.apply(u) > 0


def test_apply_equals_assembled_matrix_times_vector(orc):
    """Matrix-free apply == (dense matrix assembled column by column) . u
    (the self-consistency check of dune/fempy/test/testoperator.py:33-71)."""
    prob = orc.DGProblem((2, 2, 1), 1, velocity=(0.4, -0.2, 0.1), mass=1.0, periodic=(1, 0, 0))
    n = prob.ndofs
    A = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        A[:, j] = prob.apply(e)
    u = np.random.default_rng(1).uniform(-1, 1, n)
    assert relmax(A @ u, prob.apply(u)) < 1e-14
    # the diagonal blocks of that matrix are the oracle's block diagonal
    B = prob.block_diagonal()
    for c in range(prob.ncells):
        s = slice(c * prob.nloc, (c + 1) * prob.nloc)
        assert relmax(B[c], A[s, s]) < 1e-14


def test_threaded_apply_matches_serial(orc):
    prob = orc.DGProblem((4, 4, 4), 2, velocity=(1, 0.5, 0.25))
    u = np.random.default_rng(2).uniform(-1, 1, prob.ndofs)
    assert relmax(prob.apply(u, nthreads=4), prob.apply(u, nthreads=1)) < 1e-14


def test_constant_is_in_kernel_of_periodic_diffusion(orc):
    """On a fully periodic grid the SIPG Laplacian annihilates constants."""
    prob = orc.DGProblem((3, 3, 3), 2, periodic=(1, 1, 1), weak_dirichlet=False)
    u = np.zeros(prob.ndofs)
    u[::prob.nloc] = 1.0  # L_0 = 1 in every cell
    assert np.max(np.abs(prob.apply(u))) < 1e-12


def test_smoother_oracle_converges_as_a_stationary_iteration():
    """The restated sweeps are stationary iterations: on a diagonally dominant
    matrix, many Jacobi / Gauss-Seidel / SSOR sweeps from 0 reach A^{-1} b."""
    import numpy as np
    import smoother_oracle
    rng = np.random.default_rng(0)
    n = 12
    A = rng.uniform(-1, 1, (n, n)) * (rng.uniform(0, 1, (n, n)) < 0.4)
    A = A + A.T + np.diag(2.0 + np.abs(A).sum(axis=1) + np.abs(A).sum(axis=0))
    b = rng.uniform(-1, 1, n)
    x = np.linalg.solve(A, b)
    for method in ("jacobi", "gauss-seidel", "ssor"):
        y = smoother_oracle.smoother_apply(A, b, method, iterations=200)
        assert np.max(np.abs(y - x)) < 1e-12 * np.max(np.abs(x)), method
    # one Gauss-Seidel sweep is the forward substitution with the lower triangle
    y = smoother_oracle.smoother_apply(A, b, "gauss-seidel", iterations=1)
    assert np.allclose(y, np.linalg.solve(np.tril(A), b), rtol=0, atol=1e-14)


@pytest.mark.parametrize("zr", [(0, 2), (3, 5), (6, 8)])
def test_rk3_step_on_planes_equals_full_step(orc, zr):
    """The plane-restricted SSP-RK3 step (used to compare whole planes of a
    large grid) against the full step: periodic in z, so the first and last
    plane ranges wrap."""
    kw = dict(diffusion=1e-2, velocity=(1.0, 0.5, 0.25), periodic=(1, 1, 1), weak_dirichlet=False)
    prob = orc.DGProblem((3, 4, 8), 2, **kw)
    u = np.random.default_rng(5).uniform(-1, 1, prob.ndofs)
    dt = 1e-3
    full = prob.rk3_step(u, dt)
    part = prob.rk3_step_planes(u, dt, zr[0], zr[1], nthreads=3)
    per = 3 * 4 * 27
    sl = slice(zr[0] * per, zr[1] * per)
    assert relmax(part[sl], full[sl]) < 1e-14
    rest = np.ones(prob.ndofs, bool)
    rest[sl] = False
    assert np.array_equal(part[rest], u[rest])


def test_rk3_step_on_planes_non_periodic(orc):
    prob = orc.DGProblem((3, 3, 7), 1, diffusion=0.5, mass=0.2)
    u = np.random.default_rng(6).uniform(-1, 1, prob.ndofs)
    full = prob.rk3_step(u, 1e-3)
    per = 9 * 8
    for z0, z1 in ((0, 1), (3, 4), (5, 7)):
        part = prob.rk3_step_planes(u, 1e-3, z0, z1)
        assert relmax(part[z0 * per:z1 * per], full[z0 * per:z1 * per]) < 1e-14


def test_apply_on_planes_with_neighbour_planes_equals_full_apply(orc):
    """apply_cells over the planes [z0-1, z1+1) gives complete rows on
    [z0, z1): the sampling rule of the full-size parity tests."""
    prob = orc.DGProblem((4, 3, 6), 2, mass=0.3)
    u = np.random.default_rng(8).uniform(-1, 1, prob.ndofs)
    full = prob.apply(u)
    nxy, per = 12, 12 * 27
    for z0, z1 in ((0, 2), (2, 4), (4, 6)):
        w = np.zeros(prob.ndofs)
        prob.apply_cells(u, w, max(0, z0 - 1) * nxy, min(6, z1 + 1) * nxy, nthreads=2)
        assert relmax(w[z0 * per:z1 * per], full[z0 * per:z1 * per]) < 1e-14
