"""GPU Krylov solvers (through the C-ABI) against the oracle's restatement of
dune-fem's LinearSolver::cg / gmres, itself pinned to the reference's
compiled templates (tests/test_oracle_pins.py)."""
import numpy as np
import pytest

from conftest import relmax

pytestmark = pytest.mark.gpu


def _problem(gb, orc, cells=(3, 3, 3), order=2, **kw):
    op = gb.DGOperator(cells, order, **kw)
    prob = orc.DGProblem(cells, order, **kw)
    f = np.random.default_rng(4).uniform(-1, 1, prob.ndofs)
    return op, prob, f


def _solve(gb, op, f, method="cg", pc=None, tol=1e-10, **kw):
    inv = gb.KrylovInverseOperator(method, tolerance=tol, **kw)
    inv.bind(op, pc)
    u = gb.DeviceArray(op.size, op.precision)
    u.clear()
    inv(gb.DeviceArray.from_numpy(f, op.precision), u)
    return inv.info(), u.numpy()


def test_cg_matches_oracle_cg(gb, orc):
    op, prob, f = _problem(gb, orc)
    info, u = _solve(gb, op, f, "cg")
    it, uo, _ = orc.cg(prob.apply, f, epsilon=1e-10, max_iter=10000)
    assert info["converged"]
    assert abs(info["iterations"] - it) <= 1
    assert relmax(u, uo) < 1e-8
    assert info["operator_applies"] == info["iterations"] + 1


def test_pcg_diagonal_and_block_jacobi_match_oracle(gb, orc):
    op, prob, f = _problem(gb, orc, mass=0.5)
    blocks = prob.block_diagonal()
    dinv = 1.0 / np.einsum("cii->ci", blocks).ravel()
    binv = np.linalg.inv(blocks)
    nl = prob.nloc
    bj = lambda r: np.einsum("cij,cj->ci", binv, r.reshape(-1, nl)).ravel()
    for pc, ref_pc in ((gb.Preconditioner.diagonal(op), lambda r: r * dinv),
                       (gb.Preconditioner.block_jacobi(op), bj)):
        info, u = _solve(gb, op, f, "cg", pc)
        it, uo, _ = orc.cg(prob.apply, f, prec=ref_pc, epsilon=1e-10, max_iter=10000)
        assert info["converged"]
        assert abs(info["iterations"] - it) <= 1
        assert relmax(u, uo) < 1e-8


def test_block_jacobi_apply_matches_dense_inverse(gb, orc):
    op, prob, f = _problem(gb, orc, cells=(2, 3, 2), order=3, velocity=(0.5, 0.1, 0.0))
    pc = gb.Preconditioner.block_jacobi(op)
    z = gb.DeviceArray(op.size)
    pc(gb.DeviceArray.from_numpy(f), z)
    binv = np.linalg.inv(prob.block_diagonal())
    ref = np.einsum("cij,cj->ci", binv, f.reshape(-1, prob.nloc)).ravel()
    assert relmax(z.numpy(), ref) < 1e-11


def test_gmres_matches_oracle_gmres_nonsymmetric(gb, orc):
    op, prob, f = _problem(gb, orc, velocity=(1.0, 0.5, -0.25), diffusion=0.1)
    info, u = _solve(gb, op, f, "gmres", restart=10)
    it, uo, _ = orc.gmres(prob.apply, f, 10, tolerance=1e-10, max_iter=10000)
    assert info["converged"]
    assert abs(info["iterations"] - it) <= 1
    assert relmax(u, uo) < 1e-8


@pytest.mark.parametrize("method", ["bicgstab", "fcg", "fgmres", "gmres"])
def test_other_methods_reach_tolerance(gb, orc, method):
    kw = dict(velocity=(0.3, 0.0, 0.2)) if method in ("bicgstab", "fgmres", "gmres") else {}
    op, prob, f = _problem(gb, orc, **kw)
    pc = gb.Preconditioner.block_jacobi(op)
    info, u = _solve(gb, op, f, method, pc, restart=10 if "gmres" in method else 4)
    assert info["converged"], info
    res = f - prob.apply(u)
    assert np.linalg.norm(res) <= 2e-10 * np.linalg.norm(f)


def test_mixed_precision_refinement_reaches_fp64_tolerance(gb, orc):
    cells, order = (4, 4, 4), 3
    op64 = gb.DGOperator(cells, order)
    op32 = gb.DGOperator(cells, order, precision=gb.F32)
    pc32 = gb.Preconditioner.block_jacobi(op64, gb.F32)
    prob = orc.DGProblem(cells, order)
    f = np.random.default_rng(5).uniform(-1, 1, prob.ndofs)
    u = gb.DeviceArray(op64.size)
    u.clear()
    info = gb.solve_mixed(op64, op32, pc32, gb.DeviceArray.from_numpy(f), u, tolerance=1e-10, inner_tolerance=1e-3)
    assert info.converged and info.residual <= 1e-10
    x = u.numpy()
    assert np.linalg.norm(f - prob.apply(x)) <= 1.01e-10 * np.linalg.norm(f)
    _, ref = _solve(gb, op64, f, "cg", tol=1e-12)
    assert relmax(x, ref) < 1e-7


def test_q1_diagonal_pcg_matches_oracle_and_converges_at_h2(gb, orc):
    """Config-1 shape: -lap u + u = f, Q1, u = sin(pi x) sin(pi y), Dirichlet."""
    errs = []
    for N in (16, 32):
        op = gb.Q1Operator((N, N), diffusion=1.0, mass=1.0)
        f = q1_rhs(N)
        pc = gb.Preconditioner.diagonal(op)
        info, u = _solve(gb, op, f, "cg", pc)
        dg = orc.q1_apply((N, N), None, 1.0, 1.0, diag_only=True)
        it, uo, _ = orc.cg(lambda x: orc.q1_apply((N, N), x, 1.0, 1.0), f, prec=lambda r: r / dg, epsilon=1e-10)
        assert info["converged"] and abs(info["iterations"] - it) <= 1
        assert relmax(u, uo) < 1e-8
        xs = np.linspace(0, 1, N + 1)
        X, Y = np.meshgrid(xs, xs)
        errs.append(np.max(np.abs(u - (np.sin(np.pi * X) * np.sin(np.pi * Y)).ravel())))
    assert np.log2(errs[0] / errs[1]) > 1.8  # second order at the nodes


def q1_rhs(N):
    """b_i = int f phi_i with f = (2 pi^2 + 1) sin(pi x) sin(pi y), 3x3 Gauss per cell; b = 0 on the boundary."""
    h = 1.0 / N
    g, w = np.polynomial.legendre.leggauss(3)
    g, w = 0.5 * (g + 1), 0.5 * w
    b = np.zeros((N + 1) * (N + 1))
    for ey in range(N):
        for ex in range(N):
            for qy in range(3):
                for qx in range(3):
                    x, y = (ex + g[qx]) * h, (ey + g[qy]) * h
                    fv = (2 * np.pi ** 2 + 1) * np.sin(np.pi * x) * np.sin(np.pi * y) * w[qx] * w[qy] * h * h
                    for k in range(4):
                        kx, ky = k & 1, k >> 1
                        phi = (g[qx] if kx else 1 - g[qx]) * (g[qy] if ky else 1 - g[qy])
                        b[(ey + ky) * (N + 1) + ex + kx] += fv * phi
    b2 = b.reshape(N + 1, N + 1)
    b2[0, :] = b2[-1, :] = b2[:, 0] = b2[:, -1] = 0.0
    return b


def test_nonconvergence_is_a_negative_iteration_count(gb, orc):
    op, prob, f = _problem(gb, orc)
    info, _ = _solve(gb, op, f, "cg", max_iterations=3)
    assert info["iterations"] == -3 and not info["converged"]


def test_nan_input_reports_nonfinite(gb, orc):
    op, prob, f = _problem(gb, orc)
    f = f.copy()
    f[7] = np.nan
    info, _ = _solve(gb, op, f, "cg", max_iterations=50)
    assert not info["converged"]


@pytest.mark.parametrize("kw", [dict(), dict(velocity=(0.4, -0.3, 0.2), mass=0.7, periodic=(1, 0, 1))])
def test_assembled_matrix_times_vector_equals_matrix_free_apply(gb, orc, kw):
    """apply == assembled Jacobian . vector (dune/fempy/test/testoperator.py:33-71),
    on both kernels' results, and the assembled operator drives the solvers."""
    cells, order = (3, 4, 2), 2
    op = gb.DGOperator(cells, order, algorithm=gb.ALGO_QUADRATURE, **kw)
    A = op.assemble()
    prob = orc.DGProblem(cells, order, **kw)
    u = np.random.default_rng(8).uniform(-1, 1, prob.ndofs)
    y, ya = gb.DeviceArray(prob.ndofs), gb.DeviceArray(prob.ndofs)
    du = gb.DeviceArray.from_numpy(u)
    op(du, y)
    A(du, ya)
    assert relmax(ya.numpy(), y.numpy()) < 1e-13
    assert relmax(ya.numpy(), prob.apply(u)) < 1e-12
    assert relmax(A.diagonal().numpy(), op.diagonal().numpy()) < 1e-14
    method = "gmres" if "velocity" in kw else "cg"
    # preconditioned CG stops on <r, B r> (cg.hh:62-67), so ask for 1e-12 there
    info, x = _solve(gb, A, u, method, gb.Preconditioner.block_jacobi(A), tol=1e-12 if method == "cg" else 1e-10,
                     restart=10)
    assert info["converged"]
    assert np.linalg.norm(u - prob.apply(x)) <= 2e-10 * np.linalg.norm(u)


@pytest.mark.parametrize("case", ["plain", "diagonal", "block_jacobi", "fp32_bj", "q1", "bsr"])
def test_graph_cg_iterates_equal_host_loop(gb, orc, case):
    """The device-resident CG (scalars on the device, chunks of iterations in a
    CUDA graph) runs the host loop's statements: same iteration count, same
    iterate bit for bit, same residual."""
    prec = gb.F32 if case == "fp32_bj" else gb.F64
    if case == "q1":
        op = gb.Q1Operator((24, 24), diffusion=1.0, mass=1.0)
        f = q1_rhs(24)
    else:
        op = gb.DGOperator((3, 3, 3), 2, mass=0.5, precision=prec)
        if case == "bsr":
            op = op.assemble()
        f = np.random.default_rng(6).uniform(-1, 1, op.size)
    mk = {"plain": lambda: None, "diagonal": lambda: gb.Preconditioner.diagonal(op),
          "q1": lambda: gb.Preconditioner.diagonal(op)}.get(case, lambda: gb.Preconditioner.block_jacobi(op))
    pc = mk()
    tol = 1e-5 if prec == gb.F32 else 1e-10
    f = f.astype(np.float32) if prec == gb.F32 else f
    ih, uh = _solve(gb, op, f, "cg", pc, tol=tol)
    for chunk in (1, 7, 32):
        ig, ug = _solve(gb, op, f, "cg", pc, tol=tol, graph_chunk=chunk)
        assert ig["converged"] and ig["iterations"] == ih["iterations"]
        assert ig["residual"] == ih["residual"]
        assert np.array_equal(ug.view(np.uint8), uh.view(np.uint8))
        assert ig["operator_applies"] >= ig["iterations"] + 1


def test_graph_cg_cap_and_nonfinite(gb, orc):
    op, prob, f = _problem(gb, orc)
    info, _ = _solve(gb, op, f, "cg", max_iterations=3, graph_chunk=8)
    assert info["iterations"] == -3 and not info["converged"]
    g = f.copy()
    g[7] = np.nan
    info, _ = _solve(gb, op, g, "cg", max_iterations=50, graph_chunk=8)
    assert not info["converged"]


def test_fp16_block_jacobi_storage(gb, orc):
    """Scaled FP16 blocks: the apply is the dense inverse to FP16 accuracy, and
    the mixed solve with them still reaches the FP64 tolerance."""
    cells, order = (3, 3, 2), 3
    kw = dict(mass=0.5, velocity=(0.2, 0.0, -0.1))
    op = gb.DGOperator(cells, order, **kw)
    prob = orc.DGProblem(cells, order, **kw)
    pc = gb.Preconditioner.block_jacobi(op, gb.F16)
    assert pc.precision == gb.F32
    f = np.random.default_rng(9).uniform(-1, 1, op.size)
    z = gb.DeviceArray(op.size, gb.F32)
    pc(gb.DeviceArray.from_numpy(f.astype(np.float32)), z)
    binv = np.linalg.inv(prob.block_diagonal())
    ref = np.einsum("cij,cj->ci", binv, f.astype(np.float32).reshape(-1, prob.nloc)).ravel()
    err = relmax(z.numpy(), ref)
    assert 1e-6 < err < 3e-3  # FP16 rounding is visible but small
    cells, order = (4, 4, 4), 3
    op64 = gb.DGOperator(cells, order)
    op32 = gb.DGOperator(cells, order, precision=gb.F32)
    pc16 = gb.Preconditioner.block_jacobi(op64, gb.F16)
    f = np.random.default_rng(10).uniform(-1, 1, op64.size)
    u = gb.DeviceArray(op64.size)
    u.clear()
    info = gb.solve_mixed(op64, op32, pc16, gb.DeviceArray.from_numpy(f), u, tolerance=1e-10, inner_tolerance=1e-3)
    assert info.converged and info.residual <= 1e-10
    prob = orc.DGProblem(cells, order)
    assert np.linalg.norm(f - prob.apply(u.numpy())) <= 1.01e-10 * np.linalg.norm(f)


@pytest.mark.parametrize("outer", ["fgmres", "fcg"])
def test_mixed_flexible_outer_reaches_fp64_tolerance(gb, orc, outer):
    """FP64 FGMRES / FCG with the FP32 inner solve as preconditioner."""
    cells, order = (4, 4, 4), 3
    modes = gb.fourier_modes(3, 64, 0.2, 1.0)
    k64 = gb.project(cells, order, gb.FN_EXP_FOURIER, modes=modes)
    k32 = gb.project(cells, order, gb.FN_EXP_FOURIER, modes=modes, precision=gb.F32)
    op64 = gb.DGOperator(cells, order, kappa=k64)
    op32 = gb.DGOperator(cells, order, precision=gb.F32, kappa=k32)
    pc32 = gb.Preconditioner.block_jacobi(op64, gb.F32)
    f = np.random.default_rng(12).uniform(-1, 1, op64.size)
    u = gb.DeviceArray(op64.size)
    u.clear()
    info = gb.solve_mixed(op64, op32, pc32, gb.DeviceArray.from_numpy(f), u, tolerance=1e-10, inner_tolerance=1e-2,
                          outer=outer, max_outer=200)
    assert info.converged and info.residual <= 1e-10 and info.outer_iterations > 0
    prob = orc.DGProblem(cells, order)
    assert np.linalg.norm(f - prob.apply(u.numpy(), kappa=k64.numpy())) <= 1.01e-10 * np.linalg.norm(f)


@pytest.mark.parametrize("method", ["jacobi", "gauss-seidel", "sor", "ssor"])
@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 0, 1)])
def test_sor_family_matches_natural_order_sweeps(gb, orc, method, periodic):
    """FemPreconditioning jacobi / gauss-seidel / sor / ssor on the assembled
    operator: the level-wavefront GPU sweep equals the oracle's sequential
    natural-order sweep."""
    import smoother_oracle
    cells, order = (3, 2, 4), 1
    kw = dict(mass=0.3, velocity=(0.4, -0.2, 0.3), periodic=periodic)
    op = gb.DGOperator(cells, order, **kw)
    A = op.assemble()
    prob = orc.DGProblem(cells, order, **kw)
    M = np.stack([prob.apply(e) for e in np.eye(prob.ndofs)], axis=1)
    b = np.random.default_rng(13).uniform(-1, 1, prob.ndofs)
    for iterations, relax in ((1, 1.0), (2, 0.7)):
        pc = gb.Preconditioner.sor(A, method, iterations, relax)
        z = gb.DeviceArray(prob.ndofs)
        pc(gb.DeviceArray.from_numpy(b), z)
        ref = smoother_oracle.smoother_apply(M, b, method, iterations, relax)
        assert relmax(z.numpy(), ref) < 1e-12, (iterations, relax)


def test_ssor_preconditioned_cg_converges(gb, orc):
    cells, order = (4, 4, 4), 2
    op = gb.DGOperator(cells, order, mass=0.1)
    A = op.assemble()
    f = np.random.default_rng(14).uniform(-1, 1, op.size)
    info_ssor, x = _solve(gb, A, f, "cg", gb.Preconditioner.sor(A, "ssor"), tol=1e-12)
    info_none, _ = _solve(gb, A, f, "cg", None, tol=1e-12)
    assert info_ssor["converged"] and info_ssor["iterations"] < info_none["iterations"]
    prob = orc.DGProblem(cells, order, mass=0.1)
    assert np.linalg.norm(f - prob.apply(x)) <= 1e-9 * np.linalg.norm(f)


@pytest.mark.parametrize("outer", ["refinement", "fgmres"])
def test_mixed_stops_at_the_rounding_floor(gb, orc, outer):
    """A tolerance below the FP64 rounding floor of ||f - A u|| / ||f||: the
    mixed solve reports stagnation instead of spending its whole budget."""
    cells, order = (4, 4, 4), 2
    op64 = gb.DGOperator(cells, order)
    op32 = gb.DGOperator(cells, order, precision=gb.F32)
    pc32 = gb.Preconditioner.block_jacobi(op64, gb.F32)
    f = np.random.default_rng(15).uniform(-1, 1, op64.size)
    u = gb.DeviceArray(op64.size)
    u.clear()
    info = gb.solve_mixed(op64, op32, pc32, gb.DeviceArray.from_numpy(f), u, tolerance=1e-19, max_outer=200,
                          inner_tolerance=1e-3, outer=outer)
    assert not info.converged and info.stagnated and info.outer_iterations < 60
    assert info.residual < 1e-13


@pytest.mark.parametrize("cells,order", [((32, 32, 32), 1), ((28, 27, 28), 4)])
def test_scaled_block_jacobi_many_tiles(gb, orc, cells, order):
    """Grids with more quads of tiles than the persistent grid has CTAs, so
    that a CTA runs several quads, double-buffers its groups' residuals and
    meets type changes (and empty padding tiles) inside its range: against
    the oracle's kappa = 1 blocks (order 1) and against block Jacobi of the
    same operator (constant kappa)."""
    ncell = int(np.prod(cells))
    nloc = (order + 1) ** 3
    rng = np.random.default_rng(ncell)
    r = rng.uniform(-1, 1, ncell * nloc).astype(np.float32)
    if order == 1:
        kc = rng.uniform(0.5, 2.0, ncell).astype(np.float32)
        op = gb.DGOperator(cells, order, precision=gb.F32, kappa_cell=gb.DeviceArray.from_numpy(kc, gb.F32))
        z = gb.DeviceArray(ncell * nloc, gb.F32)
        gb.Preconditioner.scaled_block_jacobi(op)(gb.DeviceArray.from_numpy(r, gb.F32), z)
        hinv = np.linalg.inv(orc.DGProblem(cells, order).block_diagonal(nthreads=8))
        ref = np.einsum("cij,cj->ci", hinv, r.astype(np.float64).reshape(-1, nloc)) / kc[:, None].astype(np.float64)
        assert relmax(z.numpy(), ref.ravel()) < 2e-5
    const = gb.DGOperator(cells, order, precision=gb.F32,
                          kappa_cell=gb.DeviceArray.from_numpy(np.full(ncell, 0.8, np.float32), gb.F32))
    z1, z2 = gb.DeviceArray(ncell * nloc, gb.F32), gb.DeviceArray(ncell * nloc, gb.F32)
    gb.Preconditioner.scaled_block_jacobi(const)(gb.DeviceArray.from_numpy(r, gb.F32), z1)
    gb.Preconditioner.block_jacobi(const)(gb.DeviceArray.from_numpy(r, gb.F32), z2)
    # FP32 blocks of two assemblies: their rounding grows with the Q4 blocks'
    # condition; a tile or index mix-up would be O(1)
    assert relmax(z1.numpy(), z2.numpy()) < (5e-5 if order == 1 else 1e-3)


@pytest.mark.parametrize("cells,periodic", [((4, 3, 5), (0, 0, 0)), ((4, 2, 3), (1, 0, 0)), ((1, 4, 3), (0, 0, 1))])
def test_scaled_block_jacobi_for_cellwise_kappa(gb, orc, cells, periodic):
    """z_c = H_t^-1 r_c / kappa_c with H_t the kappa = 1 diagonal block of the
    cell's boundary type: against the oracle's blocks of the kappa = 1
    operator on the same grid; equal to block Jacobi when kappa is constant."""
    order = 2
    kw = dict(periodic=periodic)
    ncell = int(np.prod(cells))
    rng = np.random.default_rng(int(np.prod(cells)))
    kc = rng.uniform(0.5, 2.0, ncell).astype(np.float32)
    op = gb.DGOperator(cells, order, precision=gb.F32, kappa_cell=gb.DeviceArray.from_numpy(kc, gb.F32), **kw)
    pc = gb.Preconditioner.scaled_block_jacobi(op)
    prob = orc.DGProblem(cells, order, **kw)
    r = rng.uniform(-1, 1, prob.ndofs).astype(np.float32)
    z = gb.DeviceArray(prob.ndofs, gb.F32)
    pc(gb.DeviceArray.from_numpy(r, gb.F32), z)
    hinv = np.linalg.inv(prob.block_diagonal())  # kappa = 1
    ref = np.einsum("cij,cj->ci", hinv, r.astype(np.float64).reshape(-1, prob.nloc)) / kc[:, None].astype(np.float64)
    assert relmax(z.numpy(), ref.ravel()) < 2e-5
    # constant kappa: the same as block Jacobi of the operator itself
    const = gb.DGOperator(cells, order, precision=gb.F32,
                          kappa_cell=gb.DeviceArray.from_numpy(np.full(ncell, 1.7, np.float32), gb.F32), **kw)
    z1, z2 = gb.DeviceArray(prob.ndofs, gb.F32), gb.DeviceArray(prob.ndofs, gb.F32)
    gb.Preconditioner.scaled_block_jacobi(const)(gb.DeviceArray.from_numpy(r, gb.F32), z1)
    gb.Preconditioner.block_jacobi(const)(gb.DeviceArray.from_numpy(r, gb.F32), z2)
    assert relmax(z1.numpy(), z2.numpy()) < 2e-5


def test_cg_true_residual_criterion(gb, orc):
    """GBFEM_TOL_RELATIVE_RESIDUAL: block-Jacobi CG stops on the recursively
    updated ||f - A u|| <= eps ||f|| (the reference's CG stops on <r, B r>);
    the iterates are those of the reference's loop, so both criteria give
    bitwise the same u after the same number of iterations."""
    cells, order = (4, 4, 4), 2
    nloc, ncell = (order + 1) ** 3, 64
    rng = np.random.default_rng(5)
    kappa = np.zeros(ncell * nloc)
    kappa[::nloc] = np.exp(rng.uniform(-1.5, 1.5, ncell))  # positive cell means
    kappa += 0.02 * rng.uniform(-1, 1, ncell * nloc)       # small variation inside the cells
    op = gb.DGOperator(cells, order, kappa=gb.DeviceArray.from_numpy(kappa))
    pc = gb.Preconditioner.block_jacobi(op)
    f = np.random.default_rng(9).uniform(-1, 1, op.size)
    info, u = _solve(gb, op, f, "cg", pc, tol=1e-10, error_measure=gb.RELATIVE_RESIDUAL)
    assert info["converged"]
    au = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), au)
    true_rel = np.linalg.norm(f - au.numpy()) / np.linalg.norm(f)
    assert true_rel <= 1e-9  # the recursive residual may drift from f - A u by rounding
    assert info["residual"] <= 1e-10 * np.linalg.norm(f)
    i0, _ = _solve(gb, op, f, "cg", pc, tol=1e-10, error_measure=gb.RELATIVE)
    assert i0["converged"] and 0 < i0["iterations"] <= info["iterations"]
    k = max(1, info["iterations"] // 2)
    i1, u1 = _solve(gb, op, f, "cg", pc, tol=1e-30, error_measure=gb.RELATIVE_RESIDUAL, max_iterations=k)
    i2, u2 = _solve(gb, op, f, "cg", pc, tol=1e-30, error_measure=gb.RELATIVE, max_iterations=k)
    assert i1["iterations"] == i2["iterations"] == -k
    assert np.array_equal(u1.view(np.uint64), u2.view(np.uint64))


def test_unknown_error_measure_is_rejected(gb, orc):
    op, prob, f = _problem(gb, orc)
    with pytest.raises(gb.GbfemError):
        _solve(gb, op, f, "cg", error_measure=7)


@pytest.mark.parametrize("order", [3, 4])
@pytest.mark.parametrize("cells,periodic", [((5, 4, 3), (0, 0, 0)), ((9, 7, 6), (1, 0, 0)), ((20, 18, 16), (0, 1, 1)),
                                            ((40, 36, 32), (0, 0, 1))])
def test_scaled_block_jacobi_tensor_cores(gb, orc, order, cells, periodic):
    """The tile products on the tcgen05 tensor cores (TF32 with the 3xTF32
    split) against the oracle's kappa = 1 blocks and against the FP32-FMA
    engine; type changes per CTA, and on the largest grid several full tiles
    per CTA through the software pipeline (720 tiles of 64 cells at Q3,
    1440 of 32 at Q4); the kernel's bounded waits all completed (status 0);
    two applies in a row give bitwise the same result."""
    ncell = int(np.prod(cells))
    nloc = (order + 1) ** 3
    rng = np.random.default_rng(ncell + order)
    kc = rng.uniform(0.5, 2.0, ncell).astype(np.float32)
    op = gb.DGOperator(cells, order, precision=gb.F32, periodic=periodic,
                       kappa_cell=gb.DeviceArray.from_numpy(kc, gb.F32))
    r = gb.DeviceArray.from_numpy(rng.uniform(-1, 1, ncell * nloc).astype(np.float32), gb.F32)
    out = {}
    for engine in ("tensor", "fma"):
        pc = gb.Preconditioner.scaled_block_jacobi(op, engine=engine)
        z = gb.DeviceArray(ncell * nloc, gb.F32)
        pc(r, z)
        out[engine] = z.numpy()
        if engine == "tensor":
            z2 = gb.DeviceArray(ncell * nloc, gb.F32)
            pc(r, z2)
            assert np.array_equal(out[engine].view(np.uint32), z2.numpy().view(np.uint32))
            assert pc.status() == 0
    assert relmax(out["tensor"], out["fma"]) < 2e-5
    if ncell <= 200:
        prob = orc.DGProblem(cells, order, periodic=periodic)
        hinv = np.linalg.inv(prob.block_diagonal())  # kappa = 1
        ref = np.einsum("cij,cj->ci", hinv, r.numpy().astype(np.float64).reshape(-1, nloc))
        ref /= kc[:, None].astype(np.float64)
        assert relmax(out["tensor"], ref.ravel()) < 2e-5


def test_scaled_block_jacobi_rejects_unknown_engine(gb):
    op = gb.DGOperator((2, 2, 2), 3, precision=gb.F32,
                       kappa_cell=gb.DeviceArray.from_numpy(np.ones(8, np.float32), gb.F32))
    with pytest.raises((gb.GbfemError, KeyError)):
        gb.Preconditioner.scaled_block_jacobi(op, engine="nope")
