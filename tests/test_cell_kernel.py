"""The one-kernel FP32 closed form (dg_cell_kernel: a brick of 8 x 4 x 4 cells
per CTA, fluxes exchanged in shared memory, halo traces recomputed) against
the oracle and against the two-kernel form (GBFEM_ALGO_TRACE_PASS), on grids
that fill bricks exactly, leave partial bricks in every direction, span many
bricks, and wrap periodically across brick boundaries."""
import numpy as np
import pytest

from conftest import relmax

pytestmark = pytest.mark.gpu

TOL32 = 2e-5  # the FP32 bar of the parity tests

SHAPES = [(3, 4, 2), (8, 4, 4), (9, 5, 6), (17, 9, 5)]
FORMS = {
    "dirichlet": dict(),
    "periodic_mixed": dict(periodic=(1, 0, 1), mass=0.7),
    "advection": dict(diffusion=0.05, velocity=(1.0, -0.5, 0.25), periodic=(0, 1, 0), mass=0.3),
    "advection_only": dict(diffusion=0.0, velocity=(-0.4, 0.3, 1.0), periodic=(1, 1, 0), weak_dirichlet=False),
    "no_penalty": dict(penalty=0.0, mass=0.2, lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5)),
}


def _run(gb, cells, order, algo, u, kappa_cell=None, **kw):
    op = gb.DGOperator(cells, order, precision=gb.F32, algorithm=algo, kappa_cell=kappa_cell, **kw)
    w = gb.DeviceArray(u.n, gb.F32)
    op(u, w)
    return w.numpy()


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("cells", SHAPES)
@pytest.mark.parametrize("form", sorted(FORMS))
def test_cell_kernel_matches_oracle_and_two_kernel_form(gb, orc, order, cells, form):
    kw = FORMS[form]
    prob = orc.DGProblem(cells, order, **kw)
    seed = 1000 * order + 100 * cells[0] + 10 * cells[1] + cells[2] + 7 * sorted(FORMS).index(form)
    u = np.random.default_rng(seed).uniform(-1, 1, prob.ndofs)
    u = u.astype(np.float32)
    du = gb.DeviceArray.from_numpy(u)
    one = _run(gb, cells, order, gb.ALGO_AUTO, du, **kw)
    two = _run(gb, cells, order, gb.ALGO_TRACE_PASS, du, **kw)
    ref = prob.apply(u.astype(np.float64))
    assert relmax(one, ref) < TOL32
    assert relmax(one, two) < TOL32
    again = _run(gb, cells, order, gb.ALGO_AUTO, du, **kw)
    assert np.array_equal(one.view(np.uint32), again.view(np.uint32))


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("cells", [(9, 5, 6), (16, 8, 12)])
@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 1)])
def test_cell_kernel_cellwise_kappa(gb, orc, order, cells, periodic):
    """A kappa per cell (the mixed solve's inner operator): the oracle sees
    it as a DG field holding only the cell means."""
    prob = orc.DGProblem(cells, order, periodic=periodic, mass=0.25 if periodic[0] else 0.0)
    rng = np.random.default_rng(order + 7 * periodic[0])
    kc = np.exp(rng.uniform(-2, 2, prob.ncells))
    kfield = np.zeros(prob.ndofs)
    kfield[::prob.nloc] = kc
    u = rng.uniform(-1, 1, prob.ndofs).astype(np.float32)
    du = gb.DeviceArray.from_numpy(u)
    dk = gb.DeviceArray.from_numpy(kc.astype(np.float32))
    kw = dict(periodic=periodic, mass=0.25 if periodic[0] else 0.0)
    one = _run(gb, cells, order, gb.ALGO_AUTO, du, kappa_cell=dk, **kw)
    two = _run(gb, cells, order, gb.ALGO_TRACE_PASS, du, kappa_cell=dk, **kw)
    ref = prob.apply(u.astype(np.float64), kappa=kfield)
    assert relmax(one, ref) < TOL32
    assert relmax(one, two) < TOL32


def test_fp64_trace_pass_algorithm_is_the_default_closed_form(gb, orc):
    """GBFEM_ALGO_TRACE_PASS in FP64 is the same computation as the default."""
    cells = (5, 4, 3)
    prob = orc.DGProblem(cells, 3)
    u = gb.DeviceArray.from_numpy(np.random.default_rng(2).uniform(-1, 1, prob.ndofs))
    outs = []
    for algo in (gb.ALGO_AUTO, gb.ALGO_TRACE_PASS):
        op = gb.DGOperator(cells, 3, algorithm=algo)
        w = gb.DeviceArray(prob.ndofs)
        op(u, w)
        outs.append(w.numpy())
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))


def test_unknown_algorithm_is_rejected(gb):
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((2, 2, 2), 1, algorithm=3)
