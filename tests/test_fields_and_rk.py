"""Projection of the benchmark coefficient fields and SSP-RK3 stepping on the
GPU, against the oracle."""
import numpy as np
import pytest

from conftest import relmax

pytestmark = pytest.mark.gpu


def test_fourier_modes_statistics(gb):
    m = gb.fourier_modes(7, 4096, corr_length=0.1, stddev=1.0)
    # 2 pi w has std 1/0.1 = 10 per component; amplitudes give variance 1
    assert abs(np.std(2 * np.pi * m[:, :3]) - 10.0) < 0.3
    assert abs(np.sum(m[:, 4] ** 2) / 2 - 1.0) < 1e-12
    assert np.all((m[:, 3] >= 0) & (m[:, 3] < 2 * np.pi))
    assert np.array_equal(m, gb.fourier_modes(7, 4096))


@pytest.mark.parametrize("order", [1, 3, 4])
def test_projection_of_log_gaussian_kappa(gb, orc, order):
    cells = (3, 2, 4)
    modes = gb.fourier_modes(20261203, 256)
    k = gb.project(cells, order, gb.FN_EXP_FOURIER, modes=modes).numpy()
    ref = orc.DGProblem(cells, order).project(0, modes=modes)
    assert relmax(k, ref) < 1e-12


def test_projection_of_bump_and_load_vector(gb, orc):
    cells = (4, 4, 4)
    prob = orc.DGProblem(cells, 2)
    bump = (0.5, 0.5, 0.5, 0.1)
    assert relmax(gb.project(cells, 2, gb.FN_GAUSSIAN, params=bump).numpy(), prob.project(1, bump)) < 1e-12
    one = gb.project(cells, 2, gb.FN_CONSTANT, params=(1.0,), scale_by_volume=True).numpy()
    ref = np.zeros(prob.ndofs)
    ref[::prob.nloc] = 1.0 / 64  # int_K 1 * phi_0 = |K|
    assert relmax(one, ref) < 1e-14


def test_variable_kappa_operator_with_projected_field(gb, orc):
    cells, order = (3, 3, 2), 3
    modes = gb.fourier_modes(1, 256)
    kd = gb.project(cells, order, gb.FN_EXP_FOURIER, modes=modes)
    op = gb.DGOperator(cells, order, kappa=kd)
    prob = orc.DGProblem(cells, order)
    u = np.random.default_rng(0).uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u, kappa=kd.numpy())) < 1e-12


def _advdiff(gb, orc, cells, order, precision=0):
    kw = dict(diffusion=1e-3, velocity=(1.0, 0.5, 0.25), periodic=(1, 1, 1), weak_dirichlet=False)
    op = gb.DGOperator(cells, order, precision=precision, **kw)
    prob = orc.DGProblem(cells, order, **kw)
    return op, prob


def test_rk3_steps_match_oracle_fp64_and_fp32(gb, orc):
    cells, order = (4, 4, 4), 2
    op, prob = _advdiff(gb, orc, cells, order)
    u0 = gb.project(cells, order, gb.FN_GAUSSIAN, params=(0.5, 0.5, 0.5, 0.25)).numpy()
    dt = 0.2 * 0.25 / (np.sqrt(1 + 0.25 + 0.0625) * (2 * order + 1))
    ud = gb.DeviceArray.from_numpy(u0)
    rk = gb.RK3(op)
    ref = u0.copy()
    for _ in range(3):
        rk.step(ud, dt)
        ref = prob.rk3_step(ref, dt)
    assert relmax(ud.numpy(), ref) < 1e-12
    op32, _ = _advdiff(gb, orc, cells, order, precision=gb.F32)
    u32 = gb.DeviceArray.from_numpy(u0.astype(np.float32))
    rk32 = gb.RK3(op32)
    for _ in range(3):
        rk32.step(u32, dt)
    assert relmax(u32.numpy(), ref) < 1e-5


def test_rk3_conserves_mass_on_periodic_grid(gb, orc):
    """Upwind DG + SIPG on a periodic grid conserves int u exactly (a
    size-independent property checked at 32^3)."""
    cells, order = (32, 32, 32), 2
    op, _ = _advdiff(gb, orc, cells, order)
    u = gb.project(cells, order, gb.FN_GAUSSIAN, params=(0.5, 0.5, 0.5, 0.1))
    nl = (order + 1) ** 3
    m0 = u.numpy()[::nl].sum()
    rk = gb.RK3(op)
    h = 1.0 / 32
    dt = 0.2 * h / (np.sqrt(1.3125) * (2 * order + 1))
    for _ in range(10):
        rk.step(u, dt)
    x = u.numpy()
    assert np.all(np.isfinite(x))
    assert abs(x[::nl].sum() - m0) < 1e-12 * abs(m0)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_hierarchical_permute_round_trip(gb, order):
    nloc = (order + 1) ** 3
    ncells = 37
    u = np.random.default_rng(order).uniform(-1, 1, ncells * nloc)
    perm = gb.hierarchical_permutation(order)
    d = gb.DeviceArray.from_numpy(u)
    h = gb.to_hierarchical(d, order)
    assert np.array_equal(h.numpy(), u.reshape(ncells, nloc)[:, perm].ravel())
    back = gb.from_hierarchical(h, order)
    assert np.array_equal(back.numpy(), u)
    h32 = gb.to_hierarchical(gb.DeviceArray.from_numpy(u.astype(np.float32)), order)
    assert np.array_equal(h32.numpy(), u.astype(np.float32).reshape(ncells, nloc)[:, perm].ravel())
