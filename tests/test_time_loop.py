"""The explicit time loop around the RK3 step: TimeProvider semantics
(solver/timeprovider.hh), the operator's time-step estimate, and VTK output
(io/file/vtkio.hh counterpart)."""
import os

import numpy as np
import pytest

from conftest import relmax


# ---------------------------------------------------------------- CPU tests --
def _tp_cls():
    import gbfem
    return gbfem.TimeProvider


def test_time_provider_step_is_cfl_times_estimate_capped_by_upper_bound():
    tp = _tp_cls()(start_time=1.0, cfl=0.25)
    tp.provideTimeStepEstimate(0.4)
    tp.provideTimeStepEstimate(0.8)  # the minimum counts
    tp.init()
    assert tp.deltaT() == 0.25 * 0.4 and tp.time() == 1.0 and tp.timeStep() == 0
    tp.provideTimeStepEstimate(1.0)
    tp.provideTimeStepUpperBound(0.05)
    tp.next()
    assert tp.time() == 1.0 + 0.1 and tp.timeStep() == 1
    assert tp.deltaT() == 0.05
    # the estimate was reset by next(): a step without a new estimate is an error
    with pytest.raises(RuntimeError):
        tp.next()
    # an explicit step size bypasses the estimate (times the factor)
    tp.next(0.2)
    assert abs(tp.time() - 1.15) < 1e-15 and tp.deltaT() == 0.25 * 0.2


def test_time_provider_invalid_step_does_not_advance():
    tp = _tp_cls()(cfl=1.0)
    tp.init(0.5)
    tp.invalidateTimeStep()
    assert not tp.timeStepValid()
    with pytest.raises(RuntimeError):
        tp.deltaT()
    tp.next(0.5)
    assert tp.time() == 0.0 and tp.timeStepValid()
    tp.next(0.0)  # dt = 0 is not a valid step
    assert not tp.timeStepValid()


def test_time_provider_update_step_keeps_dt_between_updates():
    tp = _tp_cls()(cfl=1.0, update_step=3)
    tp.init(0.1)
    dts = []
    for k in range(6):
        dts.append(tp.deltaT())
        tp.provideTimeStepEstimate(0.1 * (k + 2))
        tp.next()
    # dt is refixed every third call of initTimeStep (counter starts full)
    assert dts[0] == 0.1 and dts[1] == 0.1 and dts[2] == 0.1 and dts[3] == pytest.approx(0.4)


def test_vtk_writer_reproduces_a_trilinear_function():
    import vtkio
    cells, order = (3, 2, 4), 2
    n = order + 1
    lower, upper = (0.0, -1.0, 0.5), (1.5, 1.0, 1.5)
    h = [(upper[k] - lower[k]) / cells[k] for k in range(3)]
    # f(x,y,z) = 1 + 2x - y + 3z + xy z: exact in Q2, coefficients by Gauss projection
    g, w = np.polynomial.legendre.leggauss(4)
    g, w = 0.5 * (g + 1), 0.5 * w
    L = vtkio.legendre_table(order, g)
    f = lambda x, y, z: 1 + 2 * x - y + 3 * z + x * y * z
    coeffs = np.zeros(int(np.prod(cells)) * n ** 3)
    for cz in range(cells[2]):
        for cy in range(cells[1]):
            for cx in range(cells[0]):
                X = lower[0] + (cx + g) * h[0]
                Y = lower[1] + (cy + g) * h[1]
                Z = lower[2] + (cz + g) * h[2]
                F = f(X[:, None, None], Y[None, :, None], Z[None, None, :])
                c = np.einsum("abc,a,b,c,ai,bj,ck->ijk", F, w, w, w, L, L, L)
                cell = cx + cells[0] * (cy + cells[1] * cz)
                coeffs[cell * n ** 3:(cell + 1) * n ** 3] = c.ravel()
    for level in (0, 1, 2):
        S = 2 ** level
        path = vtkio.write_vti(os.path.join(os.environ.get("TMPDIR", "/tmp"), "gbfem_vtk_test_%d" % level),
                               cells, order, {"u": coeffs}, lower, upper, level)
        data = vtkio.read_vti_cell_data(path)["u"]
        assert data.shape == (cells[2] * S, cells[1] * S, cells[0] * S)
        zc = lower[2] + (np.arange(cells[2] * S) + 0.5) * h[2] / S
        yc = lower[1] + (np.arange(cells[1] * S) + 0.5) * h[1] / S
        xc = lower[0] + (np.arange(cells[0] * S) + 0.5) * h[0] / S
        ref = f(xc[None, None, :], yc[None, :, None], zc[:, None, None])
        assert relmax(data, ref) < 1e-13
        os.remove(path)


# ---------------------------------------------------------------- GPU tests --
@pytest.mark.gpu
def test_time_step_estimate_bounds_the_spectral_radius(gb, orc):
    """2/rho from the device power method: rho never exceeds the true spectral
    radius of M^{-1}A (the SIPG operator is symmetric) and gets within 2 %."""
    cells, order = (2, 2, 3), 1
    op = gb.DGOperator(cells, order, mass=0.2)
    prob = orc.DGProblem(cells, order, mass=0.2)
    A = np.stack([prob.apply(e) for e in np.eye(prob.ndofs)], axis=1)
    vol = 1.0 / np.prod(cells)
    rho = np.max(np.abs(np.linalg.eigvalsh(0.5 * (A + A.T)))) / vol
    est, ub = gb.time_step_estimate(op, power_iterations=400, seed=3)
    assert est == np.inf  # no advection
    rho_gpu = 2.0 / ub
    assert rho_gpu <= rho * (1 + 1e-9) and rho_gpu >= 0.98 * rho
    opb = gb.DGOperator(cells, order, velocity=(1.0, 2.0, -2.0))
    est, _ = gb.time_step_estimate(opb, power_iterations=0)
    assert est == pytest.approx((1.0 / 3) / (3.0 * 3))


@pytest.mark.gpu
def test_time_loop_with_time_provider_matches_fixed_step_loop(gb):
    cells, order = (6, 5, 4), 2
    kw = dict(diffusion=1e-2, velocity=(1.0, 0.5, 0.25), periodic=(1, 1, 1), weak_dirichlet=False)
    op = gb.DGOperator(cells, order, **kw)
    u0 = gb.project(cells, order, gb.FN_GAUSSIAN, params=(0.5, 0.5, 0.5, 0.2))
    tp = gb.TimeProvider(cfl=0.2)
    ode = gb.ExplicitRungeKuttaSolver(op, tp)
    u = gb.DeviceArray.from_numpy(u0.numpy())
    ode.initialize(u)
    tp.init()
    dts = []
    end = 0.02
    while tp.time() < end:
        dts.append(tp.deltaT())
        ode.solve(u)
        tp.next()
    assert tp.time() >= end and tp.timeStep() == len(dts)
    assert all(dt == dts[0] for dt in dts)
    est, ub = gb.time_step_estimate(op)
    assert dts[0] == min(0.2 * est, ub)
    # the same steps through the bare RK3 step give the same bits
    v = gb.DeviceArray.from_numpy(u0.numpy())
    rk = gb.RK3(op)
    for dt in dts:
        rk.step(v, dt)
    assert np.array_equal(u.numpy().view(np.uint64), v.numpy().view(np.uint64))
    # mass is conserved by the periodic advection-diffusion operator
    m0 = u0.numpy()[::op.nloc].sum()
    assert abs(u.numpy()[::op.nloc].sum() - m0) <= 1e-12 * abs(m0)
