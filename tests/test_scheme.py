"""The dune.fem-shaped Python front end (gbfem.Scheme, Space, the zero-copy
device view): scheme(u, w), scheme.solve(target, rightHandSide=...) with
the fem.solver parameter keys, against the operator, the Krylov and Newton
inverse operators and the oracle."""
import numpy as np
import pytest

from conftest import relmax


@pytest.mark.gpu
def test_linear_scheme_call_and_solve(gb, orc):
    cells, order = (4, 3, 3), 2
    op = gb.DGOperator(cells, order, mass=0.3)
    prm = {"linear.method": "cg", "linear.tolerance": 1e-11, "linear.errormeasure": "relative",
           "linear.preconditioning.method": "blockjacobi"}
    scheme = gb.Scheme(op, parameters=prm)
    prob = orc.DGProblem(cells, order, mass=0.3)
    f = np.random.default_rng(3).uniform(-1, 1, prob.ndofs)
    # scheme(u, w) is the operator
    u = gb.DeviceArray.from_numpy(f)
    w1, w2 = gb.DeviceArray(op.size), gb.DeviceArray(op.size)
    scheme(u, w1)
    op(u, w2)
    assert np.array_equal(w1.numpy().view(np.uint64), w2.numpy().view(np.uint64))
    # solve: the Krylov inverse operator with the same parameters, same iterates
    x = scheme.space.zero
    info = scheme.solve(target=x, rightHandSide=gb.DeviceArray.from_numpy(f))
    assert info["converged"] and info["linear_iterations"] > 0 and info["iterations"] == 0
    inv = gb.KrylovInverseOperator("cg", tolerance=1e-11, error_measure=gb.RELATIVE)
    inv.bind(op, gb.Preconditioner.block_jacobi(op))
    y = gb.DeviceArray(op.size)
    y.clear()
    inv(gb.DeviceArray.from_numpy(f), y)
    assert np.array_equal(x.numpy().view(np.uint64), y.numpy().view(np.uint64))
    # and the solution solves the oracle's system
    assert relmax(prob.apply(x.numpy()), f) < 1e-8
    # the deprecated newton. prefix and other preconditioners
    for pre in ("none", "jacobi", "ssor"):
        s2 = gb.Scheme(op, parameters={"newton.linear.tolerance": 1e-10, "newton.linear.errormeasure": "relative",
                                       "newton.linear.preconditioning.method": pre})
        z = s2.space.zero
        assert s2.solve(z, rightHandSide=gb.DeviceArray.from_numpy(f))["converged"]
        assert relmax(z.numpy(), x.numpy()) < 1e-7


@pytest.mark.gpu
def test_nonlinear_scheme_solve_is_newton(gb, orc):
    """-lap u = 5 e^u: scheme.solve runs the Newton inverse operator."""
    cells, order, reaction = (3, 3, 3), 2, (0.0, 0.0, -5.0)
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction)
    scheme = gb.Scheme(op, parameters={"nonlinear.tolerance": 1e-10, "linear.tolerance": 1e-13,
                                       "linear.preconditioning.method": "blockjacobi"})
    w = scheme.space.zero
    info = scheme.solve(target=w)
    assert info["converged"] and info["iterations"] >= 2 and info["linear_iterations"] > 0
    newton = gb.NewtonInverseOperator(tolerance=1e-10, preconditioner=gb.PC_BLOCK_JACOBI, linear_tolerance=1e-13)
    newton.bind(op)
    v = gb.DeviceArray(op.size)
    v.clear()
    rhs = gb.DeviceArray(op.size)
    rhs.clear()
    newton(rhs, v)
    assert info["iterations"] == newton.info()["iterations"]
    assert relmax(w.numpy(), v.numpy()) < 1e-12
    r = gb.DeviceArray(op.size)
    scheme(w, r)
    assert np.max(np.abs(r.numpy())) < 1e-9


@pytest.mark.gpu
def test_device_array_zero_copy_view(gb):
    torch = pytest.importorskip("torch")
    a = gb.DeviceArray.from_numpy(np.arange(10, dtype=np.float64))
    t = a.as_tensor()
    assert t.data_ptr() == a.ptr.value and t.dtype == torch.float64 and t.is_cuda
    t.mul_(2.0)  # through the view
    assert np.array_equal(a.numpy(), 2.0 * np.arange(10))
    b = gb.DeviceArray(4, gb.F32)
    assert b.__cuda_array_interface__["typestr"] == "<f4"


def test_scheme_rejects_unknown_preconditioning(gb):
    class _Op:
        size, precision = 8, 0

    with pytest.raises(gb.GbfemError):
        gb.Scheme(_Op(), parameters={"linear.preconditioning.method": "ilu-42"})
