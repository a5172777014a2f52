"""Parity of the GPU DG operator apply (through the C-ABI) with the CPU oracle.

The bar: FP64 within 1e-12 relative in the max norm; FP32 within 2e-5.
"""
import numpy as np
import pytest

from conftest import relmax

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


def _pair(gb, orc, cells, order, q=0, precision=0, kappa=None, **kw):
    op = gb.DGOperator(cells, order, quad_points=q, precision=precision,
                       kappa=None if kappa is None else gb.DeviceArray.from_numpy(kappa, precision), **kw)
    prob = orc.DGProblem(cells, order, quad_points=q, **kw)
    return op, prob


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("qoff", [1, 2])
@pytest.mark.parametrize("algorithm", [0, 1])
def test_sipg_apply_fp64(gb, orc, order, qoff, algorithm):
    """algorithm 0: constant-coefficient closed form; 1: Gauss-point quadrature."""
    cells = (3, 4, 2)
    rng = np.random.default_rng(100 + order)
    op = gb.DGOperator(cells, order, quad_points=order + qoff, algorithm=algorithm)
    prob = orc.DGProblem(cells, order, quad_points=order + qoff)
    u = rng.uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u)) < TOL64


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_full_form_fp64(gb, orc, order):
    """Diffusion + variable kappa + upwind advection + mass, periodic in y,
    anisotropic cells."""
    cells = (3, 2, 4)
    kw = dict(diffusion=0.7, mass=1.3, velocity=(1.0, -0.5, 0.25), periodic=(0, 1, 0),
              lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5))
    rng = np.random.default_rng(7 + order)
    nloc = (order + 1) ** 3
    ncell = int(np.prod(cells))
    kappa = np.zeros(ncell * nloc)
    kappa[::nloc] = rng.uniform(0.5, 2.0, ncell)  # positive mean per cell
    kappa += 0.05 * rng.uniform(-1, 1, ncell * nloc)
    op, prob = _pair(gb, orc, cells, order, kappa=kappa, **kw)
    u = rng.uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u, kappa=kappa)) < TOL64


@pytest.mark.parametrize("algorithm", [0, 1])
def test_periodic_advection_only(gb, orc, algorithm):
    cells = (4, 3, 2)
    kw = dict(diffusion=0.0, velocity=(1.0, 0.5, 0.25), periodic=(1, 1, 1), weak_dirichlet=False)
    op = gb.DGOperator(cells, 2, algorithm=algorithm, **kw)
    prob = orc.DGProblem(cells, 2, **kw)
    u = np.random.default_rng(3).uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u)) < TOL64


@pytest.mark.parametrize("algorithm", [0, 1])
@pytest.mark.parametrize("case", ["no_penalty", "advection_boundaries", "tiny_diffusion"])
def test_flux_constant_edge_cases(gb, orc, algorithm, case):
    """The closed form folds A1 = |F| eps beta / h into its expansion tables and
    keeps P = v - sigma (A2 / A1) dv as its second trace; with A1 = 0 (no
    penalty, or no diffusion) it uses 1 in its place.  Each case against the
    oracle: penalty 0 with diffusion, pure advection with inflow and outflow
    boundary faces, and a diffusion small against the advection."""
    cells = (3, 4, 2)
    kw = {"no_penalty": dict(diffusion=0.8, penalty=0.0, mass=0.4),
          "advection_boundaries": dict(diffusion=0.0, velocity=(1.0, -0.5, 0.25), periodic=(0, 0, 1)),
          "tiny_diffusion": dict(diffusion=1e-6, velocity=(-0.3, 0.5, 1.0))}[case]
    op = gb.DGOperator(cells, 3, algorithm=algorithm, **kw)
    prob = orc.DGProblem(cells, 3, **kw)
    u = np.random.default_rng(11).uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u)) < TOL64


@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("algorithm", [0, 1])
def test_sipg_apply_fp32(gb, orc, order, algorithm):
    cells = (3, 3, 3)
    op = gb.DGOperator(cells, order, precision=gb.F32, algorithm=algorithm)
    prob = orc.DGProblem(cells, order)
    u = np.random.default_rng(5).uniform(-1, 1, prob.ndofs).astype(np.float32)
    w = gb.DeviceArray(prob.ndofs, gb.F32)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u.astype(np.float64))) < TOL32


def test_apply_is_deterministic_and_host_path_matches(gb, orc):
    cells = (5, 4, 3)
    op, prob = _pair(gb, orc, cells, 3)
    u = np.random.default_rng(11).uniform(-1, 1, prob.ndofs)
    du = gb.DeviceArray.from_numpy(u)
    w1 = gb.DeviceArray(prob.ndofs)
    w2 = gb.DeviceArray(prob.ndofs)
    op(du, w1)
    op(du, w2)
    a, b = w1.numpy(), w2.numpy()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    wh = np.empty(prob.ndofs)
    op.apply_host(u, wh)
    assert np.array_equal(wh.view(np.uint64), a.view(np.uint64))


def test_linearity_and_symmetry_at_size(gb):
    """Size-independent properties at a larger grid: A(au+bv) = aAu + bAv and
    <Au, v> = <u, Av> (SIPG is symmetric)."""
    cells = (16, 16, 16)
    op = gb.DGOperator(cells, 3)
    n = op.size
    rng = np.random.default_rng(1)
    u, v = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    Au, Av, Auv = (gb.DeviceArray(n) for _ in range(3))
    op(gb.DeviceArray.from_numpy(u), Au)
    op(gb.DeviceArray.from_numpy(v), Av)
    op(gb.DeviceArray.from_numpy(2.0 * u - 0.5 * v), Auv)
    au, av = Au.numpy(), Av.numpy()
    assert relmax(Auv.numpy(), 2.0 * au - 0.5 * av) < 1e-13
    s1, s2 = float(au @ v), float(u @ av)
    assert abs(s1 - s2) <= 1e-12 * (abs(s1) + abs(s2))


@pytest.mark.parametrize("order", [1, 3])
def test_block_diagonal_and_diagonal(gb, orc, order):
    cells = (3, 2, 2)
    kw = dict(mass=0.5, velocity=(0.3, 0.0, -0.2))
    op, prob = _pair(gb, orc, cells, order, **kw)
    nloc = prob.nloc
    blocks = op.block_diagonal(nloc).numpy().reshape(prob.ncells, nloc, nloc)
    ref = prob.block_diagonal()
    assert relmax(blocks, ref) < TOL64
    diag = op.diagonal().numpy()
    assert relmax(diag, np.einsum("cii->ci", ref).ravel()) < TOL64


def test_q1_apply_and_diagonal(gb, orc):
    cells = (9, 7)
    op = gb.Q1Operator(cells, diffusion=1.0, mass=1.0)
    u = np.random.default_rng(2).uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), orc.q1_apply(cells, u, 1.0, 1.0)) < 1e-14
    assert relmax(op.diagonal().numpy(), orc.q1_apply(cells, None, 1.0, 1.0, diag_only=True)) < 1e-14


def test_dot_is_deterministic_fp64_and_fp32(gb):
    n = 3_000_001
    rng = np.random.default_rng(9)
    x, y = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    dx, dy = gb.DeviceArray.from_numpy(x), gb.DeviceArray.from_numpy(y)
    d1, d2 = gb.dot(dx, dy), gb.dot(dx, dy)
    assert d1 == d2
    assert abs(d1 - float(x @ y)) < 1e-10
    fx, fy = gb.DeviceArray.from_numpy(x.astype(np.float32)), gb.DeviceArray.from_numpy(y.astype(np.float32))
    ref = float(x.astype(np.float32).astype(np.float64) @ y.astype(np.float32).astype(np.float64))
    assert abs(gb.dot(fx, fy) - ref) < 1e-9


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_constant_coefficient_form_with_mass_advection_anisotropic(gb, orc, order):
    """Closed-form (coefficient-space) apply against the quadrature oracle on
    the full constant-coefficient form."""
    cells = (3, 2, 4)
    kw = dict(diffusion=0.7, mass=1.3, velocity=(1.0, -0.5, 0.25), periodic=(0, 1, 0),
              lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5))
    op = gb.DGOperator(cells, order, **kw)
    prob = orc.DGProblem(cells, order, **kw)
    u = np.random.default_rng(17 + order).uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u)) < TOL64


@pytest.mark.parametrize("algorithm", [0, 1])
@pytest.mark.parametrize("periodic_z", [0, 1])
@pytest.mark.parametrize("chunks", [1, 2, 3, 7, 0])
def test_pipelined_host_apply_is_bitwise_the_device_apply(gb, orc, algorithm, periodic_z, chunks):
    """The host-buffer apply runs over slabs of z-planes on four streams; every
    slab count (uneven splits, periodic wrap-around in z) gives the device
    apply's result bit for bit."""
    cells = (3, 4, 7)
    kw = dict(mass=0.3, velocity=(0.2, -0.4, 0.7), periodic=(0, 1, periodic_z))
    op = gb.DGOperator(cells, 2, algorithm=algorithm, **kw)
    op.set_host_chunks(chunks)
    u = np.random.default_rng(21).uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    ref = w.numpy()
    for _ in range(2):
        wh = np.full(op.size, np.nan)
        op.apply_host(u, wh)
        assert np.array_equal(wh.view(np.uint64), ref.view(np.uint64))
    prob = orc.DGProblem(cells, 2, **kw)
    assert relmax(ref, prob.apply(u)) < TOL64


@pytest.mark.parametrize("algorithm", [0, 1])
@pytest.mark.parametrize("periodic_z", [0, 1])
@pytest.mark.parametrize("pinned", [False, True])
def test_host_apply_with_tapered_slabs(gb, orc, algorithm, periodic_z, pinned):
    """With three or more z-planes per slab the pipeline makes its first two
    and last two slabs single planes (13 planes in 4 slabs: 1, 1, 4, 4, 1, 1,
    1): bit for bit the device apply, through the direct path (pageable
    buffers) and the captured graph (page-locked buffers)."""
    cells = (3, 4, 13)
    kw = dict(mass=0.3, velocity=(0.2, -0.4, 0.7), periodic=(0, 1, periodic_z))
    op = gb.DGOperator(cells, 2, algorithm=algorithm, **kw)
    op.set_host_chunks(4)
    u = np.random.default_rng(23).uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    ref = w.numpy()
    if pinned:
        torch = pytest.importorskip("torch")
        keep = (torch.from_numpy(u).pin_memory(), torch.empty(op.size, dtype=torch.float64).pin_memory())
        uh, wh = keep[0].numpy(), keep[1].numpy()
    else:
        uh, wh = u, np.empty(op.size)
    for _ in range(2):
        wh[:] = np.nan
        op.apply_host(uh, wh)
        assert np.array_equal(wh.view(np.uint64), ref.view(np.uint64))
    assert relmax(ref, orc.DGProblem(cells, 2, **kw).apply(u)) < TOL64


@pytest.mark.parametrize("precision", [0, 1])
def test_kappa_point_cache_follows_update_coefficients(gb, orc, precision):
    """kappa is evaluated at the Gauss points when the operator is created; a
    changed kappa vector takes effect after update_coefficients."""
    cells, order = (3, 2, 3), 2
    rng = np.random.default_rng(77)
    nloc = (order + 1) ** 3
    ncell = int(np.prod(cells))
    kappa = np.zeros(ncell * nloc)
    kappa[::nloc] = rng.uniform(0.5, 2.0, ncell)
    kappa += 0.05 * rng.uniform(-1, 1, ncell * nloc)
    dt = np.float64 if precision == 0 else np.float32
    dk = gb.DeviceArray.from_numpy(kappa.astype(dt), precision)
    kw = dict(mass=0.2, velocity=(0.1, 0.2, -0.3), periodic=(0, 0, 1))
    op = gb.DGOperator(cells, order, precision=precision, kappa=dk, **kw)
    prob = orc.DGProblem(cells, order, **kw)
    u = rng.uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs, precision)
    tol = TOL64 if precision == 0 else TOL32
    op(gb.DeviceArray.from_numpy(u.astype(dt), precision), w)
    assert relmax(w.numpy(), prob.apply(u.astype(dt).astype(np.float64), kappa=kappa.astype(dt).astype(np.float64))) < tol
    kappa2 = 1.5 * kappa
    k2 = np.ascontiguousarray(kappa2.astype(dt))  # held while the copy reads it
    gb.check(gb.lib().gbfem_memcpy_h2d(dk.ptr, k2.ctypes.data, k2.nbytes))
    op.update_coefficients()
    op(gb.DeviceArray.from_numpy(u.astype(dt), precision), w)
    assert relmax(w.numpy(), prob.apply(u.astype(dt).astype(np.float64), kappa=kappa2.astype(dt).astype(np.float64))) < tol


@pytest.mark.parametrize("cells,periodic", [((1, 1, 1), (0, 0, 0)), ((1, 3, 1), (0, 0, 0)), ((2, 1, 2), (1, 0, 1)),
                                            ((5, 1, 1), (1, 0, 0))])
@pytest.mark.parametrize("algorithm", [0, 1])
def test_degenerate_grids(gb, orc, cells, periodic, algorithm):
    """One cell, one cell thick in some directions, periodic with two cells:
    every face of a direction with one non-periodic cell is a boundary face."""
    kw = dict(mass=0.4, velocity=(0.3, -0.2, 0.1), periodic=periodic)
    op = gb.DGOperator(cells, 2, algorithm=algorithm, **kw)
    prob = orc.DGProblem(cells, 2, **kw)
    u = np.random.default_rng(sum(cells)).uniform(-1, 1, prob.ndofs)
    w = gb.DeviceArray(prob.ndofs)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), prob.apply(u)) < TOL64
    wh = np.empty(prob.ndofs)
    op.set_host_chunks(0)
    op.apply_host(u, wh)
    assert np.array_equal(wh.view(np.uint64), w.numpy().view(np.uint64))
    nl = prob.nloc
    assert relmax(op.block_diagonal(nl).numpy().reshape(-1, nl, nl), prob.block_diagonal()) < TOL64


def test_invalid_descriptors_are_refused(gb):
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((0, 2, 2), 2)          # no cells
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((2, 2, 2), 5)          # order outside 1..4
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((2, 2, 2), 2, quad_points=7)
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((1, 2, 2), 2, periodic=(1, 0, 0))  # periodic needs two cells


@pytest.mark.parametrize("periodic_z", [0, 1])
@pytest.mark.parametrize("chunks", [1, 3, 0])
@pytest.mark.parametrize("nonlinear", [False, True])
def test_host_apply_on_page_locked_buffers_is_bitwise_the_device_apply(gb, orc, periodic_z, chunks, nonlinear):
    """Page-locked host buffers: the kernels read u and write w in host memory
    (NVLink-C2C); the result is the device apply's, bit for bit, and the same as
    the copy pipeline's."""
    torch = pytest.importorskip("torch")
    cells = (3, 4, 7)
    kw = dict(mass=0.3, velocity=(0.2, -0.4, 0.7), periodic=(0, 1, periodic_z))
    op = (gb.NonlinearDGOperator(cells, 2, reaction=(0.1, 0.5, -0.2), **kw) if nonlinear
          else gb.DGOperator(cells, 2, **kw))
    op.set_host_chunks(chunks)
    u = np.random.default_rng(22).uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    ref = w.numpy()
    uh = torch.from_numpy(u).pin_memory()
    wh = torch.full((op.size,), float("nan"), dtype=torch.float64).pin_memory()
    for in_place in (True, False, True):
        op.set_host_transfer(in_place)
        wh.fill_(float("nan"))
        op.apply_host(uh.numpy(), wh.numpy())
        assert np.array_equal(wh.numpy().view(np.uint64), ref.view(np.uint64)), in_place


@pytest.mark.parametrize("algorithm", [0, 1])
def test_host_apply_graph_follows_buffers_and_contents(gb, orc, algorithm):
    """With page-locked buffers the copy pipeline runs as a captured graph.  It
    must read the buffers' contents at each call, be captured again for other
    buffers or another slab count, and agree bit for bit with the device
    apply; pageable buffers take the direct path."""
    torch = pytest.importorskip("torch")
    cells = (4, 3, 8)
    op = gb.DGOperator(cells, 2, mass=0.2, velocity=(0.3, 0.0, -0.5), periodic=(0, 0, 1), algorithm=algorithm)
    rng = np.random.default_rng(31)

    def device_apply(u):
        w = gb.DeviceArray(op.size)
        op(gb.DeviceArray.from_numpy(u), w)
        return w.numpy()

    ua, ub = (torch.from_numpy(rng.uniform(-1, 1, op.size)).pin_memory() for _ in range(2))
    wa, wb = (torch.empty(op.size, dtype=torch.float64).pin_memory() for _ in range(2))
    steps = [(ua, wa, 0, False), (ua, wa, 0, True), (ub, wb, 0, False), (ua, wa, 0, False), (ua, wa, 5, False),
             (ub, wb, 5, True)]
    for u, w, chunks, refill in steps:
        if refill:  # same buffer, new contents
            u.copy_(torch.from_numpy(rng.uniform(-1, 1, op.size)))
        op.set_host_chunks(chunks)
        w.fill_(float("nan"))
        op.apply_host(u.numpy(), w.numpy())
        ref = device_apply(u.numpy())
        assert np.array_equal(w.numpy().view(np.uint64), ref.view(np.uint64)), (chunks, refill)
    u_pageable = rng.uniform(-1, 1, op.size)
    w_pageable = np.full(op.size, np.nan)
    op.apply_host(u_pageable, w_pageable)
    assert np.array_equal(w_pageable.view(np.uint64), device_apply(u_pageable).view(np.uint64))
    assert relmax(w_pageable, orc.DGProblem(cells, 2, mass=0.2, velocity=(0.3, 0.0, -0.5),
                                            periodic=(0, 0, 1)).apply(u_pageable)) < TOL64


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("precision", [0, 1])
def test_cellwise_kappa_closed_form(gb, orc, order, precision):
    """A constant kappa per cell: the closed form (per-cell diffusion scaling,
    two-sided flux weights) equals the Gauss-point oracle on the DG field with
    only the means, and the Gauss-point kernel on the same operator."""
    cells = (3, 2, 4)
    kw = dict(mass=0.6, periodic=(0, 1, 0), lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5))
    rng = np.random.default_rng(90 + order)
    ncell = int(np.prod(cells))
    nloc = (order + 1) ** 3
    kc = rng.uniform(0.2, 3.0, ncell)
    field = np.zeros(ncell * nloc)
    field[::nloc] = kc
    dt = np.float64 if precision == 0 else np.float32
    dkc = gb.DeviceArray.from_numpy(kc.astype(dt), precision)
    op = gb.DGOperator(cells, order, precision=precision, kappa_cell=dkc, **kw)
    opq = gb.DGOperator(cells, order, precision=precision, kappa_cell=dkc, algorithm=gb.ALGO_QUADRATURE, **kw)
    prob = orc.DGProblem(cells, order, **kw)
    u = rng.uniform(-1, 1, prob.ndofs)
    du = gb.DeviceArray.from_numpy(u.astype(dt), precision)
    w, wq = gb.DeviceArray(prob.ndofs, precision), gb.DeviceArray(prob.ndofs, precision)
    op(du, w)
    opq(du, wq)
    ref = prob.apply(u.astype(dt).astype(np.float64), kappa=field.astype(dt).astype(np.float64))
    tol = TOL64 if precision == 0 else TOL32
    assert relmax(w.numpy(), ref) < tol
    assert relmax(wq.numpy(), ref) < tol
    if precision == 0:
        nl = prob.nloc
        assert relmax(op.block_diagonal(nl).numpy().reshape(-1, nl, nl), prob.block_diagonal(kappa=field)) < TOL64
        means = gb.cell_means(gb.DeviceArray.from_numpy(field), order).numpy()
        assert np.array_equal(means, kc)
