"""GPU against the oracle at the benchmark problems' own sizes.

The small-grid parity tests pin every term of the form; these pin the index
arithmetic and the launch shapes at the sizes that are benchmarked:
- 64^3 DG Q3 SIPG apply, q = 5 (16.8M dofs): the whole vector against the
  oracle's whole apply (all host threads);
- 128^3 DG Q2 periodic advection-diffusion, one SSP-RK3 step (56.6M dofs):
  whole z-planes at both ends (across the periodic wrap) and in the middle,
  against the oracle's step restricted to where those planes depend on it;
- 96^3 DG Q4 variable-kappa SIPG apply, q = 6 (110.6M dofs), kappa a
  log-Gaussian field of 256 Fourier modes: whole z-planes at both ends and
  in the middle against the oracle's apply over those planes and their
  neighbour planes, for kappa as a DG field (Gauss-point kernel) and for
  kappa's cell means (the closed form of the mixed solve's inner operator).

The bar: FP64 within 1e-12 of the oracle, relative to the max norm of the
oracle's whole result (sampled planes: of the sampled rows); FP32 within the
bound written at each assertion, its measured value printed.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
NTHREADS = os.cpu_count() or 1


def _err(a, b, scale=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.max(np.abs(b)) if scale is None else scale
    return float(np.max(np.abs(a - b)) / s)


def test_sipg_q3_64cube_whole_apply(gb, orc):
    cells, p = (64, 64, 64), 3
    prob = orc.DGProblem(cells, p, quad_points=5)
    u = np.random.default_rng(20261203).uniform(-1.0, 1.0, prob.ndofs)
    ref = prob.apply(u, nthreads=NTHREADS)
    du = gb.DeviceArray.from_numpy(u)
    w = gb.DeviceArray(prob.ndofs)
    for algo in (gb.ALGO_AUTO, gb.ALGO_QUADRATURE):
        op = gb.DGOperator(cells, p, quad_points=5, algorithm=algo)
        op(du, w)
        e = _err(w.numpy(), ref)
        print("64^3 Q3 FP64 algorithm %d: rel max err %.3e" % (algo, e))
        assert e < TOL64
        del op
    op32 = gb.DGOperator(cells, p, quad_points=5, precision=gb.F32)
    u32 = gb.DeviceArray.from_numpy(u.astype(np.float32))
    w32 = gb.DeviceArray(prob.ndofs, gb.F32)
    op32(u32, w32)
    ref32 = prob.apply(u.astype(np.float32).astype(np.float64), nthreads=NTHREADS)
    e32 = _err(w32.numpy(), ref32)
    print("64^3 Q3 FP32 closed form: rel max err %.3e" % e32)
    assert e32 < 1e-6


def test_rk3_step_q2_128cube_periodic_planes(gb, orc):
    cells, p = (128, 128, 128), 2
    kw = dict(diffusion=1e-3, velocity=(1.0, 0.5, 0.25), periodic=(1, 1, 1), weak_dirichlet=False)
    prob = orc.DGProblem(cells, p, **kw)
    dt = 1.95e-5  # the step of the benchmark run: the SIPG stability bound 2 / rho(M^-1 A)
    u0 = np.random.default_rng(3).uniform(-1.0, 1.0, prob.ndofs)
    per = 128 * 128 * 27
    ranges = ((0, 2), (63, 65), (126, 128))
    refs = {zr: prob.rk3_step_planes(u0, dt, zr[0], zr[1], nthreads=NTHREADS)[zr[0] * per:zr[1] * per]
            for zr in ranges}
    scale = max(np.max(np.abs(r)) for r in refs.values())
    for prec, tol, name in ((gb.F64, TOL64, "FP64"), (gb.F32, 1e-6, "FP32")):
        op = gb.DGOperator(cells, p, precision=prec, **kw)
        u = gb.DeviceArray.from_numpy(u0 if prec == gb.F64 else u0.astype(np.float32))
        gb.RK3(op).step(u, dt)
        got = u.numpy()
        for zr in ranges:
            e = _err(got[zr[0] * per:zr[1] * per], refs[zr], scale)
            print("128^3 Q2 RK3 %s planes %s: rel max err %.3e" % (name, zr, e))
            assert e < tol
        del op, u, got


def test_sipg_q4_96cube_variable_kappa_planes(gb, orc):
    cells, p, q = (96, 96, 96), 4, 6
    nloc = 125
    nxy = 96 * 96
    per = nxy * nloc
    modes = gb.fourier_modes(1)
    kap = gb.project(cells, p, gb.FN_EXP_FOURIER, modes=modes)
    kappa = kap.numpy()
    prob = orc.DGProblem(cells, p, quad_points=q)
    u = np.random.default_rng(11).uniform(-1.0, 1.0, prob.ndofs)
    ranges = ((0, 2), (47, 49), (94, 96))
    # kappa's cell means as a DG field: the cellwise-constant coefficient
    kmean = np.zeros_like(kappa)
    kmean[::nloc] = kappa[::nloc]

    def oracle_planes(kv):
        out = {}
        for z0, z1 in ranges:
            w = np.zeros(prob.ndofs)
            prob.apply_cells(u, w, max(0, z0 - 1) * nxy, min(96, z1 + 1) * nxy, kappa=kv, nthreads=NTHREADS)
            out[(z0, z1)] = w[z0 * per:z1 * per].copy()
        return out

    ref_k = oracle_planes(kappa)
    ref_m = oracle_planes(kmean)
    du = gb.DeviceArray.from_numpy(u)
    u32 = gb.DeviceArray.from_numpy(u.astype(np.float32))
    cases = [
        ("DG-field kappa FP64", ref_k, gb.F64, TOL64,
         lambda: gb.DGOperator(cells, p, quad_points=q, kappa=kap)),
        ("DG-field kappa FP32", ref_k, gb.F32, 1e-6,
         lambda: gb.DGOperator(cells, p, quad_points=q, precision=gb.F32, kappa=gb.convert(kap, gb.F32))),
        ("cell-mean kappa FP64", ref_m, gb.F64, TOL64,
         lambda: gb.DGOperator(cells, p, quad_points=q, kappa_cell=gb.cell_means(kap, p))),
        ("cell-mean kappa FP32", ref_m, gb.F32, 1e-6,
         lambda: gb.DGOperator(cells, p, quad_points=q, precision=gb.F32,
                               kappa_cell=gb.convert(gb.cell_means(kap, p), gb.F32))),
    ]
    for name, ref, prec, tol, make in cases:
        op = make()
        w = gb.DeviceArray(prob.ndofs, prec)
        op(du if prec == gb.F64 else u32, w)
        got = w.numpy()
        scale = max(np.max(np.abs(r)) for r in ref.values())
        for zr in ranges:
            e = _err(got[zr[0] * per:zr[1] * per], ref[zr], scale)
            print("96^3 Q4 %s planes %s: rel max err %.3e" % (name, zr, e))
            assert e < tol
        del op, w, got
