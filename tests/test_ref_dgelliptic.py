"""The DG operator against dune-fem's own DGEllipticOperator.

tests/golden/ref_dgelliptic.json holds w = A u computed by the reference's
DGEllipticOperator::apply and DefaultPenalty (dune/fem/schemes/dgelliptic.hh)
over its LegendreShapeFunctionSet and GaussPts, compiled unmodified by
oracle/make_ref_golden.sh against a small Cartesian grid layer of our own
(oracle/shim_dg).  The model is diffusion * kappa(x) grad u with a mass term,
kappa an optional Q_p field; the cases cover Q1..Q4, q = p+1 and p+2,
anisotropic cells, periodic, do-nothing and weak Dirichlet boundaries.

On weak Dirichlet faces that operator weights the symmetry term
-[u] kappa grad v . n by 1/2 (dgelliptic.hh:426-431); the SIPG form of this
path (and of the reference's UFL demo form on interior faces) takes it in
full.  The oracle reproduces either (weak_dirichlet=True or "dgelliptic");
the GPU DG operator implements the full term, so its Dirichlet cases are
checked through the oracle, and the reference's boundary variant itself runs
on the GPU as a run-time compiled form.
"""
import json
import os

import numpy as np
import pytest

from conftest import relmax

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_dgelliptic.json")
with open(GOLD) as _f:
    CASES = {c["name"]: c for c in json.load(_f)["cases"]}
# the same operator's assembled Jacobian (DifferentiableDGEllipticOperator::
# jacobian, dgelliptic.hh:456-766): J v, its diagonal, some diagonal blocks
# and the Frobenius norms of all nonzero cell blocks
with open(os.path.join(os.path.dirname(__file__), "golden", "ref_dgelliptic_jacobian.json")) as _f:
    JAC = {c["name"]: c for c in json.load(_f)["cases"]}


def inputs(case):
    """u and the kappa field exactly as the reference driver built them
    (integer formulas whose conversion to double is exact)."""
    p = case["order"]
    nl = (p + 1) ** 3
    ncell = int(np.prod(case["cells"]))
    i = np.arange(ncell * nl, dtype=np.int64)
    u = ((i * 7919 + 13) % 2003 - 1001) / 1000.0
    kappa = None
    if case["kappa_field"]:
        c = np.arange(ncell, dtype=np.int64)
        idx = c[:, None] * nl + np.arange(nl, dtype=np.int64)[None, :]
        kappa = ((idx * 37 + 5) % 9 - 4) / 1000.0
        kappa[:, 0] = 1.0 + ((c * 31 + 7) % 11) / 10.0
        kappa = kappa.reshape(-1)
    return u, kappa


def probe(n):
    """The second probe vector of the Jacobian golden (exact, as u)."""
    i = np.arange(n, dtype=np.int64)
    return ((i * 4243 + 7) % 1999 - 999) / 1000.0


def problem_kw(case):
    return dict(quad_points=case["quad_points"], diffusion=case["diffusion"], penalty=case["penalty"],
                mass=case["mass"], periodic=tuple(case["periodic"]), upper=tuple(case["upper"]))


def test_golden_cases_present():
    assert len(CASES) == 8
    assert {c["order"] for c in CASES.values()} == {1, 2, 3, 4}
    assert any(c["dirichlet"] for c in CASES.values())


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_equals_reference_dgelliptic(orc, name):
    case = CASES[name]
    u, kappa = inputs(case)
    prob = orc.DGProblem(tuple(case["cells"]), case["order"],
                         weak_dirichlet="dgelliptic" if case["dirichlet"] else False, **problem_kw(case))
    assert relmax(prob.apply(u, kappa=kappa), case["w"]) < 1e-13


def test_full_symmetry_term_differs_only_in_boundary_cells(orc):
    """The symmetric SIPG boundary of this path and the reference operator's
    differ only in cells with a Dirichlet face (here: all but the 2x2x2 core
    of a 4^3 grid)."""
    cells, p = (4, 4, 4), 2
    rng = np.random.default_rng(3)
    kw = dict(quad_points=3, penalty=90.0, mass=0.3)
    full = orc.DGProblem(cells, p, weak_dirichlet=True, **kw)
    half = orc.DGProblem(cells, p, weak_dirichlet="dgelliptic", **kw)
    u = rng.uniform(-1, 1, full.ndofs)
    d = np.abs(full.apply(u) - half.apply(u)).reshape(4, 4, 4, -1).max(axis=-1)
    assert np.all(d[1:3, 1:3, 1:3] == 0.0)
    border = np.ones((4, 4, 4), bool)
    border[1:3, 1:3, 1:3] = False
    assert np.all(d[border] > 1e-3)


def test_gpu_operator_rejects_the_half_symmetry_boundary(gb):
    """DGOperator implements the symmetric boundary only; asking it for the
    reference operator's variant is an error, not a silent substitution."""
    with pytest.raises(ValueError):
        gb.DGOperator((2, 2, 2), 2, weak_dirichlet="dgelliptic")


@pytest.mark.parametrize("name", sorted(JAC))
def test_oracle_matrix_equals_reference_jacobian(orc, name):
    """The oracle's operator, assembled column by column, is the reference's
    assembled Jacobian: the same nonzero cell blocks with the same norms,
    products, diagonal and diagonal blocks."""
    case = JAC[name]
    _, kappa = inputs(case)
    prob = orc.DGProblem(tuple(case["cells"]), case["order"],
                         weak_dirichlet="dgelliptic" if case["dirichlet"] else False, **problem_kw(case))
    n, nl = prob.ndofs, prob.nloc
    A = np.stack([prob.apply(e, kappa=kappa) for e in np.eye(n)], axis=1)
    assert relmax(A @ probe(n), case["Jv"]) < 1e-13
    assert relmax(np.diag(A), case["diag"]) < 1e-13
    ref_norms = {(r, c): f for r, c, f in case["block_norms"]}
    blocks = A.reshape(prob.ncells, nl, prob.ncells, nl)
    norms = np.linalg.norm(blocks, axis=(1, 3))
    assert set(zip(*np.nonzero(norms))) == set(ref_norms)
    assert max(abs(norms[k] - f) / f for k, f in ref_norms.items()) < 1e-13
    bd = prob.block_diagonal(kappa=kappa)
    cells = case["block_cells"]
    if cells:
        assert relmax(bd[cells], np.array(case["blocks"]).reshape(len(cells), nl, nl)) < 1e-13


# ---- the reference operator's integrands as a raw form ------------------------------


def _raw_numpy(eps, c, dirichlet):
    """interior / skeleton / boundary integrands of DGEllipticOperator for
    flux eps grad u, source c u (constant kappa), in the form oracle's
    convention (own side's test coefficients)."""

    def interior(x, u, g):
        return c * u, eps * g

    def skeleton(x, n, sigma, uL, gL, uR, gR):
        j = uL - uR
        s = sigma * eps * j - 0.5 * eps * np.einsum("pmk,k->pm", gL + gR, n)
        return s, -0.5 * eps * j[:, :, None] * n[None, None, :]

    def boundary(x, n, sigma, u, g):
        if not dirichlet:
            return np.zeros_like(u), np.zeros_like(g)
        s = sigma * eps * u - eps * np.einsum("pmk,k->pm", g, n)
        return s, -0.5 * eps * u[:, :, None] * n[None, None, :]

    return interior, skeleton, boundary


def _raw_form(integrands, eps, c, dirichlet):
    """The same integrands as CUDA statements for integrands.Form."""
    e = repr(float(eps))
    interior = "s[0] = %r * u[0]; for (int k = 0; k < 3; ++k) F[0][k] = %s * g[0][k];" % (float(c), e)
    skeleton = ("const D j = uL[0] - uR[0];"
                " const D gn = (gL[0][0] + gR[0][0]) * n[0] + (gL[0][1] + gR[0][1]) * n[1]"
                " + (gL[0][2] + gR[0][2]) * n[2];"
                " s[0] = sigma * %s * j - 0.5 * %s * gn;"
                " for (int k = 0; k < 3; ++k) F[0][k] = -0.5 * %s * j * n[k];" % (e, e, e))
    boundary = ""
    if dirichlet:
        boundary = ("const D gn = g[0][0] * n[0] + g[0][1] * n[1] + g[0][2] * n[2];"
                    " s[0] = sigma * %s * u[0] - %s * gn;"
                    " for (int k = 0; k < 3; ++k) F[0][k] = -0.5 * %s * u[0] * n[k];" % (e, e, e))
    return integrands.Form(interior=interior, skeleton=skeleton, boundary=boundary)


CONST_CASES = sorted(n for n, c in CASES.items() if not c["kappa_field"])


@pytest.mark.parametrize("name", CONST_CASES)
def test_form_oracle_raw_integrands_equal_reference(name):
    import form_oracle as fo
    case = CASES[name]
    u, _ = inputs(case)
    I, S, B = _raw_numpy(case["diffusion"], case["mass"], case["dirichlet"])
    spec = fo.FormSpec(tuple(case["cells"]), case["order"], 1, I, S, B, quad_points=case["quad_points"],
                       penalty=case["penalty"], periodic=tuple(case["periodic"]), upper=tuple(case["upper"]))
    assert relmax(fo.residual(spec, u), case["w"]) < 1e-13


def test_raw_form_compiles(gb, tmp_path):
    import integrands
    case = CASES["q3_dirichlet_aniso_qp2"]
    form = _raw_form(integrands, case["diffusion"], case["mass"], True)
    assert form.compile(gb.F64, case["order"], case["quad_points"], cache_dir=str(tmp_path)).endswith(".cubin")


# ---- GPU ------------------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", [0, 1])
@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if not c["dirichlet"]))
def test_gpu_dg_operator_equals_reference_dgelliptic(gb, name, algorithm):
    """DGOperator (do-nothing or periodic boundaries) against the reference
    operator's output; algorithm 0 is the closed form where kappa is constant
    (the Gauss-point kernel otherwise), 1 the Gauss-point kernel."""
    case = CASES[name]
    u, kappa = inputs(case)
    op = gb.DGOperator(tuple(case["cells"]), case["order"], weak_dirichlet=False, algorithm=algorithm,
                       kappa=None if kappa is None else gb.DeviceArray.from_numpy(kappa), **problem_kw(case))
    w = gb.DeviceArray(u.size)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), case["w"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", CONST_CASES)
def test_gpu_raw_form_equals_reference_dgelliptic(gb, name):
    """The reference operator's integrands, boundary variant included, as a
    run-time compiled form on the GPU."""
    import integrands
    case = CASES[name]
    u, _ = inputs(case)
    op = integrands.FormOperator(_raw_form(integrands, case["diffusion"], case["mass"], case["dirichlet"]),
                                 tuple(case["cells"]), case["order"], quad_points=case["quad_points"],
                                 penalty=case["penalty"], periodic=tuple(case["periodic"]),
                                 upper=tuple(case["upper"]))
    w = gb.DeviceArray(u.size)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), case["w"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(n for n, c in JAC.items() if not c["dirichlet"]))
def test_gpu_jacobian_equals_reference_jacobian(gb, name):
    """The block diagonal, the diagonal and the assembled block-sparse matrix
    of DGOperator against the reference's assembled Jacobian."""
    case = JAC[name]
    _, kappa = inputs(case)
    op = gb.DGOperator(tuple(case["cells"]), case["order"], weak_dirichlet=False,
                       kappa=None if kappa is None else gb.DeviceArray.from_numpy(kappa), **problem_kw(case))
    nl = (case["order"] + 1) ** 3
    ncells = int(np.prod(case["cells"]))
    assert relmax(op.diagonal().numpy(), case["diag"]) < 1e-12
    cells = case["block_cells"]
    if cells:
        bd = op.block_diagonal(nl).numpy().reshape(ncells, nl, nl)
        assert relmax(bd[cells], np.array(case["blocks"]).reshape(len(cells), nl, nl)) < 1e-12
    A = op.assemble()
    v = probe(ncells * nl)
    y = gb.DeviceArray(v.size)
    A(gb.DeviceArray.from_numpy(v), y)
    assert relmax(y.numpy(), case["Jv"]) < 1e-12
    assert relmax(A.diagonal().numpy(), case["diag"]) < 1e-12
