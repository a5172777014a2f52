"""dune-fem's own Krylov templates (solver/linear/cg.hh:18-117,
gmres.hh:116-299, bicgstab.hh:63-222) on an SIPG system: 8^3 DG Q2, q = 4,
penalty 90, weak u = 0, b_i = sin(0.37 i + 0.2) (GMRES and BiCGstab on the
advection-diffusion form: diffusion 0.1, mass 1, velocity (1, 0.5, 0.25)).

tests/golden/ref_krylov_sipg.json was written by oracle/make_ref_golden.sh,
which compiles those templates unmodified and runs them over the oracle's
operator.  The reference sources do not travel to the GPU machine, so the GPU
solver is pinned against these vectors: the same iteration counts (within
the spread that the GPU's tree-ordered dot products can cause) and the same
solution at every 97th dof, in norm and in sum.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_krylov_sipg.json")
SYM = dict()
ADV = dict(diffusion=0.1, mass=1.0, velocity=(1.0, 0.5, 0.25))


def _ref():
    with open(GOLD) as f:
        return json.load(f)


def _b(n):
    return np.sin(0.37 * np.arange(n) + 0.2)


def _check_sample(x, rec, tol):
    smp = np.asarray(rec["every97"])
    assert np.max(np.abs(x[::97] - smp)) <= tol * np.max(np.abs(smp))
    assert abs(np.linalg.norm(x) - rec["norm2"]) <= tol * rec["norm2"]
    assert abs(x.sum() - rec["sum"]) <= tol * np.abs(x).sum()


def test_oracle_cg_on_sipg_matches_reference_templates(orc):
    """The oracle's restated CG over the same operator reproduces the
    reference's templates exactly (same sequential dots, same apply)."""
    ref = _ref()
    prob = orc.DGProblem((8, 8, 8), 2, **SYM)
    b = _b(prob.ndofs)
    it, x, _ = orc.cg(prob.apply, b, epsilon=1e-10, max_iter=5000)
    assert it == ref["cg_iterations"]
    _check_sample(x, ref["cg_x"], 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cg", "diag_pcg", "gmres", "bicgstab"])
def test_gpu_krylov_on_sipg_matches_reference_templates(gb, case):
    ref = _ref()
    kw = SYM if case in ("cg", "diag_pcg") else ADV
    op = gb.DGOperator((8, 8, 8), 2, **kw)
    method = {"cg": "cg", "diag_pcg": "cg", "gmres": "gmres", "bicgstab": "bicgstab"}[case]
    pc = gb.Preconditioner.diagonal(op) if case == "diag_pcg" else None
    inv = gb.KrylovInverseOperator(method, tolerance=1e-10, max_iterations=5000, restart=ref["gmres_restart"])
    inv.bind(op, pc)
    b = gb.DeviceArray.from_numpy(_b(op.size))
    u = gb.DeviceArray(op.size)
    u.clear()
    inv(b, u)
    info = inv.info()
    want = ref[case + "_iterations"]
    print("%s: gpu %d iterations, reference %d" % (case, info["iterations"], want))
    assert info["converged"]
    # BiCGstab's residual is not monotone, so where it first drops below the
    # tolerance moves with the rounding of the dot products (here 435 vs 418);
    # CG and GMRES stay within 1 %
    spread = 0.05 if case == "bicgstab" else 0.01
    assert abs(info["iterations"] - want) <= max(1, int(spread * want))
    _check_sample(u.numpy(), ref[case + "_x"], 1e-7)
