"""The stationary-iteration preconditioners against dune-fem's own
FemPreconditioning.

tests/golden/ref_precond.json was made by oracle/make_ref_golden.sh, which
compiles the reference's solver/fempreconditioning.hh and the sweeps of
operator/matrix/spmatrix.hh (SparseRowMatrix::forwardIterative /
backwardIterative) unmodified and applies its Jacobi, Gauss-Seidel, SOR and
SSOR preconditioners to a vector, on the assembled Jacobian of the
reference's DGEllipticOperator (Q2, 3x2x2 cells, kappa field, mass term).
They were built with 3 iterations and relaxation 1.5 requested, as
KrylovInverseOperator passes them (krylovinverseoperators.hh:226-250);
FemPreconditioning's constructor drops both (fempreconditioning.hh:184-186),
so one sweep with relaxation 1 is what runs.  The GPU preconditioner
(gbfem_preconditioner_sor_create) is checked against the same smoother
oracle in tests/test_solvers.py.
"""
import json
import os

import numpy as np
import pytest

from conftest import relmax

with open(os.path.join(os.path.dirname(__file__), "golden", "ref_precond.json")) as _f:
    GOLD = json.load(_f)


def _matrix_and_probe(orc):
    p = GOLD["order"]
    prob = orc.DGProblem(tuple(GOLD["cells"]), p, quad_points=GOLD["quad_points"], penalty=GOLD["penalty"],
                         mass=GOLD["mass"], weak_dirichlet=False)
    nl, n = prob.nloc, prob.ndofs
    i = np.arange(n, dtype=np.int64)
    r = ((i * 7919 + 13) % 2003 - 1001) / 1000.0
    c = np.arange(prob.ncells, dtype=np.int64)
    idx = c[:, None] * nl + np.arange(nl, dtype=np.int64)[None, :]
    kappa = ((idx * 37 + 5) % 9 - 4) / 1000.0
    kappa[:, 0] = 1.0 + ((c * 31 + 7) % 11) / 10.0
    A = np.stack([prob.apply(e, kappa=kappa.reshape(-1)) for e in np.eye(n)], axis=1)
    return A, r


@pytest.mark.parametrize("method", ["jacobi", "gauss-seidel", "sor", "ssor"])
def test_smoother_oracle_equals_reference(orc, method):
    import smoother_oracle as so
    A, r = _matrix_and_probe(orc)
    assert relmax(so.smoother_apply(A, r, method, iterations=1, relaxation=1.0), GOLD[method]) < 1e-13


def test_reference_drops_iterations_and_relaxation(orc):
    """SOR equals Gauss-Seidel in the golden vectors, and honouring the
    requested 3 sweeps with relaxation 1.5 would give something else."""
    import smoother_oracle as so
    A, r = _matrix_and_probe(orc)
    assert GOLD["requested_iterations"] == 3 and GOLD["requested_relaxation"] == 1.5
    assert GOLD["sor"] == GOLD["gauss-seidel"]
    honoured = so.smoother_apply(A, r, "sor", iterations=3, relaxation=1.5)
    assert relmax(honoured, GOLD["sor"]) > 1e-2
