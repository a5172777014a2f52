"""Pins the CPU oracle against the reference's own compiled code.

tests/golden/ref_tables.json and ref_krylov.json were produced by
oracle/make_ref_golden.sh, which compiles dune-fem's gausspoints.hh,
legendrepolynomials.cc and solver/linear/{cg,gmres,bicgstab}.hh unmodified.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_gauss_rules_match_reference(orc):
    ref = load("ref_tables.json")["gauss"]
    for m_str, rule in ref.items():
        m = int(m_str)
        p, w = orc.gauss(m)
        assert rule["order"] == 2 * m - 1
        np.testing.assert_allclose(p, rule["points"], rtol=0, atol=2e-16)
        np.testing.assert_allclose(w, rule["weights"], rtol=0, atol=4e-16)


def test_legendre_tables_match_reference(orc):
    """Degrees 0..9 agree with the reference's table.  Degree 10 does not: the
    reference's coefficient factor[10][3] (legendrepolynomials.cc:27) reads
    -34920, while (-1)^13 C(10,3) C(13,3) = -34320.  This build uses p <= 4."""
    ref = load("ref_tables.json")["legendre"]
    xs = ref["x"]
    for k, (vals, ders) in enumerate(zip(ref["value"][:10], ref["jacobian"][:10])):
        for x, v, d in zip(xs, vals, ders):
            assert abs(orc.legendre(k, x) - v) <= 1e-13 * max(1.0, abs(v))
            assert abs(orc.legendre_d(k, x) - d) <= 1e-13 * max(1.0, abs(d))


def _tri(lo, up, d0, slope):
    def op(x):
        n = x.size
        d = d0 + slope * np.arange(n) / n
        y = d * x
        y[1:] += lo * x[:-1]
        y[:-1] += up * x[1:]
        return y
    return op


def test_cg_matches_reference_iterates(orc):
    ref = load("ref_krylov.json")
    b = np.array(ref["b"])
    spd = _tri(-1.0, -1.0, 2.05, 0.5)
    it, x, _ = orc.cg(spd, b, epsilon=1e-10, max_iter=1000)
    assert it == ref["cg_iterations"]
    np.testing.assert_allclose(x, ref["cg_x"], rtol=0, atol=1e-12 * np.abs(ref["cg_x"]).max())
    jac = lambda r: r / (2.05 + 0.5 * np.arange(r.size) / r.size)
    it, x, _ = orc.cg(spd, b, prec=jac, epsilon=1e-10, max_iter=1000)
    assert it == ref["pcg_iterations"]
    np.testing.assert_allclose(x, ref["pcg_x"], rtol=0, atol=1e-12 * np.abs(ref["pcg_x"]).max())


def test_gmres_matches_reference_iterates(orc):
    ref = load("ref_krylov.json")
    b = np.array(ref["b"])
    A = _tri(-1.3, -0.7, 2.5, 0.3)
    m = ref["gmres_restart"]
    it, x, _ = orc.gmres(A, b, m, tolerance=1e-10, max_iter=1000)
    assert it == ref["gmres_iterations"]
    np.testing.assert_allclose(x, ref["gmres_x"], rtol=0, atol=1e-12 * np.abs(ref["gmres_x"]).max())
    jac = lambda r: r / (2.5 + 0.3 * np.arange(r.size) / r.size)
    it, x, _ = orc.gmres(A, b, m, prec=jac, tolerance=1e-10, max_iter=1000)
    assert it == ref["pgmres_iterations"]
    np.testing.assert_allclose(x, ref["pgmres_x"], rtol=0, atol=1e-12 * np.abs(ref["pgmres_x"]).max())


def test_reference_degree10_table_defect_is_what_we_think(orc):
    ref = load("ref_tables.json")["legendre"]
    # at x = 1 every shifted Legendre polynomial is 1 before normalisation:
    # sqrt(21) * P_10(1) = sqrt(21); the reference's table misses it by
    # sqrt(21) * (34920 - 34320) = 600 sqrt(21).
    x1 = ref["x"].index(1.0)
    assert abs(orc.legendre(10, 1.0) - np.sqrt(21.0)) < 1e-9
    assert abs(ref["value"][10][x1] - np.sqrt(21.0) * (1 - 600)) < 1e-6
