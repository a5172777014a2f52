"""The C-ABI library loads and exports every entry point include/*.h declares.

No compute call is made: this runs without a GPU.
"""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gbfem_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbfem_operator_apply" in syms
    assert "gbfem_dot" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(gb):
    lib = ctypes.CDLL(gb.LIB_PATH)
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, "not exported: %s" % missing


def test_version_and_error_string(gb):
    L = gb.lib()
    assert L.gbfem_version() >= 100
    assert isinstance(L.gbfem_last_error(), bytes)


def test_invalid_descriptor_is_rejected_without_gpu(gb):
    # order 9 is out of range: rejected on the host before any device call
    import pytest
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((2, 2, 2), 9)


def _reference_hierarchical_order(order, dim):
    """LegendreShapeFunctionSet with hierarchical ordering (legendre.hh:236-249,
    294-299): the multi-indices of DefaultFactory::fill (first index slowest)
    sorted by maximal degree, then lexicographically."""
    import itertools
    idx = list(itertools.product(range(order + 1), repeat=dim))  # fill order: non-hierarchical index = position
    return sorted(range(len(idx)), key=lambda l: (max(idx[l]), idx[l]))


def test_hierarchical_permutation_equals_the_compiled_reference_set(gb):
    """tests/golden/ref_legendre_order.json: the order of dune-fem's own
    LegendreShapeFunctionSet<FS, true> (legendre.hh, compiled unmodified by
    oracle/make_ref_golden.sh) as indices into the default set, dims 1-3,
    orders 0-4."""
    import json
    with open(os.path.join(os.path.dirname(__file__), "golden", "ref_legendre_order.json")) as f:
        orders = json.load(f)["orders"]
    assert len(orders) == 15
    for o in orders:
        assert list(gb.hierarchical_permutation(o["order"], o["dim"])) == o["perm"]


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_hierarchical_permutation_matches_the_reference_sort(gb, order, dim):
    perm = gb.hierarchical_permutation(order, dim)
    assert list(perm) == _reference_hierarchical_order(order, dim)
    if order == 1 and dim == 3:
        assert list(perm) == list(range(8))  # every Q1 function other than 1 has degree 1: lexicographic = natural
    if order == 2 and dim == 2:
        assert list(perm) == [0, 1, 3, 4, 2, 5, 6, 7, 8]
