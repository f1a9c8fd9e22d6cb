"""GPU orthonormalize_generators! / recompress! (src/generators.jl:64-114,
src/compression.jl:148-260) against the oracle's restatement.

Both sides take every rank decision with the same column-pivoted QR rule
(xLAQP2 pivots, keep |R_ii| > max(atol, rtol |R_11|)), so ranks agree node by
node and the results agree as operators within 1e-10 relative.  The
orthonormalized bases are orthonormal to 1e-12 and leave the operator
unchanged to 1e-12; recompression stays within the reference suite's bound
(c = 50 times the tolerance, test/runtests.jl:38-40)."""
import copy

import numpy as np
import pytest

from conftest import unpack_tree

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def as_oracle(pkg, orc, h):
    table, packed = pkg.pack(h)
    return unpack_tree(table, packed, orc)


def ranks(orc, h):
    return [orc.gensize(x) for x in orc.iter_nodes(h) if not x.rootnode]


def _product_case(orc):
    rng = np.random.default_rng(3)
    A = orc.synthetic_hss(1024, 64, 10, rng)
    B = orc.synthetic_hss(1024, 64, 8, rng)
    return orc.hssmul(A, B)


def _cauchy_case(orc, n=2001, tol=1e-6):
    M = orc.cauchy_matrix(n)
    cl = orc.bisection_cluster(n, 64)
    return orc.compress(M, cl, cl, tol, tol)


@pytest.mark.parametrize("case", ["product", "cauchy"])
def test_orthonormalize_matches_oracle(pkg, orc, case):
    h = _product_case(orc) if case == "product" else _cauchy_case(orc)
    ho = orc.orthonormalize_generators(copy.deepcopy(h))
    hg = as_oracle(pkg, orc, pkg.orthonormalize_generators(pkg.HssMatrix.from_tree(h)))
    F = orc.full(h)
    assert rel(orc.full(hg), F) <= 1e-12
    assert ranks(orc, hg) == ranks(orc, ho)
    for x in orc.iter_nodes(hg):
        if x.rootnode:
            continue
        Q = x.U if x.leafnode else np.vstack([x.R1, x.R2])
        P = x.V if x.leafnode else np.vstack([x.W1, x.W2])
        for M in (Q, P):
            assert np.abs(M.T @ M - np.eye(M.shape[1])).max() <= 1e-12


@pytest.mark.parametrize("case,tol", [("product", 1e-10), ("cauchy", 1e-4), ("cauchy", 1e-8)])
def test_recompress_matches_oracle(pkg, orc, case, tol):
    h = _product_case(orc) if case == "product" else _cauchy_case(orc)
    ho = orc.recompress(copy.deepcopy(h), tol, tol)
    hg = as_oracle(pkg, orc, pkg.recompress(pkg.HssMatrix.from_tree(h), atol=tol, rtol=tol))
    assert ranks(orc, hg) == ranks(orc, ho)
    F = orc.full(h)
    assert rel(orc.full(hg), orc.full(ho)) <= 1e-10
    err = np.linalg.norm(orc.full(hg) - F)
    assert err / np.linalg.norm(F) <= 50 * tol or err <= 50 * tol


def test_recompress_after_product_lowers_ranks(pkg, orc):
    """The HSS product of two compressed kernel matrices doubles the ranks;
    recompression brings them down and keeps the product within tolerance."""
    h = _cauchy_case(orc)
    A = pkg.HssMatrix.from_tree(h)
    C = pkg.hssmul(A, A)
    Cr = pkg.recompress(C, atol=1e-8, rtol=1e-8)
    assert pkg.hssrank(Cr) < pkg.hssrank(C)
    ref = orc.full(h) @ orc.full(h)
    assert rel(orc.full(as_oracle(pkg, orc, Cr)), ref) <= 1e-6


def test_recompress_single_leaf_and_forest(pkg, orc):
    """A single leaf has nothing to recompress (compression.jl:152); forests
    are rejected (the reference works on one tree)."""
    h = orc.synthetic_hss(60, 64, 5, np.random.default_rng(8))
    r = as_oracle(pkg, orc, pkg.recompress(pkg.HssMatrix.from_tree(h), atol=1e-6, rtol=1e-6))
    assert rel(orc.full(r), orc.full(h)) <= 1e-15
    rng = np.random.default_rng(9)
    trees = [orc.synthetic_hss(300, 64, 8, rng), orc.synthetic_hss(200, 64, 8, rng)]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    with pytest.raises(ValueError):
        pkg.recompress(dev)
    with pytest.raises(ValueError):
        pkg.orthonormalize_generators(dev)
