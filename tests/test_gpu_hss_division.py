"""GPU: HSS-valued division hssA \\ hssB and hssB / hssA (src/ulvdivide.jl:13-17,
src/hssmatrix.jl:235-237) against dense inverses, as the reference's own test
does (test/runtests.jl:68-77): the identity compressed by randcompress with
kest = 0, then A \\ I and I / A against inv(A), within c rtol with c = 50.
"""
import numpy as np
import pytest

from conftest import load_golden, unpack_tree

pytestmark = pytest.mark.gpu

C = 50.0


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _identity(pkg, A, tol):
    rcl, ccl = pkg.cluster_trees(A)
    n = A.size()[0]
    return pkg.randcompress(np.eye(n), rcl, ccl, 0, atol=tol, rtol=tol)


@pytest.mark.parametrize("name", ["cauchy2001_compress", "synthetic_uneven"])
def test_ldiv_rdiv_identity(pkg, orc, name):
    """A \\ I and I / A approximate inv(A) (runtests.jl:73, :74)."""
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    A = pkg.HssMatrix.from_tree(h)
    tol = 1e-6
    I = _identity(pkg, A, tol)
    assert rel(pkg.full(I), np.eye(A.size()[0])) <= C * tol
    Ainv = np.linalg.inv(orc.full(h))
    st = {}
    X = pkg.ldiv(A, I, atol=tol, rtol=tol, stats=st)
    assert isinstance(X, pkg.HssMatrix) and st["rounds"] >= 1
    assert rel(pkg.full(X), Ainv) <= C * tol
    Y = I / A
    assert rel(pkg.full(Y), Ainv) <= C * tol


def test_ldiv_general(pkg, orc):
    """A \\ B and B / A for a second HSS matrix B on the same cluster tree."""
    rng = np.random.default_rng(7)
    ha = orc.synthetic_hss(1536, 128, 16, rng)
    hb = orc.synthetic_hss(1536, 128, 12, rng)
    A, B = pkg.HssMatrix.from_tree(ha), pkg.HssMatrix.from_tree(hb)
    Af, Bf = orc.full(ha), orc.full(hb)
    tol = 1e-9
    X = pkg.hss_ldiv(A, B, atol=tol, rtol=tol)
    assert rel(pkg.full(X), np.linalg.solve(Af, Bf)) <= C * tol
    Y = pkg.rdiv(B, A, atol=tol, rtol=tol)
    assert rel(pkg.full(Y), np.linalg.solve(Af.T, Bf.T).T) <= C * tol
    # the ranks stay near rank(A) + rank(B)
    assert pkg.hssrank(X) <= 16 + 12 + 16


def test_ldiv_shape_errors(pkg, orc):
    rng = np.random.default_rng(2)
    A = pkg.HssMatrix.from_tree(orc.synthetic_hss(512, 64, 8, rng))
    B = pkg.HssMatrix.from_tree(orc.synthetic_hss(640, 64, 8, rng))
    with pytest.raises(ValueError):
        pkg.hss_ldiv(A, B)
    with pytest.raises(ValueError):
        pkg.rdiv(B, A)
