"""GPU HSS x HSS product (src/matmul.jl:65-117) against the oracle's
restatement (oracle.hssmul): the same tree, ranks adding up, every generator
block equal within 1e-12 relative (FP64 small products in a different
summation order), and full(C) = full(A) full(B) within 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _blocks(h, orc):
    out = []
    for x in orc.iter_nodes(h):
        if x.leafnode:
            out += [x.D, x.U, x.V]
        else:
            out += [x.B12, x.B21, x.R1, x.R2, x.W1, x.W2]
    return out


@pytest.mark.parametrize("n,ls,ka,kb", [(700, 64, 8, 11), (1001, 62, 12, 5), (2048, 128, 16, 16), (60, 64, 5, 7),
                                        (513, 64, 0, 6)])
def test_hssmul_matches_oracle(pkg, orc, n, ls, ka, kb):
    rng = np.random.default_rng(n + ka)
    A = orc.synthetic_hss(n, ls, ka, rng)
    B = orc.synthetic_hss(n, ls, kb, rng)
    Co = orc.hssmul(A, B)
    C = unpack_like(pkg, orc, pkg.hssmul(pkg.HssMatrix.from_tree(A), pkg.HssMatrix.from_tree(B)))
    assert rel(orc.full(C), orc.full(A) @ orc.full(B)) <= 1e-12
    gb, ob = _blocks(C, orc), _blocks(Co, orc)
    assert len(gb) == len(ob)
    for g, o in zip(gb, ob):
        assert g.shape == o.shape
        assert np.linalg.norm(g - o) <= 1e-12 * max(np.linalg.norm(o), 1.0)


def unpack_like(pkg, orc, h):
    """The package HssMatrix as an oracle tree (same fields)."""
    from conftest import unpack_tree
    table, packed = pkg.pack(h)
    return unpack_tree(table, packed, orc)


def test_hssmul_product_operator(pkg, orc):
    """A * B through the reference operator: (A * B) x = A (B x)."""
    rng = np.random.default_rng(21)
    A = pkg.HssMatrix.from_tree(orc.synthetic_hss(3000, 128, 24, rng))
    B = pkg.HssMatrix.from_tree(orc.synthetic_hss(3000, 128, 20, rng))
    C = A * B
    x = rng.standard_normal((3000, 3))
    assert rel(pkg.matmul(C, x), pkg.matmul(A, pkg.matmul(B, x))) <= 1e-12


def test_hssmul_rejects_mismatched_trees(pkg, orc):
    rng = np.random.default_rng(2)
    A = pkg.HssMatrix.from_tree(orc.synthetic_hss(700, 64, 8, rng))
    B = pkg.HssMatrix.from_tree(orc.synthetic_hss(700, 128, 8, rng))
    with pytest.raises(ValueError):
        pkg.hssmul(A, B)
