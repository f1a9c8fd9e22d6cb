"""GPU entry extraction: getindex / full (src/hssmatrix.jl:102-153, 270-305)
against the oracle's restatement (oracle.getindex, oracle.full).

FP64: every entry is a sum of at most (levels x rank) products of generator
entries, so the device result agrees with the oracle within 1e-13 relative
(max-norm over the whole extracted block, relative to its largest entry)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

pytestmark = pytest.mark.gpu


def close(a, b, tol=1e-13):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    return np.max(np.abs(a - b), initial=0.0) <= tol * max(np.max(np.abs(b), initial=0.0), 1e-300)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_full_matches_oracle(pkg, orc, name):
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    A = pkg.HssMatrix.from_tree(h)
    assert close(pkg.full(A), orc.full(h))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_getindex_random_lists(pkg, orc, seed):
    """Unsorted index lists with repeats (the sortperm / invperm of :110-113)."""
    rng = np.random.default_rng(seed)
    n, ls, k = [(1500, 64, 20), (3000, 128, 32), (777, 50, 9)][seed]
    h = orc.synthetic_hss(n, ls, k, rng)
    A = pkg.HssMatrix.from_tree(h)
    i = rng.integers(0, n, 300)
    j = rng.integers(0, n, 250)
    assert close(pkg.getindex(A, i, j), orc.getindex(h, i, j))
    # a contiguous range crossing several leaves, and single entries
    assert close(pkg.getindex(A, slice(100, 700), slice(650, 900)), orc.full(h)[100:700, 650:900])
    Af = orc.full(h)
    for (a, b) in [(0, 0), (n - 1, 0), (17, n - 2), (n // 2, n // 2 - 1)]:
        assert abs(A[a, b] - Af[a, b]) <= 1e-13 * np.abs(Af).max()
    assert close(A[5, :], Af[5, :]) and close(A[:, 9], Af[:, 9])


def test_getindex_empty_and_errors(pkg, orc):
    h = orc.synthetic_hss(400, 64, 8, np.random.default_rng(4))
    A = pkg.HssMatrix.from_tree(h)
    assert pkg.getindex(A, [], [1, 2]).shape == (0, 2)
    assert pkg.getindex(A, [3], []).shape == (1, 0)
    with pytest.raises(IndexError):
        pkg.getindex(A, [400], [0])
    dev = A.device()
    with pytest.raises(ValueError):   # the C ABI's own check (HSS_ERR_BAD_DIMS)
        dev.getindex(np.array([0, -1]), np.array([0]))


def test_full_single_leaf_and_uneven(pkg, orc):
    for n, ls, k in [(60, 64, 5), (1001, 62, 12)]:
        h = orc.synthetic_hss(n, ls, k, np.random.default_rng(n))
        A = pkg.HssMatrix.from_tree(h)
        assert close(pkg.full(A), orc.full(h))


def test_full_forest_rejected(pkg, orc):
    rng = np.random.default_rng(6)
    trees = [orc.synthetic_hss(300, 64, 8, rng), orc.synthetic_hss(200, 64, 8, rng)]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    with pytest.raises(ValueError):
        dev.full()
