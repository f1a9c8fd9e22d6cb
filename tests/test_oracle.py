"""The oracle against the reference's own tests and the golden fixtures (CPU)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

C_SAFETY = 50.0   # test/runtests.jl:27
TOL = 1e-6        # test/runtests.jl:28


def _ok(err_rel, err_abs):
    # test/runtests.jl:38: rel <= c*rtol or abs <= c*atol
    return err_rel <= C_SAFETY * TOL or err_abs <= C_SAFETY * TOL


@pytest.mark.parametrize("leafsize", [50, 64])
def test_runtests_compression_and_arithmetic(orc, leafsize):
    """test/runtests.jl:16-67 for T = Float64 (leafsize 50 is what the suite runs with
    after its options testset, :8)."""
    A = orc.runtests_matrix(2001)
    rng = np.random.default_rng(1)
    rcl = orc.bisection_cluster(2001, leafsize)
    ccl = orc.bisection_cluster(2001, leafsize)
    h = orc.compress(A, rcl, ccl, TOL, TOL)
    E = A - orc.full(h)
    assert _ok(np.linalg.norm(E) / np.linalg.norm(A), np.linalg.norm(E))
    hb = orc.randcompress_adaptive(A, rcl, ccl, 10, TOL, TOL, 5, 10, rng=rng)
    E = A - orc.full(hb)
    assert _ok(np.linalg.norm(E) / np.linalg.norm(A), np.linalg.norm(E))
    # arithmetic (:59-67): adjoint, matvec with 5 rhs, ULV solve with 5 rhs
    E = A.T - orc.full(orc.adjoint(h))
    assert _ok(np.linalg.norm(E) / np.linalg.norm(A), np.linalg.norm(E))
    x = rng.standard_normal((2001, 5))
    E = A @ x - orc.matmul(h, x)
    assert _ok(np.linalg.norm(E) / np.linalg.norm(A @ x), np.linalg.norm(E))
    rhs = rng.standard_normal((2001, 5))
    x0 = np.linalg.solve(A, rhs)
    xs = orc.ulvfactsolve(h, rhs)
    assert _ok(np.linalg.norm(x0 - xs) / np.linalg.norm(x0), np.linalg.norm(x0 - xs))


@pytest.mark.parametrize("leafsize", [50, 64])
def test_runtests_hss_division(orc, leafsize):
    """test/runtests.jl:68-77 for T = Float64: hssA \\ hssI and hssI / hssA against
    inv(A), then the same with A11 of both pruned (an unbalanced tree), through
    the restatement of src/ulvdivide.jl."""
    A = orc.runtests_matrix(2001)
    ccl = orc.bisection_cluster(2001, leafsize)
    h = orc.compress(A, ccl, ccl, TOL, TOL)
    hI = orc.hss_blkdiag(np.eye(2001), ccl, ccl)
    Ainv = np.linalg.inv(A)

    def check(X):
        E = Ainv - orc.full(X)
        assert _ok(np.linalg.norm(E) / np.linalg.norm(Ainv), np.linalg.norm(E))

    check(orc.ldiv_hss(h, hI, TOL, TOL))
    check(orc.rdiv_hss(hI, h, TOL, TOL))
    h.A11 = orc.prune_leaves(h.A11)
    h.sz1 = h.A11.size()
    hI.A11 = orc.prune_leaves(hI.A11)
    hI.sz1 = hI.A11.size()
    check(orc.ldiv_hss(h, hI, TOL, TOL))
    check(orc.rdiv_hss(hI, h, TOL, TOL))


def test_hss_division_is_exact_division(orc):
    """At a tight tolerance the division equals full(hssA)^-1 full(hssB) to rounding
    (a general B of rank 8 on the same tree)."""
    rng = np.random.default_rng(4)
    hA = orc.synthetic_hss(1000, 64, 10, rng)
    hB = orc.synthetic_hss(1000, 64, 8, rng)
    FA, FB = orc.full(hA), orc.full(hB)
    X = orc.ldiv_hss(hA, hB, 1e-13, 1e-13)
    ref = np.linalg.solve(FA, FB)
    assert np.linalg.norm(ref - orc.full(X)) / np.linalg.norm(ref) < 1e-12
    Y = orc.rdiv_hss(hB, hA, 1e-13, 1e-13)
    ref = FB @ np.linalg.inv(FA)
    assert np.linalg.norm(ref - orc.full(Y)) / np.linalg.norm(ref) < 1e-12


def test_config1_cauchy(orc):
    """Cauchy-type kernel on -1:0.001:1 with leafsize 64 and compress at 1e-6."""
    A = orc.cauchy_matrix(2001)
    cl = orc.bisection_cluster(2001, 64)
    h = orc.compress(A, cl, cl, TOL, TOL)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(2001)
    E = A @ x - orc.matmul(h, x)
    assert _ok(np.linalg.norm(E) / np.linalg.norm(A @ x), np.linalg.norm(E))
    b = rng.standard_normal((2001, 1))
    x0 = np.linalg.solve(A, b)
    xs = orc.ulvfactsolve(h, b)
    assert _ok(np.linalg.norm(x0 - xs) / np.linalg.norm(x0), np.linalg.norm(x0 - xs))


def test_bisection_cluster_known(orc):
    # 10 with leafsize 3: 1:5 | 6:10 -> 1:3, 4:5 | 6:8, 9:10 (split at ceil(len/2))
    assert orc.cluster_leaves(orc.bisection_cluster(10, 3)) == [(1, 3), (4, 5), (6, 8), (9, 10)]
    assert orc.cluster_leaves(orc.bisection_cluster(64, 64)) == [(1, 64)]
    assert orc.cluster_leaves(orc.bisection_cluster(65, 64)) == [(1, 33), (34, 65)]
    leaves = orc.cluster_leaves(orc.bisection_cluster(65536, 128))
    assert len(leaves) == 512 and all(hi - lo + 1 == 128 for lo, hi in leaves)
    with pytest.raises(ValueError):
        orc.bisection_cluster(0, 64)


def test_bisection_cluster_golden(orc, pkg):
    g = load_golden("clusters")
    for key, leaves in g.items():
        n, ls = (int(v) for v in key[1:].split("_ls"))
        got = np.array(orc.cluster_leaves(orc.bisection_cluster(n, ls)), dtype=np.int64)
        assert np.array_equal(got, leaves), key
        # the package's host mirror is bit-exact with the oracle
        t = pkg.bisection_cluster(n, ls)

        def lv(x):
            return [(x.lo, x.hi)] if x.isleaf() else lv(x.left) + lv(x.right)
        assert np.array_equal(np.array(lv(t), dtype=np.int64), leaves), key


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_reproduces_golden(orc, name):
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    y = orc.matmul(h, g["x"])
    assert np.allclose(y, g["y"], rtol=0, atol=1e-13 * np.abs(g["y"]).max())
    z = orc.ulvfactsolve(h, g["b"])
    assert np.linalg.norm(z - g["z"]) <= 1e-12 * np.linalg.norm(g["z"])
    cols = orc.ulv_cols(h)
    flat = np.concatenate([c for c, _mk, _nk in cols])
    assert np.array_equal(flat, g["cols"])
    # dense FP64 LU: the solve error statement
    A = orc.full(h)
    zd = np.linalg.solve(A, g["b"])
    assert np.linalg.norm(z - zd) <= 1e-8 * np.linalg.norm(zd)


def test_oracle_cond_estimate(orc):
    rng = np.random.default_rng(3)
    h = orc.synthetic_hss(600, 64, 12, rng)
    A = orc.full(h)
    est = orc.cond_estimate(h, iters=40)
    assert abs(est - np.linalg.cond(A)) / np.linalg.cond(A) < 0.1


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_getindex_is_full_restricted(orc, name):
    """getindex (src/hssmatrix.jl:108-128: sort, restrict the tree, full,
    unsort) equals full()[i, j] for unsorted index lists with repeats."""
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    m, n = h.size()
    rng = np.random.default_rng(m + n)
    i = rng.integers(0, m, 40)
    j = rng.integers(0, n, 33)
    Af = orc.full(h)
    assert np.allclose(orc.getindex(h, i, j), Af[np.ix_(i, j)], rtol=1e-13, atol=1e-13 * np.abs(Af).max())
    assert orc.getindex(h, [], j).shape == (0, j.size)
