"""GPU randomized compression (src/compression.jl:278-444) against the oracle.

The test matrices are drawn on the host by the same seeded NumPy generator for
the GPU path and the oracle, so both see identical Omega.  Rank decisions use
the same pivoting rule (xLAQP2), so ranks and selected indices are expected to
agree node by node; the approximation is checked as the reference's suite does
(test/runtests.jl:36-40: error <= c * tol, c = 50).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C_SAFETY = 50.0


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _host(t):
    """Column-major device tensor (cols, rows) -> numpy (rows, cols)."""
    return t.cpu().numpy().T


def _oracle_ranks(orc, h):
    """(column, row) generator ranks in pre-order, 0 for the root."""
    out = []

    def visit(x, root):
        out.append((0, 0) if root else orc.gensize(x))
        if not x.leafnode:
            visit(x.A11, False)
            visit(x.A22, False)

    visit(h, True)
    return np.array(out, dtype=np.int64)


@pytest.mark.parametrize("m,n,s", [(1000, 777, 13), (300, 20000, 37), (20000, 100, 5), (64, 64, 32), (1, 1, 1)])
def test_sample_product(pkg, m, n, s):
    """S = A * Omega and A' * Omega (:290-291), with the split-K and direct paths."""
    comp = pkg.compression
    rng = np.random.default_rng(m + n + s)
    A = rng.standard_normal((m, n))
    Ad = comp.DenseDevice(A)
    X = rng.standard_normal((n, s))
    Y = rng.standard_normal((m, s))
    assert rel(_host(comp.sample(Ad, comp._cols_to_device(X))), A @ X) <= 1e-13
    assert rel(_host(comp.sample(Ad, comp._cols_to_device(Y), trans=True)), A.T @ Y) <= 1e-13
    # alpha, beta
    C0 = rng.standard_normal((m, s))
    out = comp._cols_to_device(C0)
    comp.sample(Ad, comp._cols_to_device(X), out=out, alpha=2.0, beta=-0.5)
    assert rel(_host(out), 2.0 * (A @ X) - 0.5 * C0) <= 1e-13
    # sum of squares
    assert abs(comp.sumsq(out) - np.sum(_host(out) ** 2)) <= 1e-12 * np.sum(_host(out) ** 2)


@pytest.mark.parametrize("m,n,s", [(1000, 777, 13), (300, 20000, 37), (20000, 100, 5), (1, 1, 1)])
def test_sample_product_double_float(pkg, m, n, s):
    """The mixed-precision sampling (HSS_OPT_SAMPLE_DF): double-float products,
    ~2^-47 relative per operation.  Tolerance: normwise 5e-12 on N(0,1) data
    (the random-walk error sqrt(K) 2^-47 is ~1e-12 at K = 20000), and the
    dot-product bound 1e-11 |A| |X| entrywise on entries spread over 40
    decades with zeros."""
    comp = pkg.compression
    rng = np.random.default_rng(7 + m + n + s)
    A = rng.standard_normal((m, n))
    A.flat[3::7] = 0.0
    Ad = comp.DenseDevice(A)
    X = rng.standard_normal((n, s))
    Y = rng.standard_normal((m, s))
    with comp._SamplePrecision(Ad, "df") as sp:
        assert sp.df
        assert rel(_host(comp.sample(Ad, comp._cols_to_device(X))), A @ X) <= 5e-12
        assert rel(_host(comp.sample(Ad, comp._cols_to_device(Y), trans=True)), A.T @ Y) <= 5e-12
        C0 = rng.standard_normal((m, s))
        out = comp._cols_to_device(C0)
        comp.sample(Ad, comp._cols_to_device(X), out=out, alpha=2.0, beta=-0.5)
        assert rel(_host(out), 2.0 * (A @ X) - 0.5 * C0) <= 5e-12
        # magnitudes from 1e-20 to 1e20 (all within float's exponent range)
        W = A * 10.0 ** rng.uniform(-20, 20, size=A.shape)
        Wd = comp.DenseDevice(W)
        got = _host(comp.sample(Wd, comp._cols_to_device(X)))
        assert np.all(np.abs(got - W @ X) <= 1e-11 * (np.abs(W) @ np.abs(X)) + 1e-300)
    # the option is off again: FP64 products
    assert rel(_host(comp.sample(Ad, comp._cols_to_device(X))), A @ X) <= 1e-13


@pytest.mark.parametrize("trans", [False, True])
def test_cluster_sample_keeps_offdiagonal_accuracy(pkg, orc, trans):
    """hss_rc_sample with double-float sampling: the leaf blocks' part in FP64,
    the rest in double-float, so the corrected sample S - D X (what the tree
    pass uses) has double-float accuracy relative to itself although the
    near-diagonal entries of the kernel matrix dominate S.  Tolerance 5e-12
    relative to the corrected sample; with FP64 sampling the same call is the
    plain product (1e-13)."""
    comp = pkg.compression
    n = 3000
    A = orc.cauchy_matrix(n)
    cl = pkg.bisection_cluster(n, 64)
    c = comp.Compressor(cl, cl)
    Ad = comp.DenseDevice(A)
    X = np.random.default_rng(11).standard_normal((n, 20))
    mask = np.zeros((n, n), dtype=bool)
    for row in c.table:
        if row[0] < 0:
            mask[row[2]:row[3], row[4]:row[5]] = True
    Aop = A.T if trans else A
    D = np.where(mask.T if trans else mask, Aop, 0.0)
    off = (Aop - D) @ X
    with comp._SamplePrecision(Ad, "df"):
        S = _host(c.sample(Ad, comp._cols_to_device(X), trans=trans))
    assert rel(S - D @ X, off) <= 5e-12
    S64 = _host(c.sample(Ad, comp._cols_to_device(X), trans=trans))
    assert rel(S64, Aop @ X) <= 1e-13


def test_sample_precision_falls_back_outside_float_range(pkg):
    comp = pkg.compression
    A = np.full((40, 30), 1e200)
    assert not comp._SamplePrecision(comp.DenseDevice(A), "df").df
    with pytest.raises(ValueError):
        comp._SamplePrecision(comp.DenseDevice(A), "fp16")


def test_randcompress_adaptive_double_float_sampling(pkg, orc):
    """The reference suite's compression (runtests.jl:36-40) with double-float
    sample products: same test rounds and sample count as the oracle on the
    same draws, error within c * tol."""
    A = orc.runtests_matrix(2001)
    tol = 1e-6
    st_g, st_o = {}, {}
    rcl = pkg.bisection_cluster(2001, 50)
    h = pkg.randcompress_adaptive(A, rcl, rcl, kest=10, atol=tol, rtol=tol, noversampling=5, stepsize=10,
                                  rng=np.random.default_rng(1), stats=st_g, sample_precision="df")
    ocl = orc.bisection_cluster(2001, 50)
    orc.randcompress_adaptive(A, ocl, ocl, 10, tol, tol, 5, 10, rng=np.random.default_rng(1), stats=st_o)
    assert st_g["rounds"] == st_o["rounds"] and st_g["k"] == st_o["k"]
    err = np.linalg.norm(A - orc.full(h))
    assert err / np.linalg.norm(A) <= C_SAFETY * tol or err <= C_SAFETY * tol


def test_sample_rejects_bad_shapes(pkg):
    comp = pkg.compression
    Ad = comp.DenseDevice(np.ones((10, 7)))
    with pytest.raises(ValueError):
        comp.sample(Ad, comp._cols_to_device(np.ones((10, 2))))


def _same_sample_case(pkg, orc, A, leafsize, s, tol, seed):
    rcl = orc.bisection_cluster(A.shape[0], leafsize)
    ccl = orc.bisection_cluster(A.shape[1], leafsize)
    rng = np.random.default_rng(seed)
    Ocol = rng.standard_normal((A.shape[1], s))
    Orow = rng.standard_normal((A.shape[0], s))
    h_orc = orc._randcompress(orc.hss_blkdiag(A, rcl, ccl), A, A @ Ocol, A.T @ Orow, Ocol, Orow, 0, 0, tol, tol,
                              rootnode=True)[0]
    comp = pkg.compression
    prc = pkg.bisection_cluster(A.shape[0], leafsize)
    pcc = pkg.bisection_cluster(A.shape[1], leafsize)
    Ad = comp.DenseDevice(A)
    c = comp.Compressor(prc, pcc)
    dO, dR = comp._cols_to_device(Ocol), comp._cols_to_device(Orow)
    dev = c.compress(Ad, comp.sample(Ad, dO), comp.sample(Ad, dR, trans=True), dO, dR, tol, tol)
    return h_orc, dev, c


@pytest.mark.parametrize("case", ["runtests", "cauchy"])
def test_compress_same_samples_matches_oracle(pkg, orc, case):
    """`_randcompress!` on identical samples: ranks node by node, selected
    indices through the generators, and the approximation error."""
    if case == "runtests":
        A, leafsize, s, tol = orc.runtests_matrix(2001), 50, 30, 1e-6
    else:
        A, leafsize, s, tol = orc.cauchy_matrix(2048), 128, 40, 1e-9
    h_orc, dev, c = _same_sample_case(pkg, orc, A, leafsize, s, tol, seed=7)
    ro = _oracle_ranks(orc, h_orc)
    rg = c.ranks()
    agree = np.mean(np.all(ro == rg, axis=1))
    assert agree >= 0.95, f"ranks agree at {agree:.3f} of the nodes"
    h = dev.to_host()
    Ag = orc.full(h)
    Ao = orc.full(h_orc)
    err = np.linalg.norm(A - Ag)
    assert err / np.linalg.norm(A) <= C_SAFETY * tol or err <= C_SAFETY * tol
    # the two approximations are close to each other as well
    assert rel(Ag, Ao) <= C_SAFETY * tol


def test_compress_exact_rank_synthetic(pkg, orc):
    """A dense matrix with HSS rank exactly k: every rank is k, and the
    compressed matrix reproduces A to rounding."""
    rng = np.random.default_rng(3)
    k = 8
    h0 = orc.synthetic_hss(1024, 128, k, rng)
    A = orc.full(h0)
    h_orc, dev, c = _same_sample_case(pkg, orc, A, 128, k + 22, 1e-9, seed=9)
    rg = c.ranks()
    assert np.all(rg[1:] == k)
    assert np.all(_oracle_ranks(orc, h_orc)[1:] == k)
    assert rel(orc.full(dev.to_host()), A) <= 1e-11


def test_randcompress_adaptive_reference_suite(pkg, orc):
    """runtests.jl:36-40 with the suite's options (leafsize 50, tol 1e-6,
    noversampling 5, stepsize 10): same test-round count as the oracle on the
    same draws, error within c * tol."""
    A = orc.runtests_matrix(2001)
    tol = 1e-6
    st_g, st_o = {}, {}
    rcl = pkg.bisection_cluster(2001, 50)
    h = pkg.randcompress_adaptive(A, rcl, rcl, kest=10, atol=tol, rtol=tol, noversampling=5, stepsize=10,
                                  rng=np.random.default_rng(1), stats=st_g)
    ocl = orc.bisection_cluster(2001, 50)
    ho = orc.randcompress_adaptive(A, ocl, ocl, 10, tol, tol, 5, 10, rng=np.random.default_rng(1), stats=st_o)
    assert st_g["rounds"] == st_o["rounds"] and st_g["k"] == st_o["k"]
    Ah = orc.full(h)
    err = np.linalg.norm(A - Ah)
    assert err / np.linalg.norm(A) <= C_SAFETY * tol or err <= C_SAFETY * tol
    assert abs(pkg.hssrank(h) - orc.hssrank(ho)) <= 2
    # the compressed matrix runs the hot path: product and ULV solve
    x = np.random.default_rng(2).standard_normal((2001, 5))
    assert rel(pkg.matmul(h, x), A @ x) <= C_SAFETY * tol
    b = A @ x
    xs = pkg.ldiv(h, b)
    assert rel(xs, np.linalg.solve(A, b)) <= C_SAFETY * tol * 10


def test_randcompress_identity(pkg, orc):
    """randcompress(IdOp, ccl, ccl, 0) (runtests.jl:65-66): every sample is
    annihilated by the leaf correction, all ranks are 0, and the result is I."""
    n = 500
    ccl = pkg.bisection_cluster(n, 50)
    h = pkg.randcompress(np.eye(n), ccl, ccl, 0, noversampling=5)
    assert pkg.hssrank(h) == 0
    assert np.array_equal(orc.full(h), np.eye(n))


def test_randcompress_device_handle(pkg, orc):
    """device=True returns the resident handle; its product equals the host
    object's, and the Cauchy kernel at 1e-9 compresses within tolerance."""
    A = orc.cauchy_matrix(3000)
    cl = pkg.bisection_cluster(3000, 128)
    dev = pkg.randcompress_adaptive(A, cl, cl, kest=10, atol=1e-9, rtol=1e-9, rng=np.random.default_rng(4),
                                    device=True)
    h = dev.to_host()
    x = np.random.default_rng(5).standard_normal((3000, 3))
    y1 = dev.matmul_host(x)
    y2 = pkg.matmul(h, x)
    assert np.array_equal(y1, y2)
    err = np.linalg.norm(A - orc.full(h))
    assert err / np.linalg.norm(A) <= C_SAFETY * 1e-9


def test_compress_incompatible_clusters(pkg):
    a = pkg.bisection_cluster(100, 10)
    b = pkg.bisection_cluster(100, 30)
    with pytest.raises(ValueError):
        pkg.Compressor(a, b)
