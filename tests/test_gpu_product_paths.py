"""GPU: the persistent product (one cooperative launch per product) against the
level-by-level product and the CPU oracle.

Tolerances: FP64 products 1e-12 relative (2-norm) against the oracle and 1e-13
between the two GPU paths (same arithmetic, different summation order); the
persistent product is deterministic, so repeated calls agree bit for bit.  The
double-float refinement residual of an FP32 factorization must bring the true
(oracle) residual to 1e-10 with either product.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

pytestmark = pytest.mark.gpu

HSS_OPT_LEVEL_PRODUCT = 3


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _tree(pkg, orc, name):
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    return g, h, pkg.HssMatrix.from_tree(h)


def _both(lib, fn):
    """fn() with the persistent product (default) and with the level product."""
    out = []
    for level in (0, 1):
        assert lib.hss_set_option(HSS_OPT_LEVEL_PRODUCT, level) == 0
        try:
            out.append(fn())
        finally:
            lib.hss_set_option(HSS_OPT_LEVEL_PRODUCT, 0)
    return out


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("r", [1, 3, 8, 13, 40])
def test_products_agree(pkg, lib, orc, name, r):
    g, h, A = _tree(pkg, orc, name)
    n = g["x"].shape[0]
    x = np.random.default_rng(r).standard_normal((n, r))
    ref = orc.matmul(h, x)
    p, l = _both(lib, lambda: pkg.matmul(A, x))
    assert rel(p, ref) <= 1e-12
    assert rel(p, l) <= 1e-13


@pytest.mark.parametrize("name", ["synthetic_uneven", "synthetic_unbalanced", "single_leaf"])
def test_alpha_beta_agree(pkg, lib, orc, name):
    """mul!(C, hssA, B, alpha, beta) (src/matmul.jl:18-28) on both paths."""
    g, h, A = _tree(pkg, orc, name)
    rng = np.random.default_rng(5)
    x = rng.standard_normal((g["x"].shape[0], 9))
    C0 = np.asfortranarray(rng.standard_normal((g["y"].shape[0], 9)))
    ref = orc.matmul(h, x, 0.5, -2.0, C0)

    def run():
        C = C0.copy(order="F")
        pkg.mul(C, A, x, 0.5, -2.0)
        return C

    p, l = _both(lib, run)
    assert rel(p, ref) <= 1e-12 and rel(p, l) <= 1e-13


def test_repeated_calls_bitwise(pkg, lib, orc):
    """Launch state resets itself: ten products in a row give identical bits, and
    each product is one kernel launch."""
    g, h, A = _tree(pkg, orc, "synthetic_perfect")
    dev = A.device()
    x = np.random.default_rng(0).standard_normal((g["x"].shape[0], 5))
    first = dev.matmul_host(x)
    c0 = lib.hss_launch_counter()
    for _ in range(10):
        assert np.array_equal(dev.matmul_host(x), first)
    assert lib.hss_launch_counter() - c0 == 10
    assert rel(first, orc.matmul(h, x)) <= 1e-12


def test_forest_agrees(pkg, lib, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    trees = [orc.synthetic_hss(n, ls, k, rng) for n, ls, k in
             [(1152, 64, 48), (640, 128, 20), (2001, 64, 16), (129, 64, 8), (64, 64, 8)]]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    rs = [1, 4, 0, 11, 3]
    xs = [rng.standard_normal((t.size()[1], r)) for t, r in zip(trees, rs)]

    def run():
        dX = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in xs]
        dY = [torch.zeros((x.shape[1], t.size()[0]), dtype=torch.float64, device="cuda") for x, t in zip(xs, trees)]
        dev.matmul_batch_device(dX, [x.shape[0] for x in xs], rs, dY, [t.size()[0] for t in trees])
        torch.cuda.synchronize()
        return [y.cpu().numpy().T for y in dY]

    p, l = _both(lib, run)
    for t, x, a, b in zip(trees, xs, p, l):
        if x.shape[1] == 0:
            continue
        ref = orc.matmul(t, x)
        assert rel(a, ref) <= 1e-12 and rel(a, b) <= 1e-13


@pytest.mark.parametrize("name", ["synthetic_perfect", "synthetic_uneven", "cauchy2001_compress"])
def test_refinement_with_both_products(pkg, lib, orc, name):
    g, h, A = _tree(pkg, orc, name)
    Af = orc.full(h)

    def run():
        st = {}
        z = pkg.ldiv(A, g["b"], precision="fp32", tol=1e-10, maxit=30, stats=st)
        return z, st

    for z, st in _both(lib, run):
        assert st["converged"] and st["residual"] <= 1e-10
        res = np.linalg.norm(g["b"] - Af @ z, axis=0) / np.linalg.norm(g["b"], axis=0)
        assert res.max() <= 2e-10


def test_full_size_r1(pkg, lib, orc):
    """n = 65536, leafsize 128, k = 32 at one right-hand side (the bandwidth-bound
    product): oracle agreement and linearity."""
    rng = np.random.default_rng(3)
    A = pkg.synthetic_hss(65536, 128, 32, rng)
    h = orc.synthetic_hss(65536, 128, 32, np.random.default_rng(3))
    x = rng.standard_normal((65536, 1))
    y = rng.standard_normal((65536, 1))
    Ax = pkg.matmul(A, x)
    assert rel(Ax, orc.matmul(h, x)) <= 1e-12
    assert rel(pkg.matmul(A, x - 3 * y), Ax - 3 * pkg.matmul(A, y)) <= 1e-13


def test_autotune_keeps_results(pkg, orc):
    """The autotuner only changes which kernels run: refined solves before and
    after tuning agree with the oracle, on a forest with uneven sizes and ranks."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    trees = [orc.synthetic_hss(n, ls, k, rng) for n, ls, k in [(2048, 128, 32), (1536, 128, 48), (640, 128, 20)]]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    F = dev.ulvfactor("fp32")
    rs = [3, 8, 5]
    bs = [rng.standard_normal((t.size()[0], r)) for t, r in zip(trees, rs)]
    dB = [torch.from_numpy(np.ascontiguousarray(b.T)).cuda() for b in bs]

    def solve():
        dX = [torch.zeros_like(b) for b in dB]
        F.solve_batch_device(dB, [b.shape[0] for b in bs], rs, dX, [b.shape[0] for b in bs], tol=1e-10, maxit=20)
        torch.cuda.synchronize()
        return [x.cpu().numpy().T for x in dX]

    before = solve()
    tune = F.autotune(8)
    assert len(tune["up"]) > 0 and len(tune["down"]) > 0 and tune["product"] in (0, 1)
    assert all(v in (0, 1) for v in tune["up"] + tune["down"])
    after = solve()
    for t, b, x0, x1 in zip(trees, bs, before, after):
        ref = orc.ulvfactsolve(t, b)
        assert rel(x0, ref) <= 1e-8 and rel(x1, ref) <= 1e-8


def test_graph_replay_matches(pkg, lib, orc):
    """HSS_OPT_GRAPHS: factorizations and solve passes on a non-default stream are
    captured on their second identical call and replayed afterwards; every call
    gives the same solution as the eager launches.  From the second call the
    whole refinement loop is one graph whose convergence check runs on the
    device: the eager launches plus one check kernel per residual."""
    torch = pytest.importorskip("torch")
    HSS_OPT_GRAPHS = 4
    rng = np.random.default_rng(12)
    trees = [orc.synthetic_hss(n, 128, k, rng) for n, k in [(2048, 32), (1024, 16)]]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    rs = [4, 2]
    bs = [rng.standard_normal((t.size()[0], r)) for t, r in zip(trees, rs)]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        dB = [torch.from_numpy(np.ascontiguousarray(b.T)).cuda() for b in bs]
    F = dev.ulvfactor("fp32", stream=stream)

    def run():
        with torch.cuda.stream(stream):
            dX = [torch.zeros_like(b) for b in dB]
        c0 = lib.hss_launch_counter()
        F.refactor(stream=stream)
        st = F.solve_batch_device(dB, [b.shape[0] for b in bs], rs, dX, [b.shape[0] for b in bs], tol=1e-10,
                                  maxit=20, stream=stream)
        stream.synchronize()
        return [x.cpu().numpy().T for x in dX], lib.hss_launch_counter() - c0, st.iterations

    run()   # the first solve also prepares the plan's tensor-core slices (once)
    eager, n_eager, it_eager = run()
    assert lib.hss_set_option(HSS_OPT_GRAPHS, 1) == 0
    try:
        outs = [run() for _ in range(4)]   # eager (key seen), capture, replay, replay
    finally:
        lib.hss_set_option(HSS_OPT_GRAPHS, 0)
    for i, (xs, n, it) in enumerate(outs):
        assert it == it_eager
        assert n == (n_eager if i == 0 else n_eager + it + 1)
        for t, b, x, x0 in zip(trees, bs, xs, eager):
            assert rel(x, x0) <= 1e-12
            assert rel(x, orc.ulvfactsolve(t, b)) <= 1e-8


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_fused_factor_solve_matches(pkg, lib, prec):
    """hss_ulvfactsolve (the factorization with the first solve's upward sweep one
    level behind it on a second stream) gives the solution of hss_ulvrefactor +
    hss_ulvsolve: eagerly, on the default stream, and captured and replayed as a
    CUDA graph (HSS_OPT_GRAPHS) on a non-default stream; the host entry point
    hss_ulvfactsolve_host (fused from its second call) agrees too.  Bit for bit
    in FP64 (no refinement); in FP32 + refinement to 1e-9 relative, the
    refinement's own accuracy (the column norms that scale each pass are summed
    with atomics in any order, so the FP32 passes may round differently)."""
    torch = pytest.importorskip("torch")
    n, r = 8192, 8
    A = pkg.synthetic_hss(n, 128, 32, np.random.default_rng(3))
    dev = A.device()
    F = dev.ulvfactor(prec)
    tol = 1e-10 if prec == "fp32" else 0.0
    B = torch.randn((r, n), dtype=torch.float64, device="cuda")

    def same(a, b):
        if prec == "fp64":
            return bool(torch.equal(a, b))
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) <= 1e-9

    X1 = torch.empty_like(B)
    F.refactor()
    st = F.solve_device(B, n, r, X1, n, tol=tol, maxit=20)
    it1 = st.iterations
    torch.cuda.synchronize()
    X2 = torch.empty_like(B)
    st = F.factsolve_device(B, n, r, X2, n, tol=tol, maxit=20)
    torch.cuda.synchronize()
    assert same(X2, X1) and st.converged
    stream = torch.cuda.Stream()
    assert lib.hss_set_option(pkg._lib.HSS_OPT_GRAPHS, 1) == 0
    try:
        for _ in range(3):   # eager, captured, replayed
            X3 = torch.zeros_like(B)
            torch.cuda.synchronize()
            st = F.factsolve_device(B, n, r, X3, n, tol=tol, maxit=20, stream=stream)
            stream.synchronize()
            assert same(X3, X1) and st.converged
    finally:
        lib.hss_set_option(pkg._lib.HSS_OPT_GRAPHS, 0)
    Bh = B.cpu().numpy().T.copy(order="F")
    x0 = pkg.ldiv(A, Bh, precision=prec, tol=tol if tol > 0 else None)
    x1 = pkg.ldiv(A, Bh, precision=prec, tol=tol if tol > 0 else None)   # second call: fused
    assert same(torch.from_numpy(x1.T.copy()).cuda(), torch.from_numpy(x0.T.copy()).cuda())
    assert same(torch.from_numpy(x1.T.copy()).cuda(), X1)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_device_refinement_loop(pkg, lib, prec):
    """The refinement loop recorded as one graph (HSS_OPT_GRAPHS, non-default
    stream): the convergence check on the device ends the loop at the same step
    as the host loop, with the same residual to rounding, in FP32 (double-float
    residual) and in FP64 (FP64 residual, tol > 0); with an unreachable tolerance
    (0 in FP32; 1e-300 in FP64, where tol = 0 means no refinement) the loop stops
    after maxit steps, reports no convergence with maxit iterations, and the
    next call on the same factorization still solves."""
    torch = pytest.importorskip("torch")
    n, r = 4096, 4
    A = pkg.synthetic_hss(n, 128, 24, np.random.default_rng(21))
    F = A.device().ulvfactor(prec)
    B = torch.randn((r, n), dtype=torch.float64, device="cuda")
    tol = 1e-10 if prec == "fp32" else 1e-13
    never = 0.0 if prec == "fp32" else 1e-300
    stream = torch.cuda.Stream()

    def solve(tol, maxit):
        X = torch.zeros_like(B)
        torch.cuda.synchronize()
        try:
            st = F.solve_device(B, n, r, X, n, tol=tol, maxit=maxit, stream=stream)
            ok = True
        except pkg._lib.NoConvergence:
            st, ok = F.stats, False
        stream.synchronize()
        return X, ok, st.iterations, st.residual, st.converged

    X0, ok0, it0, res0, _ = solve(tol, 20)   # host loop (graphs off)
    assert ok0 and res0 <= tol
    Xs, ok, its, res_s, conv_s = solve(never, 3)
    assert not ok and its == 3 and conv_s == 0
    assert lib.hss_set_option(pkg._lib.HSS_OPT_GRAPHS, 1) == 0
    try:
        for _ in range(3):   # host loop (key seen), recorded, replayed
            X, ok, it, res, conv = solve(tol, 20)
            assert ok and conv == 1 and it == it0 and res <= tol
            assert abs(res - res0) <= 0.5 * res0 + 1e-300
            assert float(torch.linalg.norm(X - X0) / torch.linalg.norm(X0)) <= 1e-9
        for _ in range(3):   # unreachable tolerance: bounded by maxit on the device
            X, ok, it, res, conv = solve(never, 3)
            assert not ok and it == 3 and conv == 0 and np.isfinite(res)
            assert float(torch.linalg.norm(X - X0) / torch.linalg.norm(X0)) <= 1e-9
        X, ok, it, res, conv = solve(tol, 20)
        assert ok and it == it0
    finally:
        lib.hss_set_option(pkg._lib.HSS_OPT_GRAPHS, 0)


def test_trace_per_level_times(pkg, lib):
    """hss_trace_times: one device time per traced launch, in launch order, for
    every level of an upward solve (the tree's 7 levels at n = 8192, leafsize
    128) and of the factorization's merges; their sum is the summed time
    hss_trace_end reports for the same launches."""
    torch = pytest.importorskip("torch")
    from hssmatrices_gb300 import linalg as L
    n, r = 8192, 4
    A = pkg.synthetic_hss(n, 128, 16, np.random.default_rng(8))
    F = A.device().ulvfactor("fp32")
    B = torch.randn((r, n), dtype=torch.float64, device="cuda")
    X = torch.empty_like(B)
    F.solve_device(B, n, r, X, n, tol=-1.0)   # warm-up
    torch.cuda.synchronize()
    L.trace_begin("solve_up")
    F.solve_device(B, n, r, X, n, tol=-1.0)
    t = L.trace_times()
    assert len(t) == 7 and all(v > 0 for v in t)
    L.trace_begin("factor_merge")
    F.refactor()
    t = L.trace_times()
    L.trace_begin("factor_merge")
    F.refactor()
    total, count = L.trace_end()
    assert len(t) == count == 6 and all(v > 0 for v in t)
    assert abs(sum(t) - total) <= 0.5 * total


def test_host_solve_graph_replay_new_rhs(pkg, lib):
    """hss_ulvfactsolve_host with graph replay on: the right-hand sides are
    copied on a second stream while the factorization starts (an external event
    the recorded graph waits on), so every call with new right-hand sides (host
    loop, recorded, replayed) must solve for those, to the refinement's
    tolerance, and agree with the call made without graphs."""
    n, r = 8192, 4
    A = pkg.synthetic_hss(n, 128, 32, np.random.default_rng(13))
    rng = np.random.default_rng(14)
    Bs = [np.asfortranarray(rng.standard_normal((n, r))) for _ in range(5)]
    x_plain = [pkg.ldiv(A, b, precision="fp32", tol=1e-10) for b in Bs[:2]]
    assert lib.hss_set_option(pkg._lib.HSS_OPT_GRAPHS, 1) == 0
    try:
        xs = [pkg.ldiv(A, b, precision="fp32", tol=1e-10) for b in Bs]
    finally:
        lib.hss_set_option(pkg._lib.HSS_OPT_GRAPHS, 0)
    for b, x in zip(Bs, xs):
        res = np.linalg.norm(b - pkg.matmul(A, x), axis=0) / np.linalg.norm(b, axis=0)
        assert res.max() <= 1e-10, res
    for x0, x1 in zip(x_plain, xs):
        assert np.linalg.norm(x1 - x0) / np.linalg.norm(x0) <= 1e-9
