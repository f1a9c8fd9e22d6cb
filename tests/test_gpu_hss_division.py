"""GPU: HSS-valued division hssA \\ hssB and hssB / hssA (src/ulvdivide.jl:13-252,
src/hssmatrix.jl:235-237) by the reference's recursion on the device
(``hss_ldiv`` / ``hss_rdiv``), and the adjoint on the device (``hss_transpose``,
``hss_matmul_t``; src/hssmatrix.jl:165-178, src/matmul.jl:14, :236).

As the reference's own test (test/runtests.jl:68-77): the identity compressed
by randcompress with kest = 0, then A \\ I and I / A against inv(A) within
c rtol (c = 50), also after pruning A11 of both (an unbalanced tree).  At a
tight tolerance the division is compared with the dense solve and with the
oracle's restatement of the same recursion; at n = 65536 through the
size-independent property A (X v) = B v with the device products, with the
device memory in use during the call sampled (the recursion keeps O(n k) per
level, a dense B alone would be 34 GB).
"""
import threading
import time

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
    X = pkg.ldiv(A, I, atol=tol, rtol=tol)
    assert isinstance(X, pkg.HssMatrix)
    assert rel(pkg.full(X), Ainv) <= C * tol
    Y = I / A
    assert rel(pkg.full(Y), Ainv) <= C * tol


def test_ldiv_rdiv_identity_unbalanced(pkg, orc):
    """runtests.jl:75-77: A11 of A and of I pruned, then A \\ I and I / A again."""
    n, tol = 2001, 1e-6
    Ad = orc.runtests_matrix(n)
    cl = orc.bisection_cluster(n, 64)
    ha = orc.compress(Ad, cl, cl, tol, tol)
    hi = orc.hss_blkdiag(np.eye(n), cl, cl)
    ha.A11 = orc.prune_leaves(ha.A11)
    ha.sz1 = ha.A11.size()
    hi.A11 = orc.prune_leaves(hi.A11)
    hi.sz1 = hi.A11.size()
    A, I = pkg.HssMatrix.from_tree(ha), pkg.HssMatrix.from_tree(hi)
    Ainv = np.linalg.inv(Ad)
    assert rel(pkg.full(pkg.ldiv(A, I, atol=tol, rtol=tol)), Ainv) <= C * tol
    assert rel(pkg.full(pkg.rdiv(I, A, atol=tol, rtol=tol)), Ainv) <= C * tol


def test_ldiv_general_matches_dense_and_oracle(pkg, orc):
    """A \\ B and B / A for a second HSS matrix B on the same tree: at a tight
    tolerance equal to the dense solve to rounding, and to the oracle's
    restatement of the recursion."""
    rng = np.random.default_rng(7)
    ha = orc.synthetic_hss(1536, 128, 16, rng)
    hb = orc.synthetic_hss(1536, 128, 12, rng)
    A, B = pkg.HssMatrix.from_tree(ha), pkg.HssMatrix.from_tree(hb)
    Af, Bf = orc.full(ha), orc.full(hb)
    tol = 1e-13
    X = pkg.hss_ldiv(A, B, atol=tol, rtol=tol)
    Xf = pkg.full(X)
    assert rel(Xf, np.linalg.solve(Af, Bf)) <= 1e-11
    assert rel(Xf, orc.full(orc.ldiv_hss(ha, hb, tol, tol))) <= 1e-11
    Y = pkg.rdiv(B, A, atol=tol, rtol=tol)
    assert rel(pkg.full(Y), np.linalg.solve(Af.T, Bf.T).T) <= 1e-11
    # at the default-like tolerance the result stays within c tol and the ranks stay small
    X9 = pkg.hss_ldiv(A, B, atol=1e-9, rtol=1e-9)
    assert rel(pkg.full(X9), np.linalg.solve(Af, Bf)) <= C * 1e-9
    assert pkg.hssrank(X9) <= 16 + 12 + 16


def test_ldiv_shape_errors(pkg, orc):
    rng = np.random.default_rng(2)
    A = pkg.HssMatrix.from_tree(orc.synthetic_hss(512, 64, 8, rng))
    B = pkg.HssMatrix.from_tree(orc.synthetic_hss(640, 64, 8, rng))
    with pytest.raises(ValueError):
        pkg.hss_ldiv(A, B)
    with pytest.raises(ValueError):
        pkg.rdiv(B, A)


def test_transpose_and_adjoint_products(pkg, orc):
    """hss_transpose equals the adjoint (src/hssmatrix.jl:165-171); the product with
    the adjoint (hss_matmul_t), A * hssB for a dense A (src/matmul.jl:14) and
    B / hssA for a dense B (src/hssmatrix.jl:236) against dense arithmetic."""
    rng = np.random.default_rng(11)
    h = orc.synthetic_hss(1000, 64, 10, rng)
    A = pkg.HssMatrix.from_tree(h)
    Af = orc.full(h)
    At = A.device().transpose().to_host()
    assert rel(pkg.full(At), Af.T) <= 1e-15
    X = rng.standard_normal((3, 1000))
    assert rel(pkg.rmatmul(X, A), X @ Af) <= 1e-13
    assert rel(X @ A, X @ Af) <= 1e-13
    assert rel(X / A, np.linalg.solve(Af.T, X.T).T) <= 1e-11
    import torch
    dB = torch.from_numpy(np.ascontiguousarray(X)).cuda()      # 1000 x 3 column-major
    dC = torch.zeros_like(dB)
    dev = A.device()
    dev.matmul_device(dB, 1000, 3, dC, 1000, alpha=2.0, trans=True)
    assert rel(dC.cpu().numpy().T, 2.0 * Af.T @ X.T) <= 1e-13


def _device_used_sampler():
    """Samples (total - free) device memory every 2 ms until stopped; returns the peak."""
    import torch
    peak = [0]
    stop = threading.Event()

    def run():
        while not stop.is_set():
            free, total = torch.cuda.mem_get_info()
            peak[0] = max(peak[0], total - free)
            time.sleep(0.002)

    th = threading.Thread(target=run, daemon=True)
    th.start()
    return stop, th, peak


def test_ldiv_full_size_memory_and_residual(pkg):
    """n = 65536 (leafsize 128, k = 32): X = A \\ B for an HSS B of rank 16 on the
    same tree.  A (X v) = B v to 1e-8 for random v (device products), and the
    device memory in use during the call stays within 4 GB above what was in
    use before it (a dense B alone is 34 GB)."""
    import torch
    from hssmatrices_gb300 import synthetic as S
    n = 65536
    A = pkg.synthetic_hss(n, 128, 32, np.random.default_rng(3))
    B = S.synthetic_hss(n, 128, 16, np.random.default_rng(4))
    a, b = A.device(), B.device()
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info()
    base = total - free0
    stop, th, peak = _device_used_sampler()
    try:
        X = pkg.hss_ldiv(A, B, atol=1e-10, rtol=1e-10, device=True)
        torch.cuda.synchronize()
    finally:
        stop.set()
        th.join()
    assert peak[0] - base <= 4 * 2**30, (peak[0] - base) / 2**30
    v = torch.randn((4, n), dtype=torch.float64, device="cuda")
    Xv = torch.empty_like(v)
    X.matmul_device(v, n, 4, Xv, n)
    AXv = torch.empty_like(v)
    a.matmul_device(Xv, n, 4, AXv, n)
    Bv = torch.empty_like(v)
    b.matmul_device(v, n, 4, Bv, n)
    err = float((torch.linalg.norm(AXv - Bv, dim=1) / torch.linalg.norm(Bv, dim=1)).max())
    assert err <= 1e-8, err


def test_rectangular_products_and_refused_factorization(pkg, orc):
    """A rectangular HSS matrix (rows and columns on two trees of the same shape)
    is an operand of the products, including the adjoint's; its ULV
    factorization is refused with a dimension error."""
    rng = np.random.default_rng(5)
    m, n = 700, 900
    x, y = np.linspace(-1, 1, m), np.linspace(-1.5, 1.5, n)
    Ad = 1.0 / (2.0 + np.abs(x[:, None] - y[None, :]))
    rcl, ccl = orc.bisection_cluster(m, 64), orc.bisection_cluster(n, 90)
    h = orc.compress(Ad, rcl, ccl, 1e-10, 1e-10)
    A = pkg.HssMatrix.from_tree(h)
    Af = orc.full(h)
    B = rng.standard_normal((n, 3))
    assert rel(A * B, Af @ B) <= 1e-13
    X = rng.standard_normal((2, m))
    assert rel(X @ A, X @ Af) <= 1e-13
    assert rel(pkg.full(A.device().transpose().to_host()), Af.T) <= 1e-15
    with pytest.raises(ValueError):
        A.device().ulvfactor("fp64")
