"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances (FP64 path, relative 2-norm): products 1e-12; ULV solves 1e-12 on the
synthetic trees (cond <= 10) and 1e-10 on the Cauchy config-1 fixture (cond ~3e3,
where two correct FP64 solves differ by ~cond * eps).  The FP32 factorization
with FP64 refinement must reach a relative residual of 1e-10.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

pytestmark = pytest.mark.gpu

MV_TOL = 1e-12
SOLVE_TOL = {"cauchy2001_compress": 1e-10}


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _golden(pkg, orc, name):
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    return g, h, pkg.HssMatrix.from_tree(h)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_matvec_golden(pkg, orc, name):
    g, h, A = _golden(pkg, orc, name)
    y = pkg.matmul(A, g["x"])
    assert rel(y, g["y"]) <= MV_TOL
    # single vector (src/matmul.jl:15)
    y1 = pkg.matmul(A, g["x"][:, 0])
    assert y1.ndim == 1 and rel(y1, g["y"][:, 0]) <= MV_TOL


@pytest.mark.parametrize("r", [1, 3, 8, 13, 40])
def test_matvec_rhs_counts(pkg, orc, r):
    rng = np.random.default_rng(r)
    h = orc.synthetic_hss(1001, 64, 16, rng)
    A = pkg.HssMatrix.from_tree(h)
    x = rng.standard_normal((1001, r))
    assert rel(pkg.matmul(A, x), orc.matmul(h, x)) <= MV_TOL


def test_mul_alpha_beta(pkg, orc):
    """mul!(C, hssA, B, alpha, beta) (src/matmul.jl:18-28)."""
    g, h, A = _golden(pkg, orc, "synthetic_uneven")
    rng = np.random.default_rng(11)
    C0 = np.asfortranarray(rng.standard_normal(g["y"].shape))
    C = C0.copy(order="F")
    pkg.mul(C, A, g["x"], 0.5, -2.0)
    ref = orc.matmul(h, g["x"], 0.5, -2.0, C0)
    assert rel(C, ref) <= MV_TOL
    with pytest.raises(ValueError):
        pkg.matmul(A, np.zeros((g["x"].shape[0] + 1, 1)))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ulv_fp64_golden(pkg, orc, name):
    g, h, A = _golden(pkg, orc, name)
    z = pkg.ldiv(A, g["b"])
    assert rel(z, g["z"]) <= SOLVE_TOL.get(name, 1e-12)
    # the error statement against a dense FP64 LU solve
    zd = np.linalg.solve(orc.full(h), g["b"])
    assert rel(z, zd) <= 1e-8


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ulv_fp32_refined(pkg, orc, name):
    g, h, A = _golden(pkg, orc, name)
    st = {}
    z = pkg.ldiv(A, g["b"], precision="fp32", tol=1e-10, maxit=30, stats=st)
    assert st["converged"] and st["residual"] <= 1e-10
    Af = orc.full(h)
    res = np.linalg.norm(g["b"] - Af @ z, axis=0) / np.linalg.norm(g["b"], axis=0)
    assert res.max() <= 2e-10
    assert rel(z, g["z"]) <= 1e-6


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ulv_cols_bit_exact(pkg, orc, name):
    g, h, A = _golden(pkg, orc, name)
    dev = A.device()
    cols = orc.ulv_cols(h)
    for i, (c, mk, nk) in enumerate(cols):
        assert np.array_equal(dev.ulv_cols(i), c), i
        info = dev.node_info(i)
        if i:
            assert (info["mk"], info["nk"]) == (mk, nk)


def test_resident_factor_many_solves(pkg, orc):
    g, h, A = _golden(pkg, orc, "synthetic_uneven")
    for prec in ("fp64", "fp32"):
        F = pkg.ulvfactor(A, prec)
        for seed in range(3):
            b = np.random.default_rng(seed).standard_normal((g["b"].shape[0], 1 + seed))
            z = F.solve(b, tol=1e-10 if prec == "fp32" else 0.0)
            assert rel(z, orc.ulvfactsolve(h, b)) <= (1e-12 if prec == "fp64" else 1e-7)
        F.refactor()
        z = F.solve(g["b"], tol=1e-10 if prec == "fp32" else 0.0)
        assert rel(z, g["z"]) <= (1e-12 if prec == "fp64" else 1e-7)


def test_batched_forest_matches_single(pkg, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    trees = [orc.synthetic_hss(n, ls, k, rng) for n, ls, k in
             [(1152, 64, 48), (640, 128, 20), (2001, 64, 16), (129, 64, 8)]]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    assert dev.ntrees == 4
    xs = [rng.standard_normal((t.size()[1], r)) for t, r in zip(trees, [1, 4, 2, 7])]
    # torch tensors are row-major: store each n x r column-major matrix as an r x n tensor
    dXc = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in xs]
    dY = [torch.zeros_like(x) for x in dXc]
    dev.matmul_batch_device(dXc, [x.shape[0] for x in xs], [x.shape[1] for x in xs], dY,
                            [x.shape[0] for x in xs])
    torch.cuda.synchronize()
    for t, x, y in zip(trees, xs, dY):
        assert rel(y.cpu().numpy().T, orc.matmul(t, x)) <= MV_TOL
    for prec in ("fp64", "fp32"):
        F = dev.ulvfactor(prec)
        dZ = [torch.zeros_like(x) for x in dXc]
        F.solve_batch_device(dXc, [x.shape[0] for x in xs], [x.shape[1] for x in xs], dZ,
                             [x.shape[0] for x in xs], tol=1e-10 if prec == "fp32" else 0.0)
        torch.cuda.synchronize()
        for t, x, z in zip(trees, xs, dZ):
            assert rel(z.cpu().numpy().T, orc.ulvfactsolve(t, x)) <= (1e-12 if prec == "fp64" else 1e-7)


def test_full_size_properties(pkg, orc):
    """n = 65536, leafsize 128, k = 32 (the precision workload): size-independent checks
    plus a direct comparison with the oracle at full size."""
    rng = np.random.default_rng(3)
    A = pkg.synthetic_hss(65536, 128, 32, rng)
    h = orc.synthetic_hss(65536, 128, 32, np.random.default_rng(3))
    x = rng.standard_normal((65536, 2))
    y = rng.standard_normal((65536, 2))
    Ax, Ay = pkg.matmul(A, x), pkg.matmul(A, y)
    assert rel(pkg.matmul(A, x + 2 * y), Ax + 2 * Ay) <= 1e-13
    assert rel(Ax, orc.matmul(h, x)) <= MV_TOL
    b = rng.standard_normal((65536, 2))
    z64 = pkg.ldiv(A, b)
    assert rel(z64, orc.ulvfactsolve(h, b)) <= 1e-12
    res = np.linalg.norm(b - pkg.matmul(A, z64), axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-13
    st = {}
    z32 = pkg.ldiv(A, b, precision="fp32", tol=1e-10, stats=st)
    assert st["converged"] and st["residual"] <= 1e-10
    res = np.linalg.norm(b - pkg.matmul(A, z32), axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-10


def test_singular_root_raises(pkg):
    D = np.zeros((8, 8))
    A = pkg.HssMatrix.leaf(D)
    with pytest.raises(np.linalg.LinAlgError):
        pkg.ldiv(A, np.ones(8))
    z = np.zeros((4, 4))
    l1 = pkg.HssMatrix.leaf(np.zeros((4, 4)), np.eye(4)[:, :2], np.eye(4)[:, :2])
    l2 = pkg.HssMatrix.leaf(np.zeros((4, 4)), np.eye(4)[:, :2], np.eye(4)[:, :2])
    B = pkg.HssMatrix.branch(l1, l2, z[:2, :2], z[:2, :2])
    with pytest.raises(np.linalg.LinAlgError):
        pkg.ldiv(B, np.ones(8))


@pytest.mark.parametrize("name", ["synthetic_perfect", "synthetic_uneven", "synthetic_earlyexit",
                                  "cauchy2001_compress"])
def test_factor_kernels_agree(pkg, lib, orc, name):
    """The on-chip factor kernel and the global-memory one give the same solves."""
    g, h, A = _golden(pkg, orc, name)
    out = {}
    for generic in (0, 1):
        assert lib.hss_set_option(1, generic) == 0
        try:
            for prec in ("fp64", "fp32"):
                F = pkg.ulvfactor(A, prec)
                out[generic, prec] = F.solve(g["b"], tol=-1.0)
        finally:
            lib.hss_set_option(1, 0)
    assert rel(out[0, "fp64"], out[1, "fp64"]) <= SOLVE_TOL.get(name, 1e-12)
    assert rel(out[0, "fp64"], g["z"]) <= SOLVE_TOL.get(name, 1e-12)
    # unrefined FP32 solves: both within FP32 accuracy of the FP64 answer
    for generic in (0, 1):
        assert rel(out[generic, "fp32"], g["z"]) <= (1e-2 if name == "cauchy2001_compress" else 1e-4)


@pytest.mark.parametrize("name", ["synthetic_perfect", "synthetic_uneven", "synthetic_earlyexit",
                                  "cauchy2001_compress"])
def test_refinement_residual_paths(pkg, lib, orc, name):
    """FP32 factorization refined with the double-float residual product, its leaf
    products D X on the tensor cores (default) or on the FP32 pipe, and with the
    native FP64 product: all reach 1e-10 in true (oracle, FP64) residual, and the
    residual each reports is the true one."""
    L = pkg._lib
    g, h, A = _golden(pkg, orc, name)
    Af = orc.full(h)
    sols = []
    for native, tensor in ((0, 1), (0, 0), (1, 1)):
        assert lib.hss_set_option(L.HSS_OPT_RESIDUAL_FP64, native) == 0
        assert lib.hss_set_option(L.HSS_OPT_TENSOR_RESIDUAL, tensor) == 0
        try:
            st = {}
            z = pkg.ldiv(A, g["b"], precision="fp32", tol=1e-10, maxit=30, stats=st)
        finally:
            lib.hss_set_option(L.HSS_OPT_RESIDUAL_FP64, 0)
            lib.hss_set_option(L.HSS_OPT_TENSOR_RESIDUAL, 1)
        assert st["converged"]
        res = np.linalg.norm(g["b"] - Af @ z, axis=0) / np.linalg.norm(g["b"], axis=0)
        assert res.max() <= 2e-10, (native, tensor, res.max())
        # the reported residual is computed before the last correction's effect
        # is known only to the residual's own accuracy: ~1e-14 of |A| |x| / |b|
        assert abs(st["residual"] - res.max()) <= 1e-12 + 1e-2 * res.max(), (native, tensor)
        sols.append(z)
    assert rel(sols[0], sols[1]) <= 1e-6 and rel(sols[0], sols[2]) <= 1e-6


@pytest.mark.parametrize("r", [1, 5, 32, 40])
def test_tensor_residual_matches_fp64(pkg, lib, orc, r):
    """One refinement step from the same FP32 solution with the residual formed by
    the tensor-core leaf products and by the native FP64 product: the residual
    norms agree to the residual's accuracy (1e-13 of |A||x|), on a tree with
    uneven 62/63-row leaves and r below, at and above one 32-column chunk."""
    L = pkg._lib
    rng = np.random.default_rng(40 + r)
    h = orc.synthetic_hss(2001, 64, 16, rng)
    A = pkg.HssMatrix.from_tree(h)
    b = rng.standard_normal((2001, r))
    out = {}
    F = pkg.ulvfactor(A, "fp32")
    for native in (0, 1):
        assert lib.hss_set_option(L.HSS_OPT_RESIDUAL_FP64, native) == 0
        try:
            with pytest.raises(pkg._lib.NoConvergence):   # one correction, then the residual again
                F.solve(b, tol=1e-300, maxit=1)
        finally:
            lib.hss_set_option(L.HSS_OPT_RESIDUAL_FP64, 0)
        out[native] = (F.stats.iterations, F.stats.residual)
    assert out[0][0] == out[1][0] == 1
    r0, r1 = out[0][1], out[1][1]
    assert 0.0 < r1 < 1e-9 and abs(r0 - r1) <= 1e-12 + 1e-3 * r1, (r0, r1)
