"""GPU: the flat form of the persistent FP64 product (products of at most four
columns; every leaf carries its own chain of translator products) against the
queued persistent product, the level-by-level product and the CPU oracle.

Tolerances: 1e-12 relative (2-norm) against the oracle, 1e-13 between GPU
paths (same arithmetic, different summation order); the flat product sums in
a fixed order, so repeated calls agree bit for bit.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

pytestmark = pytest.mark.gpu

HSS_OPT_RESIDUAL_FP64 = 2
HSS_OPT_LEVEL_PRODUCT = 3
HSS_OPT_FLAT_PRODUCT = 6


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _tree(pkg, orc, name):
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    return g, h, pkg.HssMatrix.from_tree(h)


def _three(lib, fn):
    """fn() with the flat product (default), the queued persistent product and
    the level-by-level product."""
    out = []
    for flat, level in ((1, 0), (0, 0), (1, 1)):
        assert lib.hss_set_option(HSS_OPT_FLAT_PRODUCT, flat) == 0
        assert lib.hss_set_option(HSS_OPT_LEVEL_PRODUCT, level) == 0
        try:
            out.append(fn())
        finally:
            lib.hss_set_option(HSS_OPT_FLAT_PRODUCT, 1)
            lib.hss_set_option(HSS_OPT_LEVEL_PRODUCT, 0)
    return out


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("r", [1, 2, 4])
def test_flat_agrees(pkg, lib, orc, name, r):
    g, h, A = _tree(pkg, orc, name)
    x = np.random.default_rng(r).standard_normal((g["x"].shape[0], r))
    ref = orc.matmul(h, x)
    f, q, l = _three(lib, lambda: pkg.matmul(A, x))
    assert rel(f, ref) <= 1e-12
    assert rel(f, q) <= 1e-13 and rel(f, l) <= 1e-13


@pytest.mark.parametrize("name", ["synthetic_uneven", "synthetic_unbalanced", "cauchy2001_compress"])
def test_flat_alpha_beta(pkg, lib, orc, name):
    """mul!(C, hssA, B, alpha, beta) (src/matmul.jl:18-28) with C aliasing the
    beta term, on the three paths."""
    g, h, A = _tree(pkg, orc, name)
    rng = np.random.default_rng(6)
    x = rng.standard_normal((g["x"].shape[0], 3))
    C0 = np.asfortranarray(rng.standard_normal((g["y"].shape[0], 3)))
    ref = orc.matmul(h, x, -1.5, 0.25, C0)

    def run():
        C = C0.copy(order="F")
        pkg.mul(C, A, x, -1.5, 0.25)
        return C

    f, q, l = _three(lib, run)
    assert rel(f, ref) <= 1e-12 and rel(f, q) <= 1e-13 and rel(f, l) <= 1e-13


def test_flat_forest(pkg, lib, orc):
    """A forest of uneven trees (a single-leaf tree, a root with two leaves,
    ragged leaf sizes and ranks), each with its own column count <= 4."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    trees = [orc.synthetic_hss(n, ls, k, rng) for n, ls, k in
             [(1152, 64, 24), (640, 128, 20), (2001, 64, 16), (129, 64, 8), (64, 64, 8)]]
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    rs = [1, 4, 0, 2, 3]
    xs = [rng.standard_normal((t.size()[1], r)) for t, r in zip(trees, rs)]

    def run():
        dX = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in xs]
        dY = [torch.zeros((x.shape[1], t.size()[0]), dtype=torch.float64, device="cuda") for x, t in zip(xs, trees)]
        dev.matmul_batch_device(dX, [x.shape[0] for x in xs], rs, dY, [t.size()[0] for t in trees])
        torch.cuda.synchronize()
        return [y.cpu().numpy().T for y in dY]

    f, q, l = _three(lib, run)
    for t, x, a, b, c in zip(trees, xs, f, q, l):
        if x.shape[1] == 0:
            continue
        assert rel(a, orc.matmul(t, x)) <= 1e-12 and rel(a, b) <= 1e-13 and rel(a, c) <= 1e-13


def test_flat_repeated_bitwise(pkg, lib, orc):
    """Ten flat products in a row: identical bits, one launch each (the launch
    state resets itself)."""
    g, h, A = _tree(pkg, orc, "synthetic_perfect")
    dev = A.device()
    x = np.random.default_rng(2).standard_normal((g["x"].shape[0], 1))
    first = dev.matmul_host(x)
    c0 = lib.hss_launch_counter()
    for _ in range(10):
        assert np.array_equal(dev.matmul_host(x), first)
    assert lib.hss_launch_counter() - c0 == 10
    assert rel(first, orc.matmul(h, x)) <= 1e-12


@pytest.mark.parametrize("name", ["synthetic_perfect", "cauchy2001_compress"])
def test_flat_fp64_residual_refinement(pkg, lib, orc, name):
    """The FP64 refinement residual of an FP32 factorization runs the flat
    product with column norms (two right-hand sides): refined to 1e-10."""
    g, h, A = _tree(pkg, orc, name)
    Af = orc.full(h)
    b = np.random.default_rng(3).standard_normal((g["y"].shape[0], 2))
    assert lib.hss_set_option(HSS_OPT_RESIDUAL_FP64, 1) == 0
    try:
        st = {}
        z = pkg.ldiv(A, b, precision="fp32", tol=1e-10, maxit=30, stats=st)
    finally:
        lib.hss_set_option(HSS_OPT_RESIDUAL_FP64, 0)
    assert st["converged"] and st["residual"] <= 1e-10
    res = np.linalg.norm(b - Af @ z, axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 2e-10
