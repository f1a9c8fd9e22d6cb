"""GPU accuracy at the benchmark configurations, against the oracle and LAPACK.

* FP64 ULV solves of every golden fixture against ulvfactor.jl transcribed over
  LAPACK's own dgeqlf/dormql/dgelqf/dormlq/dtrsm/dgetrf (``oracle/lapack_ulv.py``):
  1e-12 relative (cond(A) * 1e-14 above cond 100).
* Precision workload (n = 65536, leafsize 128, k = 32) at r = 1: FP64 solve
  within 1e-12 of the oracle; FP32 + refinement to a true residual of 1e-10.
* Compression workload (Cauchy kernel on 16384 points, leafsize 128,
  randcompress_adaptive at 1e-9): same rounds, sample count and ranks as the
  oracle on the same Omega; 64-column product and FP64 ULV solve of the result
  within 1e-12 of the oracle on the same generators, and their error against
  the dense matrix.
* Batching workload: 32 matrices drawn as the benchmark draws its 256 (n 1024..16384
  step 128, leafsize 64/128/256, k 8..48, r 1..16, seed 2) in one forest,
  FP64 within 1e-12 of the oracle per matrix, FP32 + refinement to 1e-10 true residual.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

pytestmark = pytest.mark.gpu

MV_TOL = 1e-12
SOLVE_TOL = 1e-12
RESID_TOL = 1e-10


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _resid(Af_or_mul, x, b):
    r = b - Af_or_mul(x)
    return float((np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)).max())


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_fp64_solve_matches_lapack_transcription(pkg, orc, name):
    lap = pytest.importorskip("oracle.lapack_ulv")
    if not lap.available():
        pytest.skip("SciPy's OpenBLAS does not export the LQ/QL routines here")
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    A = pkg.HssMatrix.from_tree(h)
    z = pkg.ldiv(A, g["b"])
    cond = np.linalg.cond(orc.full(h))
    assert rel(z, lap.ulvfactsolve(h, g["b"])) <= max(SOLVE_TOL, cond * 1e-14)


def test_precision_workload_single_rhs(pkg, orc):
    """n = 65536, leafsize 128, k = 32 with one right-hand side (the r = 1 form of the workload)."""
    rng = np.random.default_rng(3)
    h = orc.synthetic_hss(65536, 128, 32, rng)
    A = pkg.HssMatrix.from_tree(h)
    b = rng.standard_normal((65536, 1))
    z64 = pkg.ldiv(A, b)
    assert rel(z64, orc.ulvfactsolve(h, b)) <= SOLVE_TOL
    st = {}
    z32 = pkg.ldiv(A, b, precision="fp32", tol=RESID_TOL, stats=st)
    assert st["converged"] and st["residual"] <= RESID_TOL
    assert _resid(lambda x: orc.matmul(h, x), z32, b) <= RESID_TOL
    # the vector form hssA \ b (src/hssmatrix.jl:234 takes a Matrix; the shim adds Vector)
    zv = pkg.ldiv(A, b[:, 0], precision="fp32", tol=RESID_TOL)
    assert zv.ndim == 1 and rel(zv, z64[:, 0]) <= 1e-8


def test_compression_workload(pkg, orc):
    """randcompress_adaptive of the Cauchy kernel matrix on 16384 points (leafsize 128,
    kest 10, atol = rtol = 1e-9, noversampling 10, stepsize 20), then a 64-column product
    and a 64-column FP64 ULV solve of the compressed matrix."""
    n, tol = 16384, 1e-9
    A = orc.cauchy_matrix(n)
    cl = pkg.bisection_cluster(n, 128)
    st = {}
    dev = pkg.randcompress_adaptive(A, cl, cl, kest=10, atol=tol, rtol=tol, noversampling=10, stepsize=20,
                                    rng=np.random.default_rng(1), stats=st, device=True)
    st_o = {}
    ho = orc.randcompress_adaptive(A, orc.bisection_cluster(n, 128), orc.bisection_cluster(n, 128), 10, tol, tol,
                                   10, 20, rng=np.random.default_rng(1), stats=st_o)
    assert (st["rounds"], st["k"], st["samples"]) == (st_o["rounds"], st_o["k"], st_o["samples"])
    h = dev.to_host()
    # rank decisions at the threshold may flip under rounding (the oracle: HSS rank 40)
    assert abs(orc.hssrank(h) - orc.hssrank(ho)) <= 2
    rng = np.random.default_rng(1)
    B = rng.standard_normal((n, 64))
    # product: against the oracle on the same generators, and against the dense matrix
    y = dev.matmul_host(B)
    assert rel(y, orc.matmul(h, B)) <= MV_TOL
    AB = A @ B
    assert rel(y, AB) <= 50 * tol                     # test/runtests.jl:64 (c = 50)
    assert rel(orc.matmul(ho, B), AB) <= 50 * tol     # the oracle's own compression, same bound
    # FP64 ULV solve of the compressed matrix
    F = dev.ulvfactor("fp64")
    x = F.solve(B, tol=0.0)
    x_o = orc.ulvfactsolve(h, B)
    assert rel(x, x_o) <= 1e-10                        # cond(A) ~ 1e4: two FP64 solves differ by ~cond * eps
    assert _resid(lambda v: orc.matmul(h, v), x, B) <= 1e-12
    # the error statement against the dense matrix: the compression error amplified by
    # the solve (the oracle's own compression of the same draws: 3.8e-8)
    assert _resid(lambda v: A @ v, x, B) <= 1e-6


def _config4_draws(count, seed=2):
    """The first `count` matrices of the batching workload's draw sequence."""
    rng = np.random.default_rng(seed)
    for _ in range(count):
        n = int(rng.integers(1024 // 128, 16384 // 128 + 1)) * 128
        ls = int(rng.choice([64, 128, 256]))
        k = int(rng.integers(8, 49))
        yield n, ls, k, rng


def test_batching_workload_forest(pkg, orc):
    torch = pytest.importorskip("torch")
    trees, rs, shapes = [], [], set()
    rng = None
    for n, ls, k, rng in _config4_draws(32):
        trees.append(orc.synthetic_hss(n, ls, k, rng))
        rs.append(int(rng.integers(1, 17)))
        shapes.add(ls)
    assert shapes == {64, 128, 256}
    dev = pkg.DeviceHss.from_trees([pkg.HssMatrix.from_tree(t) for t in trees])
    xs = [rng.standard_normal((t.size()[0], r)) for t, r in zip(trees, rs)]
    dB = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in xs]
    ns = [t.size()[0] for t in trees]
    for prec in ("fp64", "fp32"):
        F = dev.ulvfactor(prec)
        dX = [torch.zeros_like(b) for b in dB]
        st = F.solve_batch_device(dB, ns, rs, dX, ns, tol=0.0 if prec == "fp64" else RESID_TOL, maxit=20)
        torch.cuda.synchronize()
        if prec == "fp32":
            assert st.converged and st.residual <= RESID_TOL
        for t, b, x in zip(trees, xs, dX):
            z = x.cpu().numpy().T
            if prec == "fp64":
                assert rel(z, orc.ulvfactsolve(t, b)) <= SOLVE_TOL
            else:
                assert _resid(lambda v: orc.matmul(t, v), z, b) <= RESID_TOL
