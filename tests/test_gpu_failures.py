"""Failure detection without a GPU fault.

* Bounded waits: HSS_OPT_POLL_LIMIT shortens the poll limit of the persistent
  products' waits so that they run out on purpose.  The waits end, the kernel
  records a device status and returns, the host reports HSS_ERR_TIMEOUT and
  clears the plan's counters, and the next call on the same plan is correct.
* Allocation failures: HSS_OPT_FAIL_ALLOC makes a chosen device allocation
  fail on the host (before the driver is called).  The call reports
  HSS_ERR_OOM, and the handle or factorization it was working on stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MV_TOL = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def big(pkg, orc):
    rng = np.random.default_rng(21)
    h = orc.synthetic_hss(65536, 128, 32, rng)
    return h, pkg.HssMatrix.from_tree(h)


def _times_out(fn, tries=5):
    """True if fn raises HssTimeout within `tries` calls (the product's work may finish before any wait)."""
    from hssmatrices_gb300._lib import HssTimeout
    for _ in range(tries):
        try:
            fn()
        except HssTimeout:
            return True
    return False


@pytest.mark.parametrize("r", [1, 8])   # the flat product (r <= 4) and the queued one
def test_product_wait_runs_out_and_plan_recovers(pkg, lib, orc, big, r):
    L = pkg._lib
    h, A = big
    x = np.random.default_rng(r).standard_normal((65536, r))
    assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, 1) == 0
    try:
        assert _times_out(lambda: pkg.matmul(A, x))
    finally:
        assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, 0) == 0
    # counters cleared by the host: the next products on the same plan are right
    ref = orc.matmul(h, x)
    for _ in range(2):
        assert rel(pkg.matmul(A, x), ref) <= MV_TOL


def test_refinement_residual_wait_runs_out(pkg, lib, orc, big):
    L = pkg._lib
    h, A = big
    b = np.random.default_rng(5).standard_normal((65536, 4))
    F = pkg.ulvfactor(A, "fp32")
    assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, 1) == 0
    try:
        assert _times_out(lambda: F.solve(b, tol=1e-10, maxit=3))
    finally:
        assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, 0) == 0
    x = F.solve(b, tol=1e-10)
    res = np.linalg.norm(b - orc.matmul(h, x), axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-10


def test_allocation_failure_reports_oom(pkg, lib, orc):
    L = pkg._lib
    rng = np.random.default_rng(8)
    h = orc.synthetic_hss(3000, 64, 16, rng)
    b = rng.standard_normal((3000, 3))
    ref = orc.ulvfactsolve(h, b)
    # creating a handle: every allocation of the plan in turn
    for k in (1, 2, 3):
        assert lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, k) == 0
        try:
            with pytest.raises(MemoryError):
                pkg.DeviceHss(pkg.HssMatrix.from_tree(h))
        finally:
            lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, 0)
    A = pkg.HssMatrix.from_tree(h)
    dev = A.device()
    # a factorization's storage
    assert lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, 1) == 0
    try:
        with pytest.raises(MemoryError):
            dev.ulvfactor("fp64")
    finally:
        lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, 0)
    F = dev.ulvfactor("fp64")
    # a solve's first buffers (host staging and workspaces grow on first use)
    assert lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, 1) == 0
    try:
        with pytest.raises(MemoryError):
            F.solve(b, tol=0.0)
    finally:
        lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, 0)
    # the handle and the factorization are intact
    assert rel(F.solve(b, tol=0.0), ref) <= 1e-12
    assert rel(pkg.matmul(A, b), orc.matmul(h, b)) <= MV_TOL
