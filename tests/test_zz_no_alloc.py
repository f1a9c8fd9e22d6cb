"""The allocation-free HSS product (hss_matmul_noalloc) against the regular one.

Some callers cannot allocate device memory while they run (host callbacks,
pre-allocated real-time loops, runtimes that forbid cudaMalloc after start-up);
for them the library offers a product whose scratch lives in fixed device
arrays.  This file is collected last so that a failure here leaves every
other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MV_TOL = 1e-12   # the tolerance of the other FP64 product tests


def _call(fn, dev, dB, n, r, dC, m, alpha, beta):
    return fn(dev.handle, C.c_void_p(dB.data_ptr()), n, r, C.c_void_p(dC.data_ptr()), m,
              float(alpha), float(beta), None)


def test_noalloc_product_matches_regular(pkg, lib, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    h = orc.synthetic_hss(2001, 64, 16, rng)
    n, r = 2001, 5
    X = rng.standard_normal((n, r))
    Y0 = rng.standard_normal((n, r))
    # column-major n x r matrices are r x n row-major tensors
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    ref = torch.from_numpy(np.ascontiguousarray(Y0.T)).cuda()
    # the regular product on a handle of its own: it grows that handle's
    # workspace, which the allocation-free product must not touch
    reg = pkg.HssMatrix.from_tree(h).device()
    assert _call(lib.hss_matmul, reg, dX, n, r, ref, n, 0.5, -1.5) == 0, lib.hss_last_error()
    torch.cuda.synchronize()
    ref_h = ref.cpu().numpy().T
    assert np.linalg.norm(ref_h - orc.matmul(h, X, 0.5, -1.5, Y0)) <= MV_TOL * np.linalg.norm(ref_h)
    dev = pkg.HssMatrix.from_tree(h).device()   # fresh handle: never ran a product
    outs = [torch.from_numpy(np.ascontiguousarray(Y0.T)).cuda() for _ in range(2)]
    torch.cuda.synchronize()
    for i, out in enumerate(outs):   # two calls in a row share the fixed scratch
        free0 = torch.cuda.mem_get_info()[0]
        assert _call(lib.hss_matmul_noalloc, dev, dX, n, r, out, n, 0.5, -1.5) == 0, lib.hss_last_error()
        torch.cuda.synchronize()
        if i > 0:   # the first call on a device may load the library's module there
            assert torch.cuda.mem_get_info()[0] == free0, "the allocation-free product allocated device memory"
        got = out.cpu().numpy().T
        assert np.linalg.norm(got - ref_h) <= MV_TOL * np.linalg.norm(ref_h)


def test_noalloc_rejects_oversized_calls(pkg, lib, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(18)
    A = pkg.HssMatrix.from_tree(orc.synthetic_hss(65536, 128, 32, rng))
    dev = A.device()
    r = 64   # 65408 workspace rows x 64 > 2^20 doubles
    dX = torch.zeros((r, 65536), dtype=torch.float64, device="cuda")
    dC = torch.zeros_like(dX)
    rc = _call(lib.hss_matmul_noalloc, dev, dX, 65536, r, dC, 65536, 1.0, 0.0)
    assert rc == pkg._lib.HSS_ERR_BAD_DIMS
    assert b"fixed scratch" in lib.hss_last_error()
