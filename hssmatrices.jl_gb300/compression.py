"""Randomized HSS compression with the sampling products and the tree pass on the GPU.

* ``randcompress(A, rcl, ccl, kest)``           -- src/compression.jl:278-294
* ``randcompress_adaptive(A, rcl, ccl; kest)``  -- src/compression.jl:312-355
* ``hss_blkdiag``, ``_randcompress!``, ``_interpolate`` (src/compression.jl:358-475)
  run inside ``hss_rc_compress``: one launch per tree level, FP64 rank decisions.

The dense matrix is held on the device once (``DenseDevice``, column-major
FP64); the sample products ``A * Omega``, ``A' * Omega`` and the test product
``hssA * Omega`` run there.  ``sample_precision="df"`` computes the sample
products in double-float arithmetic on the FP32 pipe (the mixed-precision
form: ~2^-47 relative per operation, several times the FP64 rate of GB300;
rank decisions stay FP64); "fp64" (default) matches the reference's Float64.  The test matrices are drawn on the host with a
NumPy ``Generator`` (``rng``), in the reference's order -- Omega_col, then
Omega_row, then per test round Omega_col_test, Omega_row_test -- so that a
seeded run is repeatable.  The result is an ``HssMatrix`` whose uploaded copy
is the compressed handle itself.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import check, iptr
from .hssmatrix import HssOptions
from .linalg import DeviceHss, _stream


def _torch():
    import torch
    return torch


class DenseDevice:
    """A dense FP64 matrix on the GPU in column-major order (``lda = m``)."""

    def __init__(self, A, device="cuda"):
        torch = _torch()
        if isinstance(A, DenseDevice):
            self.t, self.m, self.n, self.lda = A.t, A.m, A.n, A.lda
            return
        if isinstance(A, torch.Tensor):
            if A.dim() != 2:
                raise ValueError("expected a matrix")
            self.m, self.n = A.shape
            # (n, m) row-major == (m, n) column-major
            self.t = A.to(device=device, dtype=torch.float64).t().contiguous()
        else:
            A = np.asarray(A, dtype=np.float64)
            if A.ndim != 2:
                raise ValueError("expected a matrix")
            self.m, self.n = A.shape
            self.t = torch.from_numpy(np.ascontiguousarray(A.T)).to(device)
        self.lda = max(self.m, 1)

    @property
    def shape(self):
        return self.m, self.n

    def ptr(self):
        return self.t.data_ptr()


def _cols_to_device(X, device="cuda"):
    """Host (rows x cols) array -> device column-major tensor of shape (cols, rows)."""
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(X, dtype=np.float64).T)).to(device)


def sample(A: DenseDevice, X, trans=False, out=None, alpha=1.0, beta=0.0, stream=None):
    """``A * X`` (or ``A' * X``) on the device; X and the result are column-major
    tensors of shape (cols, rows)."""
    lib = _lib.load()
    rows, inner = (A.n, A.m) if trans else (A.m, A.n)
    if X.shape[1] != inner:
        raise ValueError(f"DimensionMismatch: expected {inner} rows, got {X.shape[1]}")
    r = X.shape[0]
    if out is None:
        out = _torch().empty((r, rows), dtype=X.dtype, device=X.device)
        beta = 0.0
    check(lib.hss_sample(C.c_void_p(A.ptr()), A.lda, A.m, A.n, int(bool(trans)), C.c_void_p(X.data_ptr()),
                         max(inner, 1), r, C.c_void_p(out.data_ptr()), max(rows, 1), float(alpha), float(beta),
                         _stream(stream)))
    return out


def sumsq(B, stream=None):
    """Sum of squares of a column-major device matrix of shape (cols, rows)."""
    lib = _lib.load()
    out = C.c_double()
    r, m = B.shape
    check(lib.hss_sumsq(C.c_void_p(B.data_ptr()), max(m, 1), m, r, C.byref(out), _stream(stream)))
    return out.value


def cluster_table(rcl, ccl):
    """Pre-order table (left, right, rlo, rhi, clo, chi; 0-based half-open) of two
    compatible cluster trees (``compatible``, src/clustertree.jl)."""
    rows = []

    def visit(r, c):
        i = len(rows)
        rows.append([-1, -1, r.lo - 1, r.hi, c.lo - 1, c.hi])
        if r.isleaf() != c.isleaf():
            raise ValueError("row and column clusters are not compatible")
        if not r.isleaf():
            rows[i][0] = visit(r.left, c.left)
            rows[i][1] = visit(r.right, c.right)
        return i

    visit(rcl, ccl)
    return np.ascontiguousarray(np.array(rows, dtype=np.int64))


class Compressor:
    """The tree pass of randomized compression for one pair of cluster trees."""

    def __init__(self, rcl, ccl):
        self.lib = _lib.load()
        self.table = cluster_table(rcl, ccl)
        self.m, self.n = int(self.table[0, 3]), int(self.table[0, 5])
        self.handle = C.c_void_p()
        check(self.lib.hss_rc_create(self.table.shape[0], iptr(self.table), C.byref(self.handle)))

    def __del__(self):
        try:
            if self.handle:
                self.lib.hss_rc_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def compress(self, A: DenseDevice, Scol, Srow, Ocol, Orow, atol, rtol, stream=None) -> DeviceHss:
        """``_randcompress!`` from the samples (column-major device tensors of
        shapes (s, m), (s, n), (s, n), (s, m)); returns the compressed handle."""
        s = Scol.shape[0]
        for X, rows in ((Scol, A.m), (Srow, A.n), (Ocol, A.n), (Orow, A.m)):
            if X.shape != (s, rows):
                raise ValueError("DimensionMismatch: sample shapes")
        h = C.c_void_p()
        check(self.lib.hss_rc_compress(self.handle, C.c_void_p(A.ptr()), A.lda, C.c_void_p(Scol.data_ptr()),
                                       A.m, C.c_void_p(Srow.data_ptr()), A.n, C.c_void_p(Ocol.data_ptr()), A.n,
                                       C.c_void_p(Orow.data_ptr()), A.m, s, float(atol), float(rtol),
                                       C.byref(h), _stream(stream)))
        return DeviceHss(_handle=h)

    def sample(self, A: DenseDevice, X, trans=False, stream=None):
        """``A * X`` (``A' * X``) through ``hss_rc_sample``: with double-float
        sampling on, A's diagonal leaf blocks are multiplied in FP64 and the
        rest in double-float, so the corrected sample ``S - D * X`` keeps its
        own relative accuracy; otherwise the FP64 product of ``sample``."""
        rows, inner = (A.n, A.m) if trans else (A.m, A.n)
        if (A.m, A.n) != (self.m, self.n):
            raise ValueError("DimensionMismatch: matrix and clusters")
        if X.shape[1] != inner:
            raise ValueError(f"DimensionMismatch: expected {inner} rows, got {X.shape[1]}")
        r = X.shape[0]
        out = _torch().empty((r, rows), dtype=X.dtype, device=X.device)
        check(self.lib.hss_rc_sample(self.handle, C.c_void_p(A.ptr()), A.lda, int(bool(trans)),
                                     C.c_void_p(X.data_ptr()), max(inner, 1), r, C.c_void_p(out.data_ptr()),
                                     max(rows, 1), _stream(stream)))
        return out

    def ranks(self):
        """(column-side, row-side) rank per cluster node of the last compression."""
        out = np.zeros(2 * self.table.shape[0], dtype=np.int32)
        check(self.lib.hss_rc_ranks(self.handle, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out.reshape(-1, 2)


def _opts(opts, kw):
    opts = HssOptions.current() if opts is None else opts
    return opts.copy(**kw).check()


HSS_OPT_SAMPLE_DF = 5


class _SamplePrecision:
    """Sets the library's sample arithmetic for the duration of one compression.
    Double-float holds entries within float's exponent range; a matrix whose
    largest entry lies outside [2^-60, 2^100] is sampled in FP64."""

    def __init__(self, A: DenseDevice, precision):
        if precision not in ("fp64", "df"):
            raise ValueError(f"sample_precision must be 'fp64' or 'df', not {precision!r}")
        self.df = precision == "df"
        if self.df and A.t.numel() > 0:
            amax = float(A.t.abs().max())
            self.df = 2.0 ** -60 <= amax <= 2.0 ** 100

    def __enter__(self):
        check(_lib.load().hss_set_option(HSS_OPT_SAMPLE_DF, int(self.df)))
        return self

    def __exit__(self, *exc):
        _lib.load().hss_set_option(HSS_OPT_SAMPLE_DF, 0)
        return False


def randcompress(A, rcl, ccl, kest, opts=None, rng=None, device=False, sample_precision="fp64", **kw):
    """``randcompress(A, rcl, ccl, kest)`` (src/compression.jl:278-294): one
    compression from kest + noversampling samples."""
    opts = _opts(opts, kw)
    rng = np.random.default_rng(0) if rng is None else rng
    Ad = DenseDevice(A)
    m, n = Ad.shape
    comp = Compressor(rcl, ccl)
    s = kest + opts.noversampling
    Ocol = _cols_to_device(rng.standard_normal((n, s)))
    Orow = _cols_to_device(rng.standard_normal((m, s)))
    with _SamplePrecision(Ad, sample_precision):
        Scol = comp.sample(Ad, Ocol)
        Srow = comp.sample(Ad, Orow, trans=True)
    dev = comp.compress(Ad, Scol, Srow, Ocol, Orow, opts.atol, opts.rtol)
    return dev if device else dev.to_host()


def randcompress_adaptive(A, rcl, ccl, opts=None, kest=10, rng=None, stats=None, device=False,
                          sample_precision="fp64", **kw):
    """``randcompress_adaptive(A, rcl, ccl; kest)`` (src/compression.jl:312-355):
    compress, test the approximation on ``stepsize`` fresh samples
    (``sqrt(1/bs) * norm(Scol_test - hssA * Omega_test)`` against atol and
    rtol times ``sqrt(1/bs) * norm(Scol_test)``), and enlarge the sample by
    the test columns until the test passes."""
    torch = _torch()
    opts = _opts(opts, kw)
    rng = np.random.default_rng(0) if rng is None else rng
    Ad = DenseDevice(A)
    m, n = Ad.shape
    maxrank = n
    comp = Compressor(rcl, ccl)
    k, r, bs = kest, opts.noversampling, opts.stepsize
    sp = _SamplePrecision(Ad, sample_precision)
    Ocol = _cols_to_device(rng.standard_normal((n, k + r)))
    Orow = _cols_to_device(rng.standard_normal((m, k + r)))
    with sp:
        Scol = comp.sample(Ad, Ocol)
        Srow = comp.sample(Ad, Orow, trans=True)
    failed = True
    rounds = 0
    dev = None
    while failed and k < maxrank:
        dev = comp.compress(Ad, Scol, Srow, Ocol, Orow, opts.atol, opts.rtol)
        Ocol_t = _cols_to_device(rng.standard_normal((n, bs)))
        Orow_t = _cols_to_device(rng.standard_normal((m, bs)))
        with sp:
            Scol_t = comp.sample(Ad, Ocol_t)
            Srow_t = comp.sample(Ad, Orow_t, trans=True)
        nrm = math.sqrt(1.0 / bs) * math.sqrt(sumsq(Scol_t))
        E = Scol_t.clone()
        dev.matmul_device(Ocol_t, n, bs, E, m, alpha=-1.0, beta=1.0)
        nrm_est = math.sqrt(1.0 / bs) * math.sqrt(sumsq(E))
        failed = nrm_est > opts.atol and nrm_est > opts.rtol * nrm
        rounds += 1
        if opts.verbose and failed:
            print("Enlarging sampling space to ", k + bs)
        if failed:
            Ocol = torch.cat([Ocol, Ocol_t], dim=0)
            Orow = torch.cat([Orow, Orow_t], dim=0)
            Scol = torch.cat([Scol, Scol_t], dim=0)
            Srow = torch.cat([Srow, Srow_t], dim=0)
            k += bs
    if dev is None:   # kest >= n: the block diagonal alone (hss_blkdiag, :447-475)
        z = torch.zeros((0, m), dtype=torch.float64, device=Ad.t.device)
        zn = torch.zeros((0, n), dtype=torch.float64, device=Ad.t.device)
        dev = comp.compress(Ad, z, zn, zn, z, opts.atol, opts.rtol)
    if stats is not None:
        stats.update(rounds=rounds, k=k, samples=k + r, ranks=comp.ranks())
    return dev if device else dev.to_host()
