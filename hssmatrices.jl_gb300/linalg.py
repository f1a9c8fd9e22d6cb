"""GPU arithmetic behind the reference's operators, through the C ABI.

* ``matmul(hssA, B)``         -- ``*(hssA, B)`` (src/matmul.jl:13-15)
* ``mul(C, hssA, B, a, b)``   -- ``mul!(C, hssA, B, a, b)`` (src/matmul.jl:18-28)
* ``ulvfactsolve(hssA, b)``   -- ``ulvfactsolve`` (src/ulvfactor.jl:10-19), plain FP64
* ``ldiv(hssA, b)``           -- ``hssA \\ b`` (src/hssmatrix.jl:234)
* ``ulvfactor(hssA, prec)``   -- resident factorization (new; the reference's
                                 factor-only reduction is src/ulvdivide.jl:58-85)

Host arrays are column-major float64; 1-D inputs are treated as n x 1 like the
reference's vector methods.  Every call runs the CUDA library; if it cannot be
loaded the call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr
from .packing import pack, pack_cached

PREC = {"fp64": _lib.HSS_PREC_FP64, "fp32": _lib.HSS_PREC_FP32,
        _lib.HSS_PREC_FP64: _lib.HSS_PREC_FP64, _lib.HSS_PREC_FP32: _lib.HSS_PREC_FP32}


def _ptr(x):
    """Device pointer of a torch tensor / int / None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


def _as_cols(B, rows):
    B = np.asarray(B, dtype=np.float64)
    vec = B.ndim == 1
    if vec:
        B = B.reshape(-1, 1)
    if B.ndim != 2:
        raise ValueError("expected a vector or a matrix")
    if B.shape[0] != rows:
        raise ValueError(f"DimensionMismatch: expected {rows} rows, got {B.shape[0]}")
    return np.asfortranarray(B), vec


class DeviceHss:
    """One generator tree (or a forest, via ``from_trees``) resident on the GPU."""

    def __init__(self, h=None, *, _handle=None, _ntrees=1):
        self.lib = _lib.load()
        self.handle = C.c_void_p()
        if _handle is not None:
            self.handle = _handle
        else:
            table, packed = pack_cached(h)
            check(self.lib.hss_create(table.shape[0], iptr(table), dptr(packed), packed.size,
                                      C.byref(self.handle)))
        n = C.c_int32()
        check(self.lib.hss_ntrees(self.handle, C.byref(n)))
        self.ntrees = n.value
        self.sizes = []
        for t in range(self.ntrees):
            m, nn = C.c_int64(), C.c_int64()
            check(self.lib.hss_size(self.handle, t, C.byref(m), C.byref(nn)))
            self.sizes.append((m.value, nn.value))
        self.m, self.n = self.sizes[0]

    @classmethod
    def from_trees(cls, trees):
        """A forest of independent matrices in one plan (the batched form)."""
        lib = _lib.load()
        packs = [pack(h) for h in trees]
        cnt = len(packs)
        nn = np.array([t.shape[0] for t, _p in packs], dtype=np.int64)
        npk = np.array([p.size for _t, p in packs], dtype=np.int64)
        tabs = (_lib.PI64 * cnt)(*[iptr(t) for t, _p in packs])
        pks = (_lib.PD * cnt)(*[dptr(p) for _t, p in packs])
        handle = C.c_void_p()
        check(lib.hss_create_batch(cnt, iptr(nn), tabs, pks, iptr(npk), C.byref(handle)))
        obj = cls(_handle=handle)
        obj._keep = packs
        return obj

    def __del__(self):
        try:
            if self.handle:
                self.lib.hss_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    # -- bookkeeping ------------------------------------------------------
    def export(self):
        """Node table and packed generators (host copies) of a single-tree handle."""
        nn, npk = C.c_int64(), C.c_int64()
        check(self.lib.hss_export_size(self.handle, C.byref(nn), C.byref(npk)))
        table = np.zeros((nn.value, _lib.NODE_FIELDS), dtype=np.int64)
        packed = np.zeros(max(npk.value, 1), dtype=np.float64)
        check(self.lib.hss_export(self.handle, iptr(table), dptr(packed)))
        return table, packed[:npk.value]

    def to_host(self):
        """The ``HssMatrix`` of this handle, keeping this upload as its device copy."""
        from .packing import unpack
        table, packed = self.export()
        h = unpack(table, packed)
        h._device = self
        h._packed = (table, packed)
        return h

    def node_info(self, node):
        f = np.zeros(_lib.INFO_FIELDS, dtype=np.int64)
        check(self.lib.hss_node_info(self.handle, node, iptr(f)))
        keys = ["depth", "height", "row0", "col0", "m", "n", "ku", "kv", "k", "mk", "nk", "leaf", "tree"]
        return dict(zip(keys, (int(v) for v in f)))

    def ulv_cols(self, node):
        ln = C.c_int64()
        check(self.lib.hss_ulv_cols(self.handle, node, None, 0, C.byref(ln)))
        out = np.zeros(max(ln.value, 1), dtype=np.int64)
        check(self.lib.hss_ulv_cols(self.handle, node, iptr(out), out.size, C.byref(ln)))
        return out[:ln.value]

    # -- entries ------------------------------------------------------------
    def getindex_device(self, rows, cols, out=None, stream=None):
        """A[rows, cols] (0-based, any order, repeats allowed) into a device tensor
        of shape (len(cols), len(rows)) (column-major), ``hss_getindex``."""
        import torch
        rows = np.ascontiguousarray(rows, dtype=np.int64).ravel()
        cols = np.ascontiguousarray(cols, dtype=np.int64).ravel()
        if out is None:
            out = torch.empty((cols.size, rows.size), dtype=torch.float64, device="cuda")
        check(self.lib.hss_getindex(self.handle, iptr(rows), rows.size, iptr(cols), cols.size, _ptr(out),
                                    max(rows.size, 1), _stream(stream)))
        return out

    def getindex(self, rows, cols):
        """A[rows, cols] as a host array (rows x cols)."""
        import torch
        out = self.getindex_device(rows, cols)
        torch.cuda.synchronize()
        return out.cpu().numpy().T

    def full(self):
        """``full(hssA)`` (src/hssmatrix.jl:270-305) as a host array, ``hss_full``."""
        import torch
        out = torch.empty((self.n, self.m), dtype=torch.float64, device="cuda")
        check(self.lib.hss_full(self.handle, _ptr(out), max(self.m, 1), _stream(None)))
        torch.cuda.synchronize()
        return out.cpu().numpy().T

    # -- products -----------------------------------------------------------
    def matmul_host(self, B, alpha=1.0, beta=0.0, C_=None):
        B, vec = _as_cols(B, self.n)
        r = B.shape[1]
        if C_ is None:
            out = np.zeros((self.m, r), order="F")
            beta = 0.0
        else:
            out = C_
        check(self.lib.hss_matmul_host(self.handle, dptr(B), B.shape[0], r, dptr(out),
                                       out.shape[0], float(alpha), float(beta)))
        return out.reshape(-1) if vec else out

    def matmul_device(self, dB, ldb, r, dC, ldc, alpha=1.0, beta=0.0, stream=None, trans=False):
        """C = alpha op(A) B + beta C on device buffers; op(A) = A^T with trans
        (``hss_matmul_t``: the adjoint's generators made on the device once)."""
        f = self.lib.hss_matmul_t if trans else self.lib.hss_matmul
        check(f(self.handle, _ptr(dB), ldb, r, _ptr(dC), ldc, float(alpha), float(beta), _stream(stream)))

    def transpose(self):
        """The adjoint as a new device handle (``hss_transpose``, src/hssmatrix.jl:165-178)."""
        h = C.c_void_p()
        check(self.lib.hss_transpose(self.handle, C.byref(h), _stream(None)))
        return DeviceHss(_handle=h)

    def matmul_batch_device(self, dBs, ldbs, rs, dCs, ldcs, alpha=1.0, beta=0.0, stream=None):
        k = self.ntrees
        B = (C.c_void_p * k)(*[_ptr(x) for x in dBs])
        Cc = (C.c_void_p * k)(*[_ptr(x) for x in dCs])
        ldb = np.asarray(ldbs, np.int64)
        ldc = np.asarray(ldcs, np.int64)
        r = np.asarray(rs, np.int64)
        check(self.lib.hss_matmul_batch(self.handle, B, iptr(ldb), iptr(r), Cc, iptr(ldc),
                                        float(alpha), float(beta), _stream(stream)))

    # -- ULV ------------------------------------------------------------------
    def ulvfactor(self, precision="fp64", stream=None):
        return UlvFactor(self, PREC[precision], stream)


class UlvFactor:
    """A resident ULV factorization (FP64, or FP32 refined in FP64)."""

    def __init__(self, dev: DeviceHss, prec: int, stream=None):
        self.dev = dev
        self.lib = dev.lib
        self.prec = prec
        self.handle = C.c_void_p()
        check(self.lib.hss_ulvfactor(dev.handle, prec, C.byref(self.handle), _stream(stream)))
        self.stats = _lib.SolveStats()

    def __del__(self):
        try:
            if self.handle:
                self.lib.hss_factor_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def refactor(self, stream=None):
        """Recompute the factorization in place (no allocation)."""
        check(self.lib.hss_ulvrefactor(self.handle, _stream(stream)))

    def autotune(self, r, stream=None):
        """Time the solve kernel variants of every tree level and the residual
        products on scratch right-hand sides (r columns); later solves of this
        factorization use the faster per level.  Returns the choices."""
        check(self.lib.hss_autotune(self.handle, int(r), _stream(stream)))
        return self.tuning()

    def tuning(self):
        """{"up": [...], "down": [...], "product": p}: per level 1 blocked solve,
        0 register solve, -1 not tuned; product 1 persistent, 0 per level."""
        nu, nd, pm = C.c_int32(), C.c_int32(), C.c_int32()
        check(self.lib.hss_autotune_info(self.handle, C.byref(nu), None, C.byref(nd), None, C.byref(pm)))
        up = C.create_string_buffer(max(nu.value, 1))
        dn = C.create_string_buffer(max(nd.value, 1))
        check(self.lib.hss_autotune_info(self.handle, C.byref(nu), up, C.byref(nd), dn, C.byref(pm)))
        sgn = lambda b: [x - 256 if x > 127 else x for x in b]
        return {"up": sgn(up.raw[:nu.value]), "down": sgn(dn.raw[:nd.value]), "product": pm.value}

    def nbytes(self):
        b = C.c_int64()
        check(self.lib.hss_factor_bytes(self.handle, C.byref(b)))
        return b.value

    def default_tol(self):
        return 1e-10 if self.prec == _lib.HSS_PREC_FP32 else 0.0

    def solve(self, b, tol=None, maxit=10):
        """x = A \\ b with host arrays."""
        tol = self.default_tol() if tol is None else tol
        b, vec = _as_cols(b, self.dev.m)
        r = b.shape[1]
        x = np.zeros((self.dev.n, r), order="F")
        check(self.lib.hss_ulvsolve_host(self.handle, dptr(b), b.shape[0], r, dptr(x), x.shape[0],
                                         float(tol), int(maxit), C.byref(self.stats)))
        return x.reshape(-1) if vec else x

    def solve_device(self, dB, ldb, r, dX, ldx, tol=None, maxit=10, stream=None):
        tol = self.default_tol() if tol is None else tol
        check(self.lib.hss_ulvsolve(self.handle, _ptr(dB), ldb, r, _ptr(dX), ldx, float(tol),
                                    int(maxit), C.byref(self.stats), _stream(stream)))
        return self.stats

    def factsolve_device(self, dB, ldb, r, dX, ldx, tol=None, maxit=10, stream=None):
        """Refactor (the generators may have changed) and solve in one call
        (``hss_ulvfactsolve``): the first solve's upward sweep runs one tree level
        behind the factorization on a second stream."""
        tol = self.default_tol() if tol is None else tol
        check(self.lib.hss_ulvfactsolve(self.handle, _ptr(dB), ldb, r, _ptr(dX), ldx, float(tol),
                                        int(maxit), C.byref(self.stats), _stream(stream)))
        return self.stats

    def solve_batch_device(self, dBs, ldbs, rs, dXs, ldxs, tol=None, maxit=10, stream=None):
        tol = self.default_tol() if tol is None else tol
        k = self.dev.ntrees
        B = (C.c_void_p * k)(*[_ptr(x) for x in dBs])
        X = (C.c_void_p * k)(*[_ptr(x) for x in dXs])
        ldb = np.asarray(ldbs, np.int64)
        ldx = np.asarray(ldxs, np.int64)
        r = np.asarray(rs, np.int64)
        check(self.lib.hss_ulvsolve_batch(self.handle, B, iptr(ldb), iptr(r), X, iptr(ldx),
                                          float(tol), int(maxit), C.byref(self.stats),
                                          _stream(stream)))
        return self.stats


def trace_begin(kind):
    """Bracket every launch of one kernel kind (``_lib.TRACE`` key) with CUDA events."""
    lib = _lib.load()
    check(lib.hss_trace_begin(_lib.TRACE[kind] if isinstance(kind, str) else int(kind)))


def trace_end():
    """(summed device milliseconds, number of launches) since ``trace_begin``."""
    lib = _lib.load()
    ms, n = C.c_double(), C.c_int64()
    check(lib.hss_trace_end(C.byref(ms), C.byref(n)))
    return ms.value, n.value


def trace_times(cap=4096):
    """Per-launch device milliseconds (launch order) since ``trace_begin``; ends the trace."""
    lib = _lib.load()
    buf = np.zeros(cap, dtype=np.float64)
    n = C.c_int64()
    check(lib.hss_trace_times(buf.ctypes.data_as(_lib.PD), cap, C.byref(n)))
    return buf[:min(n.value, cap)].tolist()


def launch_counter():
    return _lib.load().hss_launch_counter()


# ---------------------------------------------------------------------------
# reference-shaped entry points
# ---------------------------------------------------------------------------


def matmul(hssA, B):
    """``hssA * B`` (src/matmul.jl:13-15)."""
    return hssA.device().matmul_host(B)


def mul(C_, hssA, B, alpha=1.0, beta=0.0):
    """``mul!(C, hssA, B, alpha, beta)`` (src/matmul.jl:18-28): overwrites C."""
    dev = hssA.device()
    B, _vec = _as_cols(B, dev.n)
    if not (isinstance(C_, np.ndarray) and C_.dtype == np.float64 and C_.flags.f_contiguous):
        raise ValueError("C must be a column-major float64 array")
    Cv = C_.reshape(C_.shape[0], -1, order="F")
    if Cv.shape != (dev.m, B.shape[1]):
        raise ValueError("Dimensions of C don't match up with A and B.")
    dev.matmul_host(B, alpha, beta, Cv)
    return C_


def ulvfactor(hssA, precision="fp64"):
    """Resident ULV factorization of ``hssA``."""
    return hssA.device().ulvfactor(precision)


def ulvfactsolve(hssA, b):
    """``ulvfactsolve(hssA, b)`` (src/ulvfactor.jl:10): FP64 factor + solve."""
    return ldiv(hssA, b, precision="fp64")


def _index_list(k, size):
    """One index of ``getindex`` (src/hssmatrix.jl:102-107): an int, a slice
    (range or colon) or a sequence, 0-based; returns (array, scalar?)."""
    if isinstance(k, (int, np.integer)):
        if not -size <= k < size:
            raise IndexError(f"index {k} out of range for size {size}")
        return np.array([k % size], dtype=np.int64), True
    if isinstance(k, slice):
        return np.arange(size, dtype=np.int64)[k], False
    a = np.asarray(k, dtype=np.int64).ravel()
    if a.size and (a.min() < 0 or a.max() >= size):
        raise IndexError("index out of range")
    return a, False


def getindex(hssA, i, j):
    """``hssA[i, j]`` (src/hssmatrix.jl:102-114) on the device: ints, slices and
    index sequences (0-based); a scalar for two ints, a vector when one index
    is an int, else a matrix."""
    m, n = hssA.size()
    ri, si = _index_list(i, m)
    cj, sj = _index_list(j, n)
    dev = hssA.device() if hasattr(hssA, "device") else hssA
    out = dev.getindex(ri, cj) if ri.size and cj.size else np.zeros((ri.size, cj.size))
    if si and sj:
        return float(out[0, 0])
    if si:
        return out[0, :]
    if sj:
        return out[:, 0]
    return out


def hssmul(hssA, hssB, device=False):
    """``hssA * hssB`` for two HSS matrices (src/matmul.jl:65-117) on the
    device: the product on the same cluster tree, ranks adding up.  Returns an
    ``HssMatrix`` (or the ``DeviceHss`` handle with ``device=True``)."""
    a = hssA.device() if hasattr(hssA, "device") else hssA
    b = hssB.device() if hasattr(hssB, "device") else hssB
    h = C.c_void_p()
    check(a.lib.hss_hssmul(a.handle, b.handle, C.byref(h), _stream(None)))
    dev = DeviceHss(_handle=h)
    return dev if device else dev.to_host()


def recompress(hssA, atol=None, rtol=None, device=False):
    """``recompress!(hssA; atol, rtol)`` (src/compression.jl:148-260) on the
    device: orthonormalized generators, couplings truncated top-down.  Returns
    a new ``HssMatrix`` (the reference modifies hssA in place); tolerances
    default to ``HssOptions``'."""
    from .hssmatrix import HssOptions
    opts = HssOptions.current()
    atol = opts.atol if atol is None else atol
    rtol = opts.rtol if rtol is None else rtol
    a = hssA.device() if hasattr(hssA, "device") else hssA
    h = C.c_void_p()
    check(a.lib.hss_recompress(a.handle, float(atol), float(rtol), C.byref(h), _stream(None)))
    dev = DeviceHss(_handle=h)
    return dev if device else dev.to_host()


def orthonormalize_generators(hssA, device=False):
    """``orthonormalize_generators!(hssA)`` (src/generators.jl:64-114) on the
    device; returns a new ``HssMatrix``."""
    a = hssA.device() if hasattr(hssA, "device") else hssA
    h = C.c_void_p()
    check(a.lib.hss_orthonormalize(a.handle, C.byref(h), _stream(None)))
    dev = DeviceHss(_handle=h)
    return dev if device else dev.to_host()


def full(hssA):
    """``full(hssA)`` / ``Matrix(hssA)`` (src/hssmatrix.jl:268-305) on the device."""
    dev = hssA.device() if hasattr(hssA, "device") else hssA
    return dev.full()


def ldiv(hssA, b, precision="fp64", tol=None, maxit=10, stats=None, **kw):
    """``hssA \\ b`` (src/hssmatrix.jl:234).  ``precision='fp32'`` factors in FP32 and
    refines with FP64 HSS products to ``tol`` (default 1e-10 relative residual).
    An HssMatrix ``b`` gives ``hssA \\ hssB`` (``hss_ldiv``)."""
    from .hssmatrix import HssMatrix
    if isinstance(b, HssMatrix):
        return hss_ldiv(hssA, b, stats=stats, **kw)
    dev = hssA.device()
    prec = PREC[precision]
    tol = (1e-10 if prec == _lib.HSS_PREC_FP32 else 0.0) if tol is None else tol
    b, vec = _as_cols(b, dev.m)
    r = b.shape[1]
    x = np.zeros((dev.n, r), order="F")
    st = _lib.SolveStats()
    check(dev.lib.hss_ulvfactsolve_host(dev.handle, prec, dptr(b), b.shape[0], r, dptr(x), x.shape[0],
                                        float(tol), int(maxit), C.byref(st)))
    if stats is not None:
        stats.update(iterations=st.iterations, converged=bool(st.converged), residual=st.residual)
    return x.reshape(-1) if vec else x


# ---------------------------------------------------------------------------
# HSS-valued division (src/ulvdivide.jl:13-17, src/hssmatrix.jl:235-237)
# ---------------------------------------------------------------------------


def transpose(hssA):
    """``hssA'`` for real generators (the adjoint of src/hssmatrix.jl): every
    leaf's D transposed with U and V swapped, every branch's B12 and B21
    exchanged and transposed, R and W swapped."""
    from .hssmatrix import HssMatrix
    if hssA.isleaf():
        cp = lambda x: None if x is None else np.array(x, dtype=np.float64)
        return HssMatrix.leaf(np.asarray(hssA.D).T.copy(), cp(hssA.V), cp(hssA.U), rootnode=hssA.rootnode)
    return HssMatrix.branch(transpose(hssA.A11), transpose(hssA.A22), hssA.B21.T.copy(), hssA.B12.T.copy(),
                            R1=hssA.W1.copy(), W1=hssA.R1.copy(), R2=hssA.W2.copy(), W2=hssA.R2.copy(),
                            rootnode=hssA.rootnode)


def cluster_trees(hssA, r0=1, c0=1):
    """The row and column cluster trees of ``hssA`` (1-based ranges, as
    ``bisection_cluster`` makes them)."""
    from .hssmatrix import ClusterTree
    m, n = hssA.size()
    rc, cc = ClusterTree(r0, r0 + m - 1), ClusterTree(c0, c0 + n - 1)
    if hssA.isbranch():
        m1, n1 = hssA.A11.size()
        rc.left, cc.left = cluster_trees(hssA.A11, r0, c0)
        rc.right, cc.right = cluster_trees(hssA.A22, r0 + m1, c0 + n1)
    return rc, cc


def _div_tols(opts, kw):
    from .hssmatrix import HssOptions
    o = (opts or HssOptions.current()).copy(**{k: v for k, v in kw.items() if k in ("atol", "rtol")})
    return float(o.atol), float(o.rtol)


def hss_ldiv(hssA, hssB, opts=None, stats=None, device=False, **kw):
    """``hssA \\ hssB`` / ``ldiv!(hssA, hssB)`` (src/hssmatrix.jl:235,
    src/ulvdivide.jl:13-54) on the device (``hss_ldiv``): the reference's
    recursion on the generators -- A's leaves reduced with its FP64 ULV
    factorization, the same transforms applied to B's leaf rows, the remainder
    recompressed to (atol, rtol) and pruned level by level, the root block
    solved, the solution unpacked back up with recompression.  Memory is
    O(n k) per level; no dense n x n block is formed.  Returns an HssMatrix on
    B's column clusters (or the DeviceHss handle with ``device=True``)."""
    (am, an), (bm, _bn) = hssA.size(), hssB.size()
    if am != an:
        raise ValueError("hssA must be square")
    if bm != am:
        raise ValueError("DimensionMismatch: rows of hssB must match hssA")
    atol, rtol = _div_tols(opts, kw)
    a, b = hssA.device(), hssB.device()
    h = C.c_void_p()
    check(a.lib.hss_ldiv(a.handle, b.handle, atol, rtol, C.byref(h), _stream(None)))
    dev = DeviceHss(_handle=h)
    if stats is not None:
        stats.update(hssrank=dev_rank(dev))
    return dev if device else dev.to_host()


def rdiv(hssB, hssA, opts=None, stats=None, device=False, **kw):
    """``hssB / hssA``: for an HssMatrix hssB, ``rdiv!`` = adjoint(hssA' \\ hssB')
    (src/hssmatrix.jl:237, src/ulvdivide.jl:15-17) on the device
    (``hss_rdiv``: the adjoints made on the device); for a dense B,
    ``B / hssA`` = (hssA' \\ B')' (src/hssmatrix.jl:236) with the FP64 ULV
    factorization of the device adjoint."""
    from .hssmatrix import HssMatrix
    (am, an) = hssA.size()
    if am != an:
        raise ValueError("hssA must be square")
    if not isinstance(hssB, HssMatrix):
        B = np.asarray(hssB, dtype=np.float64)
        vec = B.ndim == 1
        B2 = B.reshape(1, -1) if vec else B
        if B2.shape[1] != an:
            raise ValueError("DimensionMismatch: columns of B must match hssA")
        a = hssA.device()
        # B' as a column-major array is B's rows: a host layout change only
        Bt = np.asfortranarray(B2.T)
        at = a.transpose()
        Xt = at.ulvfactor("fp64").solve(Bt)
        X = np.asarray(Xt).T
        return X.reshape(-1) if vec else X
    (_bm, bn) = hssB.size()
    if bn != am:
        raise ValueError("DimensionMismatch: columns of hssB must match hssA")
    atol, rtol = _div_tols(opts, kw)
    a, b = hssA.device(), hssB.device()
    h = C.c_void_p()
    check(a.lib.hss_rdiv(b.handle, a.handle, atol, rtol, C.byref(h), _stream(None)))
    dev = DeviceHss(_handle=h)
    if stats is not None:
        stats.update(hssrank=dev_rank(dev))
    return dev if device else dev.to_host()


def rmatmul(A, hssB):
    """``A * hssB`` for a dense A (src/matmul.jl:14): (hssB' * A')' with the
    product by the adjoint on the device (``hss_matmul_t``)."""
    import torch
    dev = hssB.device()
    A = np.asarray(A, dtype=np.float64)
    vec = A.ndim == 1
    A2 = A.reshape(1, -1) if vec else A
    if A2.shape[1] != dev.m:
        raise ValueError("DimensionMismatch: columns of A must match rows of hssB")
    p = A2.shape[0]
    # A' (m x p, column-major) is A's rows, i.e. A row-major: a p x m tensor
    dAt = torch.from_numpy(np.ascontiguousarray(A2)).cuda()
    dCt = torch.empty((p, dev.n), dtype=torch.float64, device="cuda")
    dev.matmul_device(dAt, dev.m, p, dCt, dev.n, trans=True, stream=torch.cuda.current_stream())
    out = dCt.cpu().numpy()     # row-major p x n = C
    return out.reshape(-1) if vec else out


def dev_rank(dev):
    """``hssrank`` of a device handle from its node table."""
    table, _packed = dev.export()
    return int(max(table[:, 4].max(initial=0), table[:, 5].max(initial=0)))
