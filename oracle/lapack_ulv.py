"""ULV factor + solve transcribed over the LAPACK routines the reference calls -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` may import this module; the product never does.

The reference's ``ulvfactsolve`` (src/ulvfactor.jl:10-107) is Julia code over
``LinearAlgebra.LAPACK``: ``geqlf!``/``ormql!`` for the QL factorization of the
row generator U (:39-42), ``gelqf!``/``ormlq!`` for the LQ factorization of the
top block of D (:44, :47, :50, :102), BLAS ``trsm`` (:48) and ``D \\ b`` at the
root (:83, LU with partial pivoting: ``getrf``/``getrs``).  Julia links those
to OpenBLAS.  This module calls the same Fortran routines (``dgeqlf``,
``dormql``, ``dgelqf``, ``dormlq``, ``dtrsm``, ``dgetrf``, ``dgetrs``) from the
OpenBLAS build that SciPy ships, through ctypes, in the order and with the
arguments of ulvfactor.jl.  It is the reference's numerical floor without
Julia: the restatement in ``hss_oracle.py`` (QL as a reversed QR, LQ as the
QR of the transpose) is checked against it.
"""
from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np

_LIB = None
_PREFIX = ""


def _load():
    """The OpenBLAS library bundled with SciPy (LP64, symbols ``scipy_<name>_``)."""
    global _LIB, _PREFIX
    if _LIB is not None:
        return _LIB
    import scipy
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    cands += sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), ".dylibs", "libscipy_openblas*")))
    for path in cands:
        try:
            lib = C.CDLL(path)
        except OSError:
            continue
        for pre in ("scipy_", ""):
            if hasattr(lib, pre + "dgeqlf_") and hasattr(lib, pre + "dormlq_"):
                _LIB, _PREFIX = lib, pre
                return lib
    raise OSError("no OpenBLAS with dgeqlf/dgelqf/dormql/dormlq found next to SciPy")


def available() -> bool:
    try:
        _load()
        return True
    except OSError:
        return False


def _fn(name):
    return getattr(_load(), _PREFIX + name + "_")


_I = C.c_int
_Ip = C.POINTER(C.c_int)
_Dp = C.POINTER(C.c_double)
_L = C.c_size_t   # hidden Fortran character lengths


def _i(v):
    return C.byref(_I(int(v)))


def _ptr(a):
    return a.ctypes.data_as(_Dp)


def _ch(c):
    return C.c_char_p(c.encode())


def _fortran(a):
    return np.array(a, dtype=np.float64, order="F", copy=True)


def _check(info, name):
    if info.value != 0:
        raise RuntimeError(f"{name} returned info = {info.value}")


def geqlf(A):
    """``LAPACK.geqlf!(A)``: (A overwritten with L and the reflectors, tau)."""
    A = _fortran(A)
    m, n = A.shape
    k = min(m, n)
    tau = np.zeros(k)
    info = _I(0)
    if k == 0:
        return A, tau
    work = np.zeros(max(1, 64 * n))
    _fn("dgeqlf")(_i(m), _i(n), _ptr(A), _i(max(1, m)), _ptr(tau), _ptr(work), _i(work.size), C.byref(info))
    _check(info, "dgeqlf")
    return A, tau


def gelqf(A):
    """``LAPACK.gelqf!(A)``: (A overwritten with L and the reflectors, tau)."""
    A = _fortran(A)
    m, n = A.shape
    k = min(m, n)
    tau = np.zeros(k)
    info = _I(0)
    if k == 0:
        return A, tau
    work = np.zeros(max(1, 64 * m))
    _fn("dgelqf")(_i(m), _i(n), _ptr(A), _i(max(1, m)), _ptr(tau), _ptr(work), _i(work.size), C.byref(info))
    _check(info, "dgelqf")
    return A, tau


def _orm(name, side, trans, A, tau, Cm):
    Cm = _fortran(Cm)
    m, n = Cm.shape
    k = tau.size
    if m == 0 or n == 0 or k == 0:
        return Cm
    info = _I(0)
    work = np.zeros(max(1, 64 * max(m, n)))
    lda = max(1, A.shape[0])
    _fn(name)(_ch(side), _ch(trans), _i(m), _i(n), _i(k), _ptr(A), _i(lda), _ptr(tau), _ptr(Cm), _i(max(1, m)),
              _ptr(work), _i(work.size), C.byref(info), _L(1), _L(1))
    _check(info, name)
    return Cm


def ormql(side, trans, A, tau, Cm):
    """``LAPACK.ormql!(side, trans, A, tau, C)``."""
    return _orm("dormql", side, trans, A, tau, Cm)


def ormlq(side, trans, A, tau, Cm):
    """``LAPACK.ormlq!(side, trans, A, tau, C)``."""
    return _orm("dormlq", side, trans, A, tau, Cm)


def trsm_llnn(A, B):
    """``BLAS.trsm('L', 'L', 'N', 'N', 1.0, A, B)`` (a new matrix, as Julia's ``trsm``)."""
    B = _fortran(B)
    A = _fortran(A)
    m, n = B.shape
    if m == 0 or n == 0:
        return B
    one = C.c_double(1.0)
    _fn("dtrsm")(_ch("L"), _ch("L"), _ch("N"), _ch("N"), _i(m), _i(n), C.byref(one), _ptr(A), _i(max(1, A.shape[0])),
                 _ptr(B), _i(max(1, m)), _L(1), _L(1), _L(1), _L(1))
    return B


def lu_solve(A, B):
    """``A \\ B`` for a square dense A: ``getrf`` (partial pivoting) then ``getrs``."""
    A = _fortran(A)
    B = _fortran(B)
    n = A.shape[0]
    if n == 0:
        return B
    ipiv = np.zeros(n, dtype=np.int32)
    info = _I(0)
    _fn("dgetrf")(_i(n), _i(n), _ptr(A), _i(n), ipiv.ctypes.data_as(_Ip), C.byref(info))
    if info.value > 0:
        raise np.linalg.LinAlgError("singular root block")
    _check(info, "dgetrf")
    _fn("dgetrs")(_ch("N"), _i(n), _i(B.shape[1]), _ptr(A), _i(n), ipiv.ctypes.data_as(_Ip), _ptr(B),
                  _i(max(1, n)), C.byref(info), _L(1))
    _check(info, "dgetrs")
    return B


# ---------------------------------------------------------------------------
# src/ulvfactor.jl transcribed (Float64: adj = 'T')
# ---------------------------------------------------------------------------


def ulvfactsolve(h, b):
    """``ulvfactsolve(hssA, b::Matrix)`` (src/ulvfactor.jl:10-19) for an oracle HssMatrix."""
    b = np.asarray(b, dtype=np.float64)
    if b.ndim == 1:
        b = b.reshape(-1, 1)
    if h.leafnode:
        return lu_solve(h.D, b)                                          # :12
    z = np.zeros((h.size()[1], b.shape[1]), order="F")                  # :14
    *_, QV = _ulvfactsolve(h, b.copy(order="F"), z, 0, rootnode=True)   # :15
    _topdown(QV, z)                                                      # :16
    return z


def _ulvreduce(D, U, V, b):
    """``_ulvreduce!(D, U, V, b)`` (src/ulvfactor.jl:22-57)."""
    m, n = D.shape
    k = min(U.shape[1], m)                                               # :27
    nk = min(m - k, n)                                                   # :28
    if k >= m:                                                           # :32-36
        return D, U, V, b, np.zeros((0, b.shape[1])), np.zeros((V.shape[1], b.shape[1])), m - k, nk, None
    qA, qtau = geqlf(U)                                                  # :39
    U = np.tril(qA[m - k:, :])                                           # :40
    D = ormql("L", "T", qA, qtau, D)                                     # :41
    b = ormql("L", "T", qA, qtau, b)                                     # :42
    lA, ltau = gelqf(D[:m - k, :])                                       # :44
    L1 = np.tril(lA)[:, :nk]                                             # :45-46
    L2 = ormlq("R", "T", lA, ltau, D[m - k:, :])                         # :47
    zloc = trsm_llnn(L1, b[:m - k, :])                                   # :48
    b = b[m - k:, :] - L2[:, :nk] @ zloc                                 # :49
    V = ormlq("L", "N", lA, ltau, V)                                     # :50
    u = V[:m - k, :].T @ zloc                                            # :51
    D = L2[:, nk:]                                                       # :53
    V = V[nk:, :]                                                        # :54
    return D, U, V, b, zloc, u, m - k, nk, (lA, ltau)


class _Node:
    __slots__ = ("data", "left", "right")

    def __init__(self, data=None):
        self.data, self.left, self.right = data, None, None


def _ulvfactsolve(h, b, z, co, rootnode=False):
    """``_ulvfactsolve!`` (src/ulvfactor.jl:60-96), 0-based ``cols``."""
    if h.leafnode:
        cols = co + np.arange(h.size()[1])                               # :62
        D, U, V, b, zloc, u, mk, nk, lqf = _ulvreduce(h.D.copy(), h.U.copy(), h.V.copy(), b)  # :63-64
        z[cols[:mk], :] = zloc                                           # :65
        return b, u, D, U, V, cols, nk, _Node((cols,) + lqf if lqf else None)
    m1, n1 = h.sz1
    b1, b2 = b[:m1, :].copy(), b[m1:, :].copy()                          # :69
    b1, u1, D1, U1, V1, cols1, nk1, QV1 = _ulvfactsolve(h.A11, b1, z, co)
    b2, u2, D2, U2, V2, cols2, nk2, QV2 = _ulvfactsolve(h.A22, b2, z, co + n1)
    b = np.vstack([b1, b2]) - np.vstack([U1 @ h.B12 @ u2, U2 @ h.B21 @ u1])   # :74
    D = np.block([[D1, U1 @ h.B12 @ V2.T], [U2 @ h.B21 @ V1.T, D2]])          # :75
    cols = np.concatenate([cols1[nk1:], cols2[nk2:]])                          # :76
    U = np.vstack([U1 @ h.R1, U2 @ h.R2])                                      # :78
    V = np.vstack([V1 @ h.W1, V2 @ h.W2])                                      # :79
    if rootnode:                                                               # :82-86
        z[cols, :] = lu_solve(D, b)
        u = np.zeros((0, b.shape[1]))
        nk = D.shape[1]
        QV = _Node()
    else:                                                                      # :87-91
        D, U, V, b, zloc, u, mk, nk, lqf = _ulvreduce(D, U, V, b)
        u = u + h.W1.T @ u1 + h.W2.T @ u2
        z[cols[:mk], :] = zloc
        QV = _Node((cols,) + lqf if lqf else None)
    QV.left, QV.right = QV1, QV2
    return b, u, D, U, V, cols, nk, QV


def _topdown(QV, z):
    """``_ulvfactsolve_topdown!`` (src/ulvfactor.jl:98-107)."""
    if QV.data is not None:
        cols, Q, tau = QV.data
        z[cols, :] = ormlq("L", "T", Q, tau, z[cols, :])                 # :102
    if QV.left is not None:
        _topdown(QV.left, z)
    if QV.right is not None:
        _topdown(QV.right, z)
