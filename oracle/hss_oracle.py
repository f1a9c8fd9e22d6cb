"""CPU restatement of the HssMatrices.jl hot path -- TEST INFRASTRUCTURE ONLY.

This module is the correctness oracle.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it; the product (the CUDA
library and its host package) never does.

It restates, in NumPy + LAPACK (``scipy.linalg.lapack.dgeqrf/dormqr``), the
algorithms of the reference (file:line within bonevbs/HssMatrices.jl v0.1.6):

* cluster trees            -- src/clustertree.jl:14-35 (``bisection_cluster``)
* the HSS generator tree    -- src/hssmatrix.jl:11-67 (leaf D,U,V / branch
                              A11,A22,B12,B21,R1,W1,R2,W2), ``size`` :94,
                              ``gensize`` :254-262, ``hssrank`` :251,
                              ``rooted`` :266, ``full`` :270-305
* HSS x dense product       -- src/matmul.jl:13-62 (``mul!``, ``_matmatup``,
                              ``_matmatdown!``)
* implicit ULV factor+solve -- src/ulvfactor.jl:10-107 (``ulvfactsolve``,
                              ``_ulvreduce!``, ``_ulvfactsolve!``,
                              ``_ulvfactsolve_topdown!``)
* deterministic compression -- src/compression.jl:22-133 (``compress``)
* randomized compression    -- src/compression.jl:278-475 (``randcompress``,
                              ``randcompress_adaptive``, ``_randcompress!``,
                              ``_interpolate``, ``hss_blkdiag``)

LAPACK conventions.  The reference calls ``geqlf!/ormql!`` (QL of U) and
``gelqf!/ormlq!`` (LQ of the top block of D).  SciPy does not wrap those, so:
QL of U is the QR (``dgeqrf``) of U with rows and columns reversed, and the LQ
of X is the QR of X^T.  Both generate the same Householder reflectors as the
LAPACK routines (``dlarfg`` on the same vectors), so results agree to rounding.

Parity status.  Julia is not available, and the reference's test-suite holds no
golden vectors (tolerance-only checks, unseeded ``randn``), so bit-level parity
with the reference is UNPINNED.  What is pinned: the reference's own tolerance
tests (test/runtests.jl:36-67) pass on this restatement, on the same fixtures,
and the integer cluster-tree bookkeeping is restated exactly.  The rank rule of
``LowRankApprox.pqrfact`` (a dependency absent from the reference tree) is
restated from its documented behaviour (stop when either atol or rtol is met,
README.md:43), so compressed ranks are unpinned too.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack

# ---------------------------------------------------------------------------
# options (src/HssMatrices.jl:52-108)
# ---------------------------------------------------------------------------


@dataclass
class HssOptions:
    """Restates ``HssOptions`` and its defaults (src/HssMatrices.jl:52-67)."""

    atol: float = 1e-9
    rtol: float = 1e-9
    leafsize: int = 64
    noversampling: int = 10
    stepsize: int = 20
    verbose: bool = False

    def check(self):
        """``chkopts!`` (src/HssMatrices.jl:90-96)."""
        if not self.atol >= 0.0:
            raise ValueError("atol")
        if not self.rtol >= 0.0:
            raise ValueError("rtol")
        if not self.leafsize >= 1:
            raise ValueError("leafsize")
        if not self.stepsize >= 1:
            raise ValueError("stepsize")
        if not self.noversampling >= 1:
            raise ValueError("noversampling")
        return self


# ---------------------------------------------------------------------------
# cluster trees (src/binarytree.jl:7-54, src/clustertree.jl:14-35)
# ---------------------------------------------------------------------------


@dataclass
class ClusterTree:
    """A ``BinaryNode{UnitRange{Int}}``; ``lo``/``hi`` are 1-based inclusive, as in Julia."""

    lo: int
    hi: int
    left: Optional["ClusterTree"] = None
    right: Optional["ClusterTree"] = None

    def __len__(self):
        return self.hi - self.lo + 1

    def isleaf(self):
        return self.left is None and self.right is None


def bisection_cluster(n, leafsize: int = 64) -> ClusterTree:
    """``bisection_cluster(1:n; leafsize)`` (src/clustertree.jl:14-20, 27-35).

    ``n`` is an int (range 1:n) or a (lo, hi) 1-based inclusive pair.
    Split point ``ceil(len/2)`` (:30), leaf when ``len <= leafsize`` (:29).
    """
    if leafsize < 1:
        raise ValueError("leafsize")
    lo, hi = (1, n) if isinstance(n, (int, np.integer)) else n
    if hi - lo + 1 <= 0:
        raise ValueError("Index range must be larger or equal to 0")
    return _bisection_cluster(lo, hi, leafsize)


def _bisection_cluster(lo, hi, leafsize):
    node = ClusterTree(lo, hi)
    length = hi - lo + 1
    if length > leafsize:
        h = (length + 1) // 2  # convert(Int, ceil(size(range,1)/2))
        node.left = _bisection_cluster(lo, lo + h - 1, leafsize)
        node.right = _bisection_cluster(lo + h, hi, leafsize)
    return node


def cluster_leaves(t: ClusterTree):
    """Leaf ranges in pre-order (list of (lo, hi) 1-based)."""
    if t.isleaf():
        return [(t.lo, t.hi)]
    return cluster_leaves(t.left) + cluster_leaves(t.right)


def cluster_depth(t: ClusterTree):
    """``depth`` (src/binarytree.jl:27-40)."""
    if t.isleaf():
        return 1
    return 1 + max(cluster_depth(t.left), cluster_depth(t.right))


def compatible(a: ClusterTree, b: ClusterTree):
    """``compatible`` (src/binarytree.jl:68-74): same branching structure."""
    if a.isleaf() and b.isleaf():
        return True
    if a.isleaf() or b.isleaf():
        return False
    return compatible(a.left, b.left) and compatible(a.right, b.right)


# ---------------------------------------------------------------------------
# HSS generator tree (src/hssmatrix.jl:11-67)
# ---------------------------------------------------------------------------


class HssMatrix:
    """Restates ``mutable struct HssMatrix`` (src/hssmatrix.jl:11-67).

    Leaf: ``D`` (m x n), ``U`` (m x ku), ``V`` (n x kv).
    Branch: ``A11``, ``A22``, ``B12`` (ku1 x kv2), ``B21`` (ku2 x kv1),
    ``R1`` (ku1 x kR), ``R2`` (ku2 x kR), ``W1`` (kv1 x kW), ``W2`` (kv2 x kW);
    at the root R/W have zero columns (:52-53).
    """

    def __init__(self):
        self.leafnode = True
        self.rootnode = True
        self.D = self.U = self.V = None
        self.A11 = self.A22 = None
        self.B12 = self.B21 = None
        self.R1 = self.W1 = self.R2 = self.W2 = None
        self.sz1 = self.sz2 = None

    @classmethod
    def leaf(cls, D, U=None, V=None, rootnode=None):
        """Leaf constructors (src/hssmatrix.jl:36-44)."""
        h = cls()
        D = np.asarray(D, dtype=float)
        m, n = D.shape
        h.leafnode = True
        if U is None:
            h.rootnode = True if rootnode is None else rootnode
            U = np.zeros((m, 0))
            V = np.zeros((n, 0))
        else:
            h.rootnode = False if rootnode is None else rootnode
            if U.shape[0] != m:
                raise ValueError("D and U must have same number of rows")
            if V.shape[0] != n:
                raise ValueError("D and V must have same number of columns")
        h.D, h.U, h.V = D, np.asarray(U, float), np.asarray(V, float)
        return h

    @classmethod
    def branch(cls, A11, A22, B12, B21, R1=None, W1=None, R2=None, W2=None, rootnode=None):
        """Branch constructors (src/hssmatrix.jl:46-67)."""
        h = cls()
        h.leafnode = False
        h.A11, h.A22 = A11, A22
        h.B12, h.B21 = np.asarray(B12, float), np.asarray(B21, float)
        h.sz1, h.sz2 = A11.size(), A22.size()
        if R1 is None:
            h.rootnode = True if rootnode is None else rootnode
            kr1, kw1 = gensize(A11)
            kr2, kw2 = gensize(A22)
            h.R1, h.W1 = np.zeros((kr1, 0)), np.zeros((kw1, 0))
            h.R2, h.W2 = np.zeros((kr2, 0)), np.zeros((kw2, 0))
        else:
            h.rootnode = False if rootnode is None else rootnode
            if R1.shape[1] != R2.shape[1]:
                raise ValueError("R1 and R2 must have same number of columns")
            if W1.shape[1] != W2.shape[1]:
                raise ValueError("W1 and W2 must have same number of rows")
            h.R1, h.W1, h.R2, h.W2 = (np.asarray(x, float) for x in (R1, W1, R2, W2))
        return h

    def isleaf(self):
        return self.leafnode

    def size(self):
        """``size`` (src/hssmatrix.jl:94)."""
        if self.leafnode:
            return self.D.shape
        return (self.sz1[0] + self.sz2[0], self.sz1[1] + self.sz2[1])

    @property
    def shape(self):
        return self.size()


def gensize(h: HssMatrix):
    """``gensize`` (src/hssmatrix.jl:254-262): (#cols of U or R, #cols of V or W)."""
    if h.leafnode:
        return h.U.shape[1], h.V.shape[1]
    kr = h.R1.shape[1]
    if kr != h.R2.shape[1]:
        raise ValueError("dimensions of column-translators do not match")
    kw = h.W1.shape[1]
    if kw != h.W2.shape[1]:
        raise ValueError("dimensions of row-translators do not match")
    return kr, kw


def hssrank(h: HssMatrix):
    """``hssrank`` (src/hssmatrix.jl:251)."""
    if h.leafnode:
        return 0
    return max(hssrank(h.A11), hssrank(h.A22), *h.B12.shape, *h.B21.shape)


def rooted(h: HssMatrix):
    """``rooted`` (src/hssmatrix.jl:266): same node with zero-column top translators."""
    if h.leafnode:
        return HssMatrix.leaf(h.D, rootnode=True)
    return HssMatrix.branch(h.A11, h.A22, h.B12, h.B21, rootnode=True)


def full(h: HssMatrix):
    """``full`` / ``_full!`` (src/hssmatrix.jl:270-305)."""
    if h.leafnode:
        return h.D.copy()
    m, n = h.size()
    A = np.zeros((m, n))
    k = max(hssrank(h), 1)
    U = np.zeros((m, k + 1))
    V = np.zeros((n, k + 1))
    _full(h, A, U, V, 0, 0, True)
    return A


def _full(h, A, U, V, ro, co, rootnode):
    if h.leafnode:
        m, n = h.D.shape
        A[ro:ro + m, co:co + n] = h.D
        U[ro:ro + m, :h.U.shape[1]] = h.U
        V[co:co + n, :h.V.shape[1]] = h.V
        return
    m1, n1 = h.sz1
    m2, n2 = h.sz2
    ru1, rv1 = gensize(h.A11)
    ru2, rv2 = gensize(h.A22)
    _full(h.A11, A, U, V, ro, co, False)
    _full(h.A22, A, U, V, ro + m1, co + n1, False)
    A[ro:ro + m1, co + n1:co + n1 + n2] = U[ro:ro + m1, :ru1] @ h.B12 @ V[co + n1:co + n1 + n2, :rv2].T
    A[ro + m1:ro + m1 + m2, co:co + n1] = U[ro + m1:ro + m1 + m2, :ru2] @ h.B21 @ V[co:co + n1, :rv1].T
    if not rootnode:
        u1 = U[ro:ro + m1, :ru1] @ h.R1
        u2 = U[ro + m1:ro + m1 + m2, :ru2] @ h.R2
        v1 = V[co:co + n1, :rv1] @ h.W1
        v2 = V[co + n1:co + n1 + n2, :rv2] @ h.W2
        U[ro:ro + m1, :u1.shape[1]] = u1
        U[ro + m1:ro + m1 + m2, :u2.shape[1]] = u2
        V[co:co + n1, :v1.shape[1]] = v1
        V[co + n1:co + n1 + n2, :v2.shape[1]] = v2


def hssmul(A: HssMatrix, B: HssMatrix):
    """``*(hssA::HssMatrix, hssB::HssMatrix)`` (src/matmul.jl:65-84): the HSS
    product of two matrices on matching cluster trees, ranks adding up
    (no recompression).  The reference tests ``isleaf(hssA)`` twice (:66, :68);
    on matching trees that is the same as testing both."""
    if A.leafnode and B.leafnode:
        return HssMatrix.leaf(A.D @ B.D, A.U, B.V, rootnode=True)
    if A.leafnode or B.leafnode:
        raise ValueError("Clusters don't seem to match")
    A, B = rooted(A), rooted(B)
    Z = _hmm_up(A, B)
    F1 = A.B12 @ Z[2][0] @ B.B21
    F2 = A.B21 @ Z[1][0] @ B.B12
    B12 = _blkdiag(A.B12, B.B12)
    B21 = _blkdiag(A.B21, B.B21)
    C11 = _hmm_down(A.A11, B.A11, Z[1], F1)
    C22 = _hmm_down(A.A22, B.A22, Z[2], F2)
    return HssMatrix.branch(C11, C22, B12, B21, rootnode=True)


def _blkdiag(X, Y):
    out = np.zeros((X.shape[0] + Y.shape[0], X.shape[1] + Y.shape[1]))
    out[:X.shape[0], :X.shape[1]] = X
    out[X.shape[0]:, X.shape[1]:] = Y
    return out


def _hmm_up(A, B):
    """``_matmatup(hssA, hssB)`` (src/matmul.jl:86-94): (Z, left, right) tree."""
    if A.leafnode and B.leafnode:
        return (A.V.T @ B.U, None, None)
    if A.leafnode or B.leafnode:
        raise ValueError("Clusters don't seem to match")
    Z1 = _hmm_up(A.A11, B.A11)
    Z2 = _hmm_up(A.A22, B.A22)
    return (A.W1.T @ Z1[0] @ B.R1 + A.W2.T @ Z2[0] @ B.R2, Z1, Z2)


def _hmm_down(A, B, Z, F):
    """``_matmatdown!(hssA, hssB, Z, F)`` (src/matmul.jl:96-117)."""
    if A.leafnode and B.leafnode:
        D = A.D @ B.D + A.U @ F @ B.V.T
        U = np.hstack([A.U, A.D @ B.U])
        V = np.hstack([B.D.T @ A.V, B.V])
        return HssMatrix.leaf(D, U, V, rootnode=False)
    if A.leafnode or B.leafnode:
        raise ValueError("Clusters don't seem to match")
    Zl, Zr = Z[1][0], Z[2][0]
    F1 = A.B12 @ Zr @ B.B21 + A.R1 @ F @ B.W1.T
    F2 = A.B21 @ Zl @ B.B12 + A.R2 @ F @ B.W2.T
    B12 = np.block([[A.B12, A.R1 @ F @ B.W2.T], [np.zeros((B.B12.shape[0], A.B12.shape[1])), B.B12]])
    B21 = np.block([[A.B21, A.R2 @ F @ B.W1.T], [np.zeros((B.B21.shape[0], A.B21.shape[1])), B.B21]])
    R1 = np.block([[A.R1, A.B12 @ Zr @ B.R2], [np.zeros((B.R1.shape[0], A.R1.shape[1])), B.R1]])
    W1 = np.block([[A.W1, np.zeros((A.W1.shape[0], B.W1.shape[1]))], [B.B21.T @ Zr.T @ A.W2, B.W1]])
    R2 = np.block([[A.R2, A.B21 @ Zl @ B.R1], [np.zeros((B.R2.shape[0], A.R2.shape[1])), B.R2]])
    W2 = np.block([[A.W2, np.zeros((A.W2.shape[0], B.W2.shape[1]))], [B.B12.T @ Zl.T @ A.W1, B.W2]])
    C11 = _hmm_down(A.A11, B.A11, Z[1], F1)
    C22 = _hmm_down(A.A22, B.A22, Z[2], F2)
    return HssMatrix.branch(C11, C22, B12, B21, R1, W1, R2, W2, rootnode=False)


def getindex(h: HssMatrix, i, j):
    """``getindex(hssA, i::Vector, j::Vector)`` (src/hssmatrix.jl:108-114):
    sort both index lists, restrict the tree to them (``_getidx``, :117-128),
    expand with ``full`` and undo the sorting.  0-based indices here."""
    i = np.asarray(i, dtype=np.int64).ravel()
    j = np.asarray(j, dtype=np.int64).ravel()
    if i.size == 0 or j.size == 0:
        return np.zeros((i.size, j.size))
    ip = np.argsort(i, kind="stable")
    jp = np.argsort(j, kind="stable")
    sub = full(_getidx(h, i[ip], j[jp]))
    out = np.empty_like(sub)
    out[np.ix_(ip, jp)] = sub      # sub[invperm(ip), invperm(jp)]
    return out


def _getidx(h: HssMatrix, i, j):
    """``_getidx(hssA, i::Vector, j::Vector)`` (src/hssmatrix.jl:117-128): the
    HSS matrix of the selected (sorted) rows and columns."""
    if h.leafnode:
        x = HssMatrix.leaf(h.D[np.ix_(i, j)], h.U[i, :], h.V[j, :], rootnode=h.rootnode)
        return x
    m1, n1 = h.sz1
    i1, j1 = i[i < m1], j[j < n1]
    i2, j2 = i[i >= m1] - m1, j[j >= n1] - n1
    A11 = _getidx(h.A11, i1, j1)
    A22 = _getidx(h.A22, i2, j2)
    return HssMatrix.branch(A11, A22, h.B12, h.B21, h.R1, h.W1, h.R2, h.W2, rootnode=h.rootnode)


def adjoint(h: HssMatrix):
    """``adjoint`` (src/hssmatrix.jl:165-171) for real matrices."""
    if h.leafnode:
        return HssMatrix.leaf(h.D.T.copy(), h.V.copy(), h.U.copy(), rootnode=h.rootnode) if not (
            h.rootnode and h.U.shape[1] == 0 and h.V.shape[1] == 0) else HssMatrix.leaf(h.D.T.copy(), rootnode=True)
    out = HssMatrix.branch(adjoint(h.A11), adjoint(h.A22), h.B21.T.copy(), h.B12.T.copy(),
                           h.W1.copy(), h.R1.copy(), h.W2.copy(), h.R2.copy(), rootnode=h.rootnode)
    return out


def iter_nodes(h: HssMatrix):
    """Pre-order traversal."""
    yield h
    if not h.leafnode:
        yield from iter_nodes(h.A11)
        yield from iter_nodes(h.A22)


def generator_entries(h: HssMatrix):
    """Number of stored generator entries (D, U, V, R, W, B) in the tree."""
    tot = 0
    for x in iter_nodes(h):
        if x.leafnode:
            tot += x.D.size + x.U.size + x.V.size
        else:
            tot += x.B12.size + x.B21.size + x.R1.size + x.R2.size + x.W1.size + x.W2.size
    return tot


# ---------------------------------------------------------------------------
# HSS x dense (src/matmul.jl:13-62)
# ---------------------------------------------------------------------------


def matmul(h: HssMatrix, B, alpha=1.0, beta=0.0, C=None):
    """``mul!(C, hssA, B, alpha, beta)`` (src/matmul.jl:18-28); ``*`` (:13-15) when C is None."""
    B = np.asarray(B, dtype=float)
    vec = B.ndim == 1
    if vec:
        B = B.reshape(-1, 1)
    m, n = h.size()
    if B.shape[0] != n:
        raise ValueError("First dimension of B does not match second dimension of A")
    if C is None:
        C = np.zeros((m, B.shape[1]))
        beta = 0.0
    else:
        C = np.array(C, dtype=float, copy=True).reshape(m, B.shape[1])
    if C.shape != (m, B.shape[1]):
        raise ValueError("Dimensions of C don't match up with A and B.")
    if h.leafnode:
        C[:] = alpha * (h.D @ B) + beta * C
    else:
        h = rooted(h)
        Z = _matmatup(h, B)
        _matmatdown(C, h, B, Z, None, alpha, beta)
    return C.reshape(-1) if vec else C


class _ZNode:
    __slots__ = ("data", "left", "right")

    def __init__(self, data, left=None, right=None):
        self.data, self.left, self.right = data, left, right


def _matmatup(h, B):
    """Post-order sweep (src/matmul.jl:32-42): leaf V'B, branch W1'Z1 + W2'Z2."""
    if h.leafnode:
        return _ZNode(h.V.T @ B)
    n1 = h.sz1[1]
    Z1 = _matmatup(h.A11, B[:n1])
    Z2 = _matmatup(h.A22, B[n1:])
    return _ZNode(h.W1.T @ Z1.data + h.W2.T @ Z2.data, Z1, Z2)


def _matmatdown(C, h, B, Z, F, alpha, beta):
    """Pre-order sweep (src/matmul.jl:44-62)."""
    if h.leafnode:
        C[:] = alpha * (h.D @ B) + beta * C
        if F is not None:
            C += alpha * (h.U @ F)
        return
    m1, n1 = h.sz1
    if F is not None:
        F1 = h.B12 @ Z.right.data + h.R1 @ F
        F2 = h.B21 @ Z.left.data + h.R2 @ F
    else:
        F1 = h.B12 @ Z.right.data
        F2 = h.B21 @ Z.left.data
    _matmatdown(C[:m1], h.A11, B[:n1], Z.left, F1, alpha, beta)
    _matmatdown(C[m1:], h.A22, B[n1:], Z.right, F2, alpha, beta)


# ---------------------------------------------------------------------------
# LAPACK helpers: QL via reversed QR, LQ via QR of the transpose
# ---------------------------------------------------------------------------


def _geqrf(A):
    qr, tau, _work, info = lapack.dgeqrf(np.asfortranarray(A, dtype=float))
    if info != 0:
        raise RuntimeError("dgeqrf failed")
    return qr, tau


def _ormqr(side, trans, qr, tau, C):
    C = np.asfortranarray(C, dtype=float)
    if C.size == 0 or tau.size == 0:
        return np.array(C, copy=True)
    lwork = max(1, 64 * max(C.shape))
    out, _work, info = lapack.dormqr(side, trans, qr, tau, C, lwork)
    if info != 0:
        raise RuntimeError("dormqr failed")
    return out


class QLFact:
    """``geqlf!(U)`` of an m x k block (k < m): U = Q [0; L]."""

    def __init__(self, U):
        self.m, self.k = U.shape
        self.qr, self.tau = _geqrf(U[::-1, ::-1])

    def L(self):
        R = np.triu(self.qr[:self.k, :self.k])
        return R[::-1, ::-1].copy()

    def apply_qt(self, C):
        """``ormql!('L', 'T', ...)``: C <- Q^T C."""
        return _ormqr("L", "T", self.qr, self.tau, C[::-1])[::-1].copy()


class LQFact:
    """``gelqf!(X)`` of an mk x n block: X = L Q (L = R^T, Q = Qqr^T of QR(X^T))."""

    def __init__(self, X):
        self.mk, self.n = X.shape
        self.qr, self.tau = _geqrf(X.T)

    def L(self):
        r = min(self.mk, self.n)
        return np.triu(self.qr[:r, :self.mk]).T.copy()  # mk x r lower trapezoidal

    def apply_right_qt(self, C):
        """``ormlq!('R', 'T', ...)``: C <- C Q^T."""
        return _ormqr("L", "T", self.qr, self.tau, C.T).T.copy()

    def apply_left_q(self, C):
        """``ormlq!('L', 'N', ...)``: C <- Q C."""
        return _ormqr("L", "T", self.qr, self.tau, C)

    def apply_left_qt(self, C):
        """``ormlq!('L', 'T', ...)``: C <- Q^T C."""
        return _ormqr("L", "N", self.qr, self.tau, C)


# ---------------------------------------------------------------------------
# implicit ULV factor + solve (src/ulvfactor.jl:10-107)
# ---------------------------------------------------------------------------


def ulvfactsolve(h: HssMatrix, b):
    """``ulvfactsolve(hssA, b)`` (src/ulvfactor.jl:10-19); ``hssA \\ b`` (src/hssmatrix.jl:234)."""
    b = np.asarray(b, dtype=float)
    vec = b.ndim == 1
    if vec:
        b = b.reshape(-1, 1)
    if h.leafnode:
        x = np.linalg.solve(h.D, b)
    else:
        z = np.zeros((h.size()[1], b.shape[1]))
        *_, QV = _ulvfactsolve(h, b.copy(), z, 0, rootnode=True)
        _ulvfactsolve_topdown(QV, z)
        x = z
    return x.reshape(-1) if vec else x


def _ulvreduce(D, U, V, b):
    """``_ulvreduce!(D, U, V, b)`` (src/ulvfactor.jl:22-57)."""
    m, n = D.shape
    if m != U.shape[0]:
        raise ValueError("D and U have different first dimensions")
    if n != V.shape[0]:
        raise ValueError("D and V have different second dimensions")
    r = b.shape[1]
    k = min(U.shape[1], m)
    nk = min(m - k, n)
    if k >= m:  # nothing can be eliminated (:32-36)
        u = np.zeros((V.shape[1], r))
        zloc = np.zeros((0, r))
        return D, U, V, b, zloc, u, m - k, nk, None
    qlf = QLFact(U)                                   # geqlf!(U)          :39
    U = np.tril(qlf.L())                              # tril(U[end-k+1:end,:]) :40
    D = qlf.apply_qt(D)                               # ormql!('L',T,..,D)  :41
    b = qlf.apply_qt(b)                               # ormql!('L',T,..,b)  :42
    lqf = LQFact(D[:m - k, :])                        # gelqf!(D[1:m-k,:])  :44
    L1 = lqf.L()[:, :nk]                              # tril(lqf[1])[:,1:nk] :45-46
    L2 = lqf.apply_right_qt(D[m - k:, :])             # ormlq!('R',T,..)    :47
    zloc = sla.solve_triangular(L1, b[:m - k], lower=True)  # trsm           :48
    b = b[m - k:] - L2[:, :nk] @ zloc                 # :49
    V = lqf.apply_left_q(V)                           # ormlq!('L','N',..,V) :50
    u = V[:m - k, :].T @ zloc                         # :51
    D = L2[:, nk:]                                    # :53
    V = V[nk:, :]                                     # :54
    return D, U, V, b, zloc, u, m - k, nk, lqf


class _QVNode:
    __slots__ = ("cols", "lqf", "left", "right")

    def __init__(self, cols=None, lqf=None):
        self.cols, self.lqf, self.left, self.right = cols, lqf, None, None


def _ulvfactsolve(h, b, z, co, rootnode=False):
    """``_ulvfactsolve!`` (src/ulvfactor.jl:60-96); ``cols`` are 0-based here."""
    if h.leafnode:
        cols = co + np.arange(h.size()[1], dtype=np.int64)           # :62
        D, U, V = h.D.copy(), h.U.copy(), h.V.copy()                   # :63
        D, U, V, b, zloc, u, mk, nk, lqf = _ulvreduce(D, U, V, b)     # :64
        z[cols[:mk]] = zloc                                            # :65
        QV = _QVNode(cols, lqf)                                        # :66
        return b, u, D, U, V, cols, nk, QV
    m1, n1 = h.sz1
    b1, b2 = b[:m1].copy(), b[m1:].copy()                              # :69
    b1, u1, D1, U1, V1, cols1, nk1, QV1 = _ulvfactsolve(h.A11, b1, z, co)
    b2, u2, D2, U2, V2, cols2, nk2, QV2 = _ulvfactsolve(h.A22, b2, z, co + n1)
    b = np.vstack([b1, b2]) - np.vstack([U1 @ h.B12 @ u2, U2 @ h.B21 @ u1])   # :74
    D = np.block([[D1, U1 @ h.B12 @ V2.T], [U2 @ h.B21 @ V1.T, D2]])          # :75
    cols = np.concatenate([cols1[nk1:], cols2[nk2:]])                          # :76
    U = np.vstack([U1 @ h.R1, U2 @ h.R2])                                      # :78
    V = np.vstack([V1 @ h.W1, V2 @ h.W2])                                      # :79
    if rootnode:                                                               # :82-86
        z[cols] = np.linalg.solve(D, b)
        u = np.zeros((0, b.shape[1]))
        QV = _QVNode()
        nk = D.shape[1]
    else:                                                                      # :87-91
        D, U, V, b, zloc, u, mk, nk, lqf = _ulvreduce(D, U, V, b)
        u = u + h.W1.T @ u1 + h.W2.T @ u2
        z[cols[:mk]] = zloc
        QV = _QVNode(cols, lqf)
    QV.left, QV.right = QV1, QV2
    return b, u, D, U, V, cols, nk, QV


def _ulvfactsolve_topdown(QV, z):
    """``_ulvfactsolve_topdown!`` (src/ulvfactor.jl:98-107): z[cols] = Q^T z[cols], pre-order."""
    if QV.cols is not None and QV.lqf is not None:
        z[QV.cols] = QV.lqf.apply_left_qt(z[QV.cols])
    if QV.left is not None:
        _ulvfactsolve_topdown(QV.left, z)
    if QV.right is not None:
        _ulvfactsolve_topdown(QV.right, z)


def ulv_cols(h: HssMatrix):
    """The per-node ``cols`` bookkeeping of ``_ulvfactsolve!`` (src/ulvfactor.jl:62,76),
    pre-order list of (cols, mk, nk) with 0-based column indices, root last entry
    being its full ``cols``.  Depends only on sizes and ranks, never on values."""
    out = []

    def rec(x, co, root):
        if x.leafnode:
            m, n = x.D.shape
            cols = co + np.arange(n, dtype=np.int64)
            k = min(x.U.shape[1], m)
            mk = m - k
            nk = min(mk, n)
            out.append((cols, mk, nk))
            return cols, nk, (k if k < m else m), x.V.shape[1], x.U.shape[1]
        m1, n1 = x.sz1
        idx = len(out)
        out.append(None)
        c1, nk1, mr1, kv1, ku1 = rec(x.A11, co, False)
        c2, nk2, mr2, kv2, ku2 = rec(x.A22, co + n1, False)
        cols = np.concatenate([c1[nk1:], c2[nk2:]])
        m = mr1 + mr2
        n = len(cols)
        if root:
            out[idx] = (cols, 0, 0)
            return cols, 0, m, 0, 0
        ku = x.R1.shape[1]
        k = min(ku, m)
        mk = m - k
        nk = min(mk, n)
        out[idx] = (cols, mk, nk)
        return cols, nk, (k if k < m else m), x.W1.shape[1], ku

    rec(h, 0, True)
    return out


# ---------------------------------------------------------------------------
# deterministic compression (src/compression.jl:22-133)
# ---------------------------------------------------------------------------


def _compress_block(A, atol, rtol):
    """``_compress_block!`` (src/compression.jl:22-30): truncated column-pivoted QR,
    returns (Q, R[:, invperm(p)]).  The rank rule restates ``LowRankApprox.pqrfact``'s
    documented tolerance (stop once atol or rtol is met): keep |R_ii| > max(atol, rtol*|R_11|)."""
    m, n = A.shape
    if m == 0 or n == 0:
        return np.zeros((m, 0)), np.zeros((0, n))
    Q, R, p = sla.qr(A, mode="economic", pivoting=True)
    d = np.abs(np.diag(R))
    thr = max(atol, rtol * d[0])
    rk = int(np.sum(d > thr)) if d[0] > 0 else 0
    inv = np.empty_like(p)
    inv[p] = np.arange(len(p))
    return Q[:, :rk].copy(), R[:rk, :][:, inv].copy()


# LowRankApprox's default relative tolerance for pqrfact without options
# (assumed: 5 eps; the package is not in the reference tree, so unpinned).
PQR_DEFAULT_RTOL = 5 * np.finfo(float).eps


def _pqr(A):
    """``pqrfact!(A, sketch=:none)`` with default tolerances: (Q, R P^T)."""
    return _compress_block(np.asarray(A, float), 0.0, PQR_DEFAULT_RTOL)


def orthonormalize_generators(h: HssMatrix):
    """``orthonormalize_generators!`` (src/generators.jl:64-114): every U and
    every stacked [R1; R2] (V, [W1; W2] likewise) replaced by the Q of its
    pivoted QR, the R factors moved into the parent's B, R and W.  In place."""
    if h.leafnode:
        return h
    def side(c):
        """(RU, RV) of child c after orthonormalizing it (R with columns unpermuted)."""
        if c.leafnode:
            QU, RU = _pqr(c.U)
            QV, RV = _pqr(c.V)
            c.U, c.V = QU, QV
            return RU, RV
        orthonormalize_generators(c)
        rm1, rn1 = c.R1.shape[0], c.W1.shape[0]
        QU, RU = _pqr(np.vstack([c.R1, c.R2]))
        QV, RV = _pqr(np.vstack([c.W1, c.W2]))
        c.R1, c.R2 = QU[:rm1, :], QU[rm1:, :]
        c.W1, c.W2 = QV[:rn1, :], QV[rn1:, :]
        return RU, RV
    RU1, RV1 = side(h.A11)
    RU2, RV2 = side(h.A22)
    h.B12 = RU1 @ h.B12 @ RV2.T
    h.B21 = RU2 @ h.B21 @ RV1.T
    h.R1 = RU1 @ h.R1
    h.R2 = RU2 @ h.R2
    h.W1 = RV1 @ h.W1
    h.W2 = RV2 @ h.W2
    return h


def _push(c, P, Q):
    """Children's generators after a parent's truncation (src/compression.jl:176-195)."""
    if c.leafnode:
        c.U = c.U @ P
        c.V = c.V @ Q
    else:
        c.R1, c.R2 = c.R1 @ P, c.R2 @ P
        c.W1, c.W2 = c.W1 @ Q, c.W2 @ Q


def recompress(h: HssMatrix, atol=1e-9, rtol=1e-9):
    """``recompress!`` (src/compression.jl:148-203): orthonormalize, then
    truncate the couplings top-down with ``_compress_block!``.  In place."""
    if h.leafnode:
        return h
    orthonormalize_generators(h)
    P1, S2 = _compress_block(h.B12, atol, rtol)
    Q2, T1 = _compress_block(h.B12.T.copy(), atol, rtol)
    P2, S1 = _compress_block(h.B21, atol, rtol)
    Q1, T2 = _compress_block(h.B21.T.copy(), atol, rtol)
    h.B12 = S2 @ Q2
    h.B21 = S1 @ Q1
    h.R1 = h.R1[:h.B12.shape[0], :]
    h.W1 = h.W1[:h.B21.shape[1], :]
    h.R2 = h.R2[:h.B21.shape[0], :]
    h.W2 = h.W2[:h.B12.shape[1], :]
    _push(h.A11, P1, Q1)
    _push(h.A22, P2, Q2)
    if not h.A11.leafnode:
        _recompress(h.A11, h.B12, h.B21.T.copy(), atol, rtol)
    if not h.A22.leafnode:
        _recompress(h.A22, h.B21, h.B12.T.copy(), atol, rtol)
    return h


def _recompress(h, Brow, Bcol, atol, rtol):
    """``_recompress!`` (src/compression.jl:205-260)."""
    Brow1 = np.hstack([h.B12, h.R1 @ Brow])
    Bcol2 = np.hstack([h.B12.T, h.W2 @ Bcol])
    P1, S2 = _compress_block(Brow1, atol, rtol)
    Q2, T1 = _compress_block(Bcol2, atol, rtol)
    rm1, rn2 = h.B12.shape
    h.B12 = S2[:, :rn2] @ Q2
    h.R1 = P1.T @ h.R1
    h.W2 = Q2.T @ h.W2
    Brow2 = np.hstack([h.B21, h.R2 @ Brow])
    Bcol1 = np.hstack([h.B21.T, h.W1 @ Bcol])
    P2, S1 = _compress_block(Brow2, atol, rtol)
    Q1, T2 = _compress_block(Bcol1, atol, rtol)
    rm2, rn1 = h.B21.shape
    h.B21 = S1[:, :rn1] @ Q1
    h.R2 = P2.T @ h.R2
    h.W1 = Q1.T @ h.W1
    _push(h.A11, P1, Q1)
    _push(h.A22, P2, Q2)
    if not h.A11.leafnode:
        _recompress(h.A11, np.hstack([h.B12, S2[:, rn2:]]), np.hstack([h.B21.T, T2[:, rm2:]]), atol, rtol)
    if not h.A22.leafnode:
        _recompress(h.A22, np.hstack([h.B21, S1[:, rn1:]]), np.hstack([h.B12.T, T1[:, rm1:]]), atol, rtol)
    return h


def compress(A, rcl: ClusterTree, ccl: ClusterTree, atol=1e-9, rtol=1e-9):
    """``compress(A, rcl, ccl; atol, rtol)`` (src/compression.jl:47-63)."""
    A = np.asarray(A, dtype=float)
    if not compatible(rcl, ccl):
        raise ValueError("row and column clusters are not compatible")
    m, n = len(rcl), len(ccl)
    if A.shape != (m, n):
        raise ValueError("size of row- and column-cluster-trees must match")
    Brow = np.zeros((m, 0))
    Bcol = np.zeros((0, n))
    if rcl.isleaf():
        return HssMatrix.leaf(A[rcl.lo - 1:rcl.hi, ccl.lo - 1:ccl.hi].copy(), rootnode=True)
    h, _, _ = _compress(A, Brow, Bcol, rcl, ccl, atol, rtol, rootnode=True)
    return h


def _compress_leaf(A, Brow, Bcol, rows, cols, atol, rtol):
    """Leaf case of ``_compress!`` (src/compression.jl:66-74)."""
    U, Brow = _compress_block(Brow, atol, rtol)
    V, Bc = _compress_block(Bcol.T.copy(), atol, rtol)
    D = A[rows[0] - 1:rows[1], cols[0] - 1:cols[1]].copy()
    return HssMatrix.leaf(D, U, V), Brow, Bc.T.copy()


def _compress(A, Brow, Bcol, rcl, ccl, atol, rtol, rootnode=False):
    """Branch case of ``_compress!`` (src/compression.jl:77-133)."""
    m1, m2 = len(rcl.left), len(rcl.right)
    n1, n2 = len(ccl.left), len(ccl.right)
    r1 = (rcl.left.lo - 1, rcl.left.hi)
    r2 = (rcl.right.lo - 1, rcl.right.hi)
    c1 = (ccl.left.lo - 1, ccl.left.hi)
    c2 = (ccl.right.lo - 1, ccl.right.hi)
    Brow1 = np.hstack([A[r1[0]:r1[1], c2[0]:c2[1]], Brow[:m1, :]])
    Bcol1 = np.vstack([A[r2[0]:r2[1], c1[0]:c1[1]], Bcol[:, :n1]])
    if rcl.left.isleaf() and ccl.left.isleaf():
        A11, Brow1, Bcol1 = _compress_leaf(A, Brow1, Bcol1, (rcl.left.lo, rcl.left.hi),
                                           (ccl.left.lo, ccl.left.hi), atol, rtol)
    elif not rcl.left.isleaf() and not ccl.left.isleaf():
        A11, Brow1, Bcol1 = _compress(A, Brow1, Bcol1, rcl.left, ccl.left, atol, rtol)
    else:
        raise ValueError("row and column clusters are not compatible")
    Brow2 = np.hstack([Bcol1[:m2, :], Brow[m1:, :]])
    Bcol2 = np.vstack([Brow1[:, :n2], Bcol[:, n1:]])
    if rcl.right.isleaf() and ccl.right.isleaf():
        A22, Brow2, Bcol2 = _compress_leaf(A, Brow2, Bcol2, (rcl.right.lo, rcl.right.hi),
                                           (ccl.right.lo, ccl.right.hi), atol, rtol)
    elif not rcl.right.isleaf() and not ccl.right.isleaf():
        A22, Brow2, Bcol2 = _compress(A, Brow2, Bcol2, rcl.right, ccl.right, atol, rtol)
    else:
        raise ValueError("row and column clusters are not compatible")
    rm1, rn1 = Brow1.shape[0], Bcol1.shape[1]
    B12 = Bcol2[:rm1, :].copy()
    B21 = Brow2[:, :rn1].copy()
    Brow = np.vstack([Brow1[:, n2:], Brow2[:, rn1:]])
    Bcol = np.hstack([Bcol1[m2:, :], Bcol2[rm1:, :]])
    if not rootnode:
        R, Brow = _compress_block(Brow, atol, rtol)
        R1, R2 = R[:rm1, :].copy(), R[rm1:, :].copy()
        W, Bc = _compress_block(Bcol.T.copy(), atol, rtol)
        Bcol = Bc.T.copy()
        W1, W2 = W[:rn1, :].copy(), W[rn1:, :].copy()
        h = HssMatrix.branch(A11, A22, B12, B21, R1, W1, R2, W2, rootnode=False)
    else:
        h = HssMatrix.branch(A11, A22, B12, B21, rootnode=True)
    return h, Brow, Bcol


def hss(A, leafsize=64, atol=1e-9, rtol=1e-9):
    """``hss(A; leafsize, atol, rtol)`` for dense A (src/hssmatrix.jl:71-76)."""
    A = np.asarray(A, dtype=float)
    rcl = bisection_cluster(A.shape[0], leafsize)
    ccl = bisection_cluster(A.shape[1], leafsize)
    return compress(A, rcl, ccl, atol, rtol)


# ---------------------------------------------------------------------------
# randomized compression (src/compression.jl:278-475)
# ---------------------------------------------------------------------------


def _interpolate(A, atol, rtol):
    """``_interpolate`` (src/compression.jl:433-444): ID via ``qr(A, ColumnNorm())``.
    Threshold ``min(atol, rtol*|R11|)`` (:439)."""
    if A.shape[1] == 0:
        return np.zeros((0, 0)), np.zeros(0, dtype=np.int64)
    if A.shape[0] == 0:
        return np.zeros((0, A.shape[1])), np.zeros(0, dtype=np.int64)
    _Q, R, p = sla.qr(A, mode="economic", pivoting=True)
    tol = min(atol, rtol * abs(R[0, 0]))
    rk = int(np.sum(np.abs(np.diag(R)) > tol))
    J = p[:rk].astype(np.int64)
    inv = np.empty_like(p)
    inv[p] = np.arange(len(p))
    X = sla.solve_triangular(R[:rk, :rk], R[:rk, :][:, inv], lower=False) if rk else np.zeros((0, A.shape[1]))
    return X, J


def hss_blkdiag(A, rcl: ClusterTree, ccl: ClusterTree, rootnode=True):
    """``hss_blkdiag`` (src/compression.jl:447-475): rank-0 HSS of the diagonal blocks."""
    if rcl.isleaf():
        D = np.asarray(A[rcl.lo - 1:rcl.hi, ccl.lo - 1:ccl.hi], dtype=float).copy()
        if rootnode:
            return HssMatrix.leaf(D, rootnode=True)
        return HssMatrix.leaf(D, np.zeros((D.shape[0], 0)), np.zeros((D.shape[1], 0)))
    A11 = hss_blkdiag(A, rcl.left, ccl.left, rootnode=False)
    A22 = hss_blkdiag(A, rcl.right, ccl.right, rootnode=False)
    z = np.zeros((0, 0))
    if rootnode:
        return HssMatrix.branch(A11, A22, z, z, rootnode=True)
    return HssMatrix.branch(A11, A22, z, z, z, z, z, z, rootnode=False)


def randcompress(A, rcl, ccl, kest, atol=1e-9, rtol=1e-9, noversampling=10, rng=None):
    """``randcompress(A, rcl, ccl, kest)`` (src/compression.jl:278-294)."""
    rng = np.random.default_rng(0) if rng is None else rng
    A = np.asarray(A, dtype=float)
    m, n = A.shape
    if not compatible(rcl, ccl):
        raise ValueError("row and column clusters are not compatible")
    h = hss_blkdiag(A, rcl, ccl)
    s = kest + noversampling
    Ocol = rng.standard_normal((n, s))
    Orow = rng.standard_normal((m, s))
    Scol = A @ Ocol
    Srow = A.T @ Orow
    h = _randcompress(h, A, Scol, Srow, Ocol, Orow, 0, 0, atol, rtol, rootnode=True)[0]
    return h


def randcompress_adaptive(A, rcl, ccl, kest=10, atol=1e-9, rtol=1e-9, noversampling=10,
                          stepsize=20, rng=None, stats=None):
    """``randcompress_adaptive`` (src/compression.jl:312-355)."""
    rng = np.random.default_rng(0) if rng is None else rng
    A = np.asarray(A, dtype=float)
    m, n = A.shape
    maxrank = n
    if not compatible(rcl, ccl):
        raise ValueError("row and column clusters are not compatible")
    h = hss_blkdiag(A, rcl, ccl)
    k, r, bs = kest, noversampling, stepsize
    Ocol = rng.standard_normal((n, k + r))
    Orow = rng.standard_normal((m, k + r))
    Scol = A @ Ocol
    Srow = A.T @ Orow
    failed = True
    rounds = 0
    while failed and k < maxrank:
        h = _randcompress(h, A, Scol, Srow, Ocol, Orow, 0, 0, atol, rtol, rootnode=True)[0]
        Ocol_t = rng.standard_normal((n, bs))
        Orow_t = rng.standard_normal((m, bs))
        Scol_t = A @ Ocol_t
        Srow_t = A.T @ Orow_t
        nrm = math.sqrt(1.0 / bs) * np.linalg.norm(Scol_t)
        nrm_est = math.sqrt(1.0 / bs) * np.linalg.norm(Scol_t - matmul(h, Ocol_t))
        failed = nrm_est > atol and nrm_est > rtol * nrm
        rounds += 1
        if failed:
            Ocol = np.hstack([Ocol, Ocol_t])
            Orow = np.hstack([Orow, Orow_t])
            Scol = np.hstack([Scol, Scol_t])
            Srow = np.hstack([Srow, Srow_t])
            k += bs
    if stats is not None:
        stats.update(rounds=rounds, k=k, samples=k + r)
    return h


def _randcompress(h, A, Scol, Srow, Ocol, Orow, ro, co, atol, rtol, rootnode=False):
    """``_randcompress!`` (src/compression.jl:358-430).  Slices are copied, as Julia does."""
    if h.leafnode:
        Scol = Scol - h.D @ Ocol                                  # :360
        Srow = Srow - h.D.T @ Orow                                # :361
        Xcol, Jcol = _interpolate(Scol.T, atol, rtol)             # :366
        h.U = Xcol.T.copy()
        Scol = Scol[Jcol, :]
        U = h.U
        Jcol = ro + Jcol
        Xrow, Jrow = _interpolate(Srow.T, atol, rtol)             # :373
        h.V = Xrow.T.copy()
        Srow = Srow[Jrow, :]
        V = h.V
        Jrow = co + Jrow
        h.rootnode = rootnode
        return h, Scol, Srow, Ocol, Orow, Jcol, Jrow, U, V
    m1, n1 = h.sz1
    (h.A11, Scol1, Srow1, Ocol1, Orow1, Jcol1, Jrow1, U1, V1) = _randcompress(
        h.A11, A, Scol[:m1].copy(), Srow[:n1].copy(), Ocol[:n1].copy(), Orow[:m1].copy(), ro, co, atol, rtol)
    (h.A22, Scol2, Srow2, Ocol2, Orow2, Jcol2, Jrow2, U2, V2) = _randcompress(
        h.A22, A, Scol[m1:].copy(), Srow[n1:].copy(), Ocol[n1:].copy(), Orow[m1:].copy(),
        ro + m1, co + n1, atol, rtol)
    Ocol2 = V2.T @ Ocol2                                          # :384-387
    Ocol1 = V1.T @ Ocol1
    Orow2 = U2.T @ Orow2
    Orow1 = U1.T @ Orow1
    Jcol = np.concatenate([Jcol1, Jcol2])
    Jrow = np.concatenate([Jrow1, Jrow2])
    Ocol = np.vstack([Ocol1, Ocol2])
    Orow = np.vstack([Orow1, Orow2])
    h.B12 = A[np.ix_(Jcol1, Jrow2)].copy()                      # :394-395
    h.B21 = A[np.ix_(Jcol2, Jrow1)].copy()
    Scol = np.vstack([Scol1 - h.B12 @ Ocol2, Scol2 - h.B21 @ Ocol1])    # :397
    Srow = np.vstack([Srow1 - h.B21.T @ Orow2, Srow2 - h.B12.T @ Orow1])  # :398
    h.sz1, h.sz2 = h.A11.size(), h.A22.size()
    if rootnode:
        rk1, wk1 = gensize(h.A11)
        rk2, wk2 = gensize(h.A22)
        h.R1, h.R2 = np.zeros((rk1, 0)), np.zeros((rk2, 0))
        h.W1, h.W2 = np.zeros((wk1, 0)), np.zeros((wk2, 0))
        h.rootnode = True
        U = np.zeros((rk1 + rk2, 0))
        V = np.zeros((wk1 + wk2, 0))
    else:
        Xcol, Jcolloc = _interpolate(Scol.T, atol, rtol)          # :413
        h.R1 = Xcol[:, :Scol1.shape[0]].T.copy()
        h.R2 = Xcol[:, Scol1.shape[0]:].T.copy()
        if Xcol.shape[0] == 0:
            h.R1 = np.zeros((Scol1.shape[0], 0))
            h.R2 = np.zeros((Scol2.shape[0], 0))
        Scol = Scol[Jcolloc, :]
        Jcol = Jcol[Jcolloc]
        U = np.vstack([h.R1, h.R2])
        Xrow, Jrowloc = _interpolate(Srow.T, atol, rtol)          # :421
        h.W1 = Xrow[:, :Srow1.shape[0]].T.copy()
        h.W2 = Xrow[:, Srow1.shape[0]:].T.copy()
        if Xrow.shape[0] == 0:
            h.W1 = np.zeros((Srow1.shape[0], 0))
            h.W2 = np.zeros((Srow2.shape[0], 0))
        Srow = Srow[Jrowloc, :]
        Jrow = Jrow[Jrowloc]
        V = np.vstack([h.W1, h.W2])
        h.rootnode = False
    return h, Scol, Srow, Ocol, Orow, Jcol, Jrow, U, V


# ---------------------------------------------------------------------------
# fixtures: kernel matrices and synthetic generator trees
# ---------------------------------------------------------------------------
# HSS-valued division (src/ulvdivide.jl), HSS sums (src/hssmatrix.jl:218-231),
# prune_leaves! and _hssleaf (src/hssmatrix.jl:325-348)
# ---------------------------------------------------------------------------


def _leaf_raw(D, U, V, rootnode):
    """``HssMatrix(D, U, V, rootnode)``: a leaf keeping U and V even at the root."""
    h = HssMatrix()
    h.leafnode, h.rootnode = True, bool(rootnode)
    h.D, h.U, h.V = np.asarray(D, float), np.asarray(U, float), np.asarray(V, float)
    return h


def _branch_raw(A11, A22, B12, B21, R1, W1, R2, W2, rootnode):
    """``HssMatrix(A11, A22, B12, B21, R1, W1, R2, W2, rootnode)``."""
    return HssMatrix.branch(A11, A22, B12, B21, R1, W1, R2, W2, rootnode=bool(rootnode))


def hssleaf(h: HssMatrix):
    """``_hssleaf`` (src/hssmatrix.jl:339-348): D, U, V of the whole subtree."""
    if h.leafnode:
        return h.D, h.U, h.V
    D1, U1, V1 = hssleaf(h.A11)
    D2, U2, V2 = hssleaf(h.A22)
    D = np.block([[D1, U1 @ h.B12 @ V2.T], [U2 @ h.B21 @ V1.T, D2]])
    return D, np.vstack([U1 @ h.R1, U2 @ h.R2]), np.vstack([V1 @ h.W1, V2 @ h.W2])


def prune_leaves(h: HssMatrix):
    """``prune_leaves!`` (src/hssmatrix.jl:325-336): every branch whose children
    are both leaves becomes one leaf."""
    if h.leafnode:
        return h
    if h.A11.leafnode and h.A22.leafnode:
        return _leaf_raw(*hssleaf(h), h.rootnode)
    h.A11 = prune_leaves(h.A11)
    h.A22 = prune_leaves(h.A22)
    h.sz1, h.sz2 = h.A11.size(), h.A22.size()
    return h


def hss_add(A: HssMatrix, B: HssMatrix, sign=1.0):
    """``+`` / ``-`` of two HSS matrices (src/hssmatrix.jl:218-231): leaves add
    (U, V side by side), branches stack the generators block-diagonally."""
    if tuple(A.size()) != tuple(B.size()):
        raise ValueError(f"A has dimensions {A.size()} but B has dimensions {B.size()}")
    root = A.rootnode and B.rootnode
    if A.leafnode and B.leafnode:
        return _leaf_raw(A.D + sign * B.D, np.hstack([A.U, B.U]), np.hstack([A.V, B.V]), root)
    if A.leafnode or B.leafnode:
        raise ValueError("Cannot add leaves and branches.")
    return _branch_raw(hss_add(A.A11, B.A11, sign), hss_add(A.A22, B.A22, sign), _blkdiag(A.B12, sign * B.B12),
                       _blkdiag(A.B21, sign * B.B21), _blkdiag(A.R1, B.R1), _blkdiag(A.W1, B.W1),
                       _blkdiag(A.R2, B.R2), _blkdiag(A.W2, B.W2), root)


class _BN:
    """``BinaryNode`` (src/binarytree.jl) holding per-node data of the division."""
    __slots__ = ("data", "left", "right")

    def __init__(self, data=None, left=None, right=None):
        self.data, self.left, self.right = data, left, right


def _ulvreduce_div(D, U, V):
    """``_ulvreduce!(D, U, V)`` (src/ulvdivide.jl:58-85): the leaf reduction without
    a right-hand side; returns L2 (k x n), tril U, Q V, L1, the QL and LQ
    factorizations, m - k, nk and k.  k > m (more generator columns than rows) is
    outside what the reference handles; it is treated like k = m here."""
    m, n = D.shape
    k = min(U.shape[1], m)
    nk = max(0, min(m - k, n))
    if k >= m:
        return D, U, V, np.zeros((0, 0)), None, None, 0, 0, k
    qlf = QLFact(U)
    Ur = np.tril(qlf.L())
    D = qlf.apply_qt(D)
    lqf = LQFact(D[:m - k, :])
    L1 = lqf.L()[:, :nk]
    L2 = lqf.apply_right_qt(D[m - k:, :])
    V = lqf.apply_left_q(V)
    return L2, Ur, V, L1, qlf, lqf, m - k, nk, k


def _ulvfactor_leaves(h: HssMatrix):
    """``_ulvfactor_leaves!`` (src/ulvdivide.jl:88-112): reduces every leaf; returns
    the reduced matrix and the trees of QL factorizations, L1 blocks, LQ
    factorizations, nk and k."""
    if h.leafnode:
        D, U, V, L1, qlf, lqf, _mk, nk, k = _ulvreduce_div(h.D, h.U, h.V)
        return _leaf_raw(D, U, V, h.rootnode), _BN(qlf), _BN(L1), _BN(lqf), _BN(nk), _BN(k)
    A11, qu1, ql1, qv1, nk1, k1 = _ulvfactor_leaves(h.A11)
    A22, qu2, ql2, qv2, nk2, k2 = _ulvfactor_leaves(h.A22)
    out = _branch_raw(A11, A22, h.B12, h.B21, h.R1, h.W1, h.R2, h.W2, h.rootnode)
    return (out, _BN(None, qu1, qu2), _BN(None, ql1, ql2), _BN(None, qv1, qv2), _BN(None, nk1, nk2),
            _BN(None, k1, k2))


def _map_leaves(h: HssMatrix, t: _BN, f):
    """Applies f(leaf, node of t) at every leaf (the generated branch functions of
    src/ulvdivide.jl:145-158 and :167-179); branches keep their generators."""
    if h.leafnode:
        return f(h, t)
    return _branch_raw(_map_leaves(h.A11, t.left, f), _map_leaves(h.A22, t.right, f), h.B12, h.B21, h.R1, h.W1,
                       h.R2, h.W2, h.rootnode)


def _utransform_leaf(h, t):
    """``_utransforms_kernel!`` (src/ulvdivide.jl:115-121): D, U <- Q^T D, Q^T U."""
    if t.data is None:
        return _leaf_raw(h.D.copy(), h.U.copy(), h.V, h.rootnode)
    return _leaf_raw(t.data.apply_qt(h.D), t.data.apply_qt(h.U), h.V, h.rootnode)


def _ltransform_leaf(h, t):
    """``_ltransforms_kernel!`` (src/ulvdivide.jl:122-129): the first nk rows of D and
    U solved with L1, the other rows zeroed."""
    L1 = t.data
    nk = L1.shape[0]
    D = np.zeros_like(h.D)
    U = np.zeros_like(h.U)
    if nk:
        D[:nk] = sla.solve_triangular(L1, h.D[:nk], lower=True)
        U[:nk] = sla.solve_triangular(L1, h.U[:nk], lower=True)
    return _leaf_raw(D, U, h.V, h.rootnode)


def _vtransform_leaf(h, t):
    """``_vtransforms_kernel!`` (src/ulvdivide.jl:130-136): D, U <- Q^T D, Q^T U with
    the LQ factor's Q."""
    if t.data is None:
        return h
    return _leaf_raw(t.data.apply_left_qt(h.D), t.data.apply_left_qt(h.U), h.V, h.rootnode)


def _unpackadd_rows(A: HssMatrix, B: HssMatrix, kt: _BN):
    """``_unpackadd_rows!`` (src/ulvdivide.jl:182-234): adds the solution B of the
    reduced problem (one level shallower) into the bottom rows of A's leaves."""
    if not A.leafnode:
        if not B.leafnode:
            A11 = _unpackadd_rows(A.A11, B.A11, kt.left)
            A22 = _unpackadd_rows(A.A22, B.A22, kt.right)
            return _branch_raw(A11, A22, _blkdiag(A.B12, B.B12), _blkdiag(A.B21, B.B21), _blkdiag(A.R1, B.R1),
                               _blkdiag(A.W1, B.W1), _blkdiag(A.R2, B.R2), _blkdiag(A.W2, B.W2), A.rootnode)
        k1, k2 = kt.left.data, kt.right.data
        if k1 + k2 != B.D.shape[0]:
            raise ValueError("first dimension of D does not match the expected k1+k2 rows")
        n1 = A.sz1[1]
        r, w = gensize(B)
        eye = lambda q: np.eye(q)
        B12 = _blkdiag(_blkdiag(A.B12, np.zeros((r, w))), eye(k1))
        B21 = _blkdiag(_blkdiag(A.B21, np.zeros((r, w))), eye(k2))
        R1 = np.vstack([_blkdiag(A.R1, eye(r)), np.zeros((k1, A.R1.shape[1] + r))])
        W1 = np.vstack([_blkdiag(A.W1, eye(w)), np.zeros((k2, A.W1.shape[1] + w))])
        R2 = np.vstack([_blkdiag(A.R2, eye(r)), np.zeros((k2, A.R2.shape[1] + r))])
        W2 = np.vstack([_blkdiag(A.W2, eye(w)), np.zeros((k1, A.W2.shape[1] + w))])
        A11 = _unpackadd_leaf(A.A11, B.D[:k1, :n1], B.U[:k1], B.V[:n1], B.D[k1:, :n1])
        A22 = _unpackadd_leaf(A.A22, B.D[k1:, n1:], B.U[k1:], B.V[n1:], B.D[:k1, n1:])
        return _branch_raw(A11, A22, B12, B21, R1, W1, R2, W2, A.rootnode)
    if not B.leafnode:
        raise ValueError("Something went wrong. Expected hssB to also be a leaf node")
    k, rk = B.U.shape
    m = A.D.shape[0]
    if k > m:
        raise ValueError("expected hssB to have less rows than hssA.")
    U = np.hstack([A.U, np.zeros((m, rk))])
    U[m - k:, U.shape[1] - rk:] = B.U
    D = A.D.copy()
    D[m - k:] += B.D
    return _leaf_raw(D, U, np.hstack([A.V, B.V]), A.rootnode)


def _unpackadd_leaf(A: HssMatrix, D, U, V, Brow):
    """``_unpackadd_rows!(hssA, D, U, V, Brow)`` (src/ulvdivide.jl:236-252)."""
    if not A.leafnode:
        raise ValueError("Expected hssA to be a leaf node")
    k = D.shape[0]
    m = A.D.shape[0]
    DA = A.D.copy()
    DA[m - k:] += D
    q = U.shape[1] + k
    UA = np.hstack([A.U, np.zeros((m, q))])
    UA[m - k:, UA.shape[1] - q:] = np.hstack([U, np.eye(k)])
    return _leaf_raw(DA, UA, np.hstack([A.V, V, Brow.T]), A.rootnode)


def ldiv_hss(A: HssMatrix, B: HssMatrix, atol=1e-9, rtol=1e-9):
    """``hssA \\ hssB`` = ``_ldiv!(copy(hssA), copy(hssB))`` (src/hssmatrix.jl:235,
    src/ulvdivide.jl:13, :22-54): the leaves of A reduced (QL of U, LQ of the
    top rows of D), the same transforms applied to B's leaf rows, the reduced
    part solved and the rest (B's remainder minus the coupling, recompressed
    and pruned) solved recursively on the pruned reduced matrix, then unpacked
    back into the leaves and recompressed."""
    if A.leafnode:
        D, U, V = hssleaf(B)
        return _leaf_raw(np.linalg.solve(full(A), D), U, V, B.rootnode)
    L, QU, QL, QV, nkt, kt = _ulvfactor_leaves(A)
    B = _map_leaves(B, QU, _utransform_leaf)
    QB = _map_leaves(B, nkt, lambda h, t: _leaf_raw(h.D[t.data:], h.U[t.data:], h.V, h.rootnode))
    Y0 = _map_leaves(B, QL, _ltransform_leaf)
    if QB.size()[0] == 0:
        return _map_leaves(Y0, QV, _vtransform_leaf)
    QB = hss_add(QB, hssmul(L, Y0), -1.0)
    QB = recompress(QB, atol, rtol)
    QB = prune_leaves(QB)
    L = _map_leaves(L, nkt, lambda h, t: _leaf_raw(h.D[:, t.data:], h.U, h.V[t.data:], h.rootnode))
    L = prune_leaves(L)
    Y1 = ldiv_hss(L, QB, atol, rtol)
    X = _unpackadd_rows(Y0, Y1, kt)
    X = _map_leaves(X, QV, _vtransform_leaf)
    return recompress(X, atol, rtol)


def rdiv_hss(B: HssMatrix, A: HssMatrix, atol=1e-9, rtol=1e-9):
    """``hssB / hssA`` = ``adjoint(_ldiv!(adjoint(hssA), adjoint(hssB)))``
    (src/hssmatrix.jl:237, src/ulvdivide.jl:15-17)."""
    return adjoint(ldiv_hss(adjoint(A), adjoint(B), atol, rtol))


# ---------------------------------------------------------------------------


def cauchy_matrix(n=2001, lo=-1.0, hi=1.0):
    """A_ij = 1/(x_i - y_j), 1 on the diagonal, x = y = n uniform points in [lo, hi]
    (README.md:15-18 kernel; ``-1:0.001:1`` is n=2001)."""
    x = np.linspace(lo, hi, n)
    d = x[:, None] - x[None, :]
    with np.errstate(divide="ignore"):
        A = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 1.0)
    return A


def runtests_matrix(n=2001):
    """The reference suite's fixture K(x,y) = (x-y) > 0 ? 0.001/(x-y) : 2 on -1:0.001:1
    (test/runtests.jl:19-20)."""
    x = np.linspace(-1.0, 1.0, n)
    d = x[:, None] - x[None, :]
    return np.where(d > 0, 0.001 / np.where(d > 0, d, 1.0), 2.0)


def _orth(rng, m, k):
    """Orthonormal m x k (Q of QR of randn)."""
    if k == 0:
        return np.zeros((m, 0))
    Q, _ = np.linalg.qr(rng.standard_normal((m, k)))
    return Q[:, :k]


def synthetic_hss(n, leafsize, k, rng, diag_shift=4.0, bscale=0.5):
    """Synthetic HSS from seeded generators, on ``bisection_cluster(n, leafsize)``:
    leaf D = randn(m,m)/sqrt(m) + shift*I; leaf U, V orthonormal m x min(k, m);
    branch [R1;R2], [W1;W2] orthonormal (k1+k2) x min(k, k1+k2);
    B12, B21 = bscale*randn/sqrt(k)."""
    cl = bisection_cluster(n, leafsize)

    def build(t, root):
        if t.isleaf():
            m = len(t)
            D = rng.standard_normal((m, m)) / math.sqrt(m) + diag_shift * np.eye(m)
            if root:
                return HssMatrix.leaf(D, rootnode=True), 0
            kk = min(k, m)
            return HssMatrix.leaf(D, _orth(rng, m, kk), _orth(rng, m, kk)), kk
        A11, k1 = build(t.left, False)
        A22, k2 = build(t.right, False)
        B12 = bscale * rng.standard_normal((k1, k2)) / math.sqrt(max(k, 1))
        B21 = bscale * rng.standard_normal((k2, k1)) / math.sqrt(max(k, 1))
        if root:
            return HssMatrix.branch(A11, A22, B12, B21, rootnode=True), 0
        kk = min(k, k1 + k2)
        R = _orth(rng, k1 + k2, kk)
        W = _orth(rng, k1 + k2, kk)
        return HssMatrix.branch(A11, A22, B12, B21, R[:k1], W[:k1], R[k1:], W[k1:], rootnode=False), kk

    h, _ = build(cl, True)
    return h


def matvec_bytes(h: HssMatrix, r: int, itemsize=8):
    """Algorithmic bytes of one HSS product with r right-hand sides: every generator
    entry once, plus B read and C written."""
    m, n = h.size()
    return itemsize * (generator_entries(h) + r * (m + n))


def cond_estimate(h: HssMatrix, iters=30, rng=None):
    """2-norm condition estimate from power iteration on A^T A (HSS products) and
    inverse power iteration (two ULV solves per step)."""
    rng = np.random.default_rng(12345) if rng is None else rng
    ht = adjoint(h)
    n = h.size()[1]
    x = rng.standard_normal(n)
    x /= np.linalg.norm(x)
    smax = 0.0
    for _ in range(iters):
        y = matmul(ht, matmul(h, x))
        smax = math.sqrt(np.linalg.norm(y))
        x = y / np.linalg.norm(y)
    x = rng.standard_normal(n)
    x /= np.linalg.norm(x)
    inv = 0.0
    for _ in range(iters):
        y = ulvfactsolve(h, ulvfactsolve(ht, x))
        inv = math.sqrt(np.linalg.norm(y))
        x = y / np.linalg.norm(y)
    return smax * inv
