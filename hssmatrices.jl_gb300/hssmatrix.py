"""Host-side mirror of the reference's data structures and options.

* ``HssOptions`` / ``setopts``      -- src/HssMatrices.jl:52-108
* ``ClusterTree`` / ``bisection_cluster`` -- src/clustertree.jl:14-35
* ``HssMatrix`` (leaf D, U, V; branch A11, A22, B12, B21, R1, W1, R2, W2)
                                      -- src/hssmatrix.jl:11-67, with ``size``
  (:94), ``gensize`` (:254-262), ``hssrank`` (:251), ``isleaf``/``isbranch``
  (:88-89)

The generator tree stays a host object; the first GPU operation packs it
(``packing.pack``) and uploads it once.  Arithmetic (``*``, ``mul``, ``ldiv``,
``ulvfactor``) lives in ``linalg.py`` and always runs on the GPU.
"""
from __future__ import annotations

import copy as _copy
from dataclasses import dataclass
from typing import Optional

import numpy as np

# ---------------------------------------------------------------------------
# options (src/HssMatrices.jl:52-108)
# ---------------------------------------------------------------------------

_defaults = dict(atol=1e-9, rtol=1e-9, leafsize=64, noversampling=10, stepsize=20, verbose=False)


@dataclass
class HssOptions:
    atol: float = _defaults["atol"]
    rtol: float = _defaults["rtol"]
    leafsize: int = _defaults["leafsize"]
    noversampling: int = _defaults["noversampling"]
    stepsize: int = _defaults["stepsize"]
    verbose: bool = _defaults["verbose"]

    @classmethod
    def current(cls, **kw):
        """``HssOptions(; args...)``: module defaults overridden by keywords (:70-77)."""
        o = cls(**_defaults)
        for k, v in kw.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown option {k}")
            setattr(o, k, v)
        return o

    def copy(self, **kw):
        o = _copy.copy(self)
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def check(self):
        """``chkopts!`` (src/HssMatrices.jl:90-96)."""
        if not self.atol >= 0:
            raise ValueError("atol")
        if not self.rtol >= 0:
            raise ValueError("rtol")
        if not self.leafsize >= 1:
            raise ValueError("leafsize")
        if not self.stepsize >= 1:
            raise ValueError("stepsize")
        if not self.noversampling >= 1:
            raise ValueError("noversampling")
        return self


def setopts(**kw):
    """``setopts`` (src/HssMatrices.jl:98-108): change the module defaults."""
    o = HssOptions.current(**kw).check()
    for k in _defaults:
        _defaults[k] = getattr(o, k)
    return o


# ---------------------------------------------------------------------------
# cluster trees (src/clustertree.jl:14-35)
# ---------------------------------------------------------------------------


@dataclass
class ClusterTree:
    """``BinaryNode{UnitRange{Int}}``; ``lo``/``hi`` 1-based inclusive like the Julia range."""

    lo: int
    hi: int
    left: Optional["ClusterTree"] = None
    right: Optional["ClusterTree"] = None

    def __len__(self):
        return self.hi - self.lo + 1

    def isleaf(self):
        return self.left is None and self.right is None

    def isbranch(self):
        return self.left is not None and self.right is not None


def bisection_cluster(n, leafsize: Optional[int] = None) -> ClusterTree:
    """``bisection_cluster(1:n; leafsize)``: split at ``ceil(len/2)`` while ``len > leafsize``."""
    leafsize = HssOptions.current().leafsize if leafsize is None else leafsize
    if leafsize < 1:
        raise ValueError("leafsize")
    lo, hi = (1, int(n)) if np.isscalar(n) else (int(n[0]), int(n[1]))
    if hi - lo + 1 <= 0:
        raise ValueError("Index range must be larger or equal to 0")
    return _bisect(lo, hi, leafsize)


def _bisect(lo, hi, leafsize):
    node = ClusterTree(lo, hi)
    length = hi - lo + 1
    if length > leafsize:
        h = (length + 1) // 2
        node.left = _bisect(lo, lo + h - 1, leafsize)
        node.right = _bisect(lo + h, hi, leafsize)
    return node


# ---------------------------------------------------------------------------
# HssMatrix (src/hssmatrix.jl:11-67)
# ---------------------------------------------------------------------------


class HssMatrix:
    """Hierarchically semiseparable matrix: a binary tree of generators.

    Leaf fields ``D`` (m x n), ``U`` (m x ku), ``V`` (n x kv); branch fields
    ``A11``, ``A22``, ``B12``, ``B21``, ``R1``, ``W1``, ``R2``, ``W2``, ``sz1``,
    ``sz2``; ``leafnode``/``rootnode`` flags, exactly as the Julia struct.
    """

    def __init__(self):
        self.leafnode = True
        self.rootnode = True
        self.D = self.U = self.V = None
        self.A11 = self.A22 = None
        self.B12 = self.B21 = None
        self.R1 = self.W1 = self.R2 = self.W2 = None
        self.sz1 = self.sz2 = None
        self._device = None

    # -- constructors (src/hssmatrix.jl:36-67) ------------------------------
    @classmethod
    def leaf(cls, D, U=None, V=None, rootnode=None):
        h = cls()
        D = np.asarray(D, dtype=np.float64)
        m, n = D.shape
        if U is None:
            U, V = np.zeros((m, 0)), np.zeros((n, 0))
            h.rootnode = True if rootnode is None else rootnode
        else:
            U, V = np.asarray(U, np.float64), np.asarray(V, np.float64)
            if U.shape[0] != m:
                raise ValueError("D and U must have same number of rows")
            if V.shape[0] != n:
                raise ValueError("D and V must have same number of columns")
            h.rootnode = False if rootnode is None else rootnode
        h.leafnode = True
        h.D, h.U, h.V = D, U, V
        return h

    @classmethod
    def branch(cls, A11, A22, B12, B21, R1=None, W1=None, R2=None, W2=None, rootnode=None):
        h = cls()
        h.leafnode = False
        h.A11, h.A22 = A11, A22
        h.B12, h.B21 = np.asarray(B12, np.float64), np.asarray(B21, np.float64)
        h.sz1, h.sz2 = A11.size(), A22.size()
        if R1 is None:
            kr1, kw1 = gensize(A11)
            kr2, kw2 = gensize(A22)
            h.R1, h.W1 = np.zeros((kr1, 0)), np.zeros((kw1, 0))
            h.R2, h.W2 = np.zeros((kr2, 0)), np.zeros((kw2, 0))
            h.rootnode = True if rootnode is None else rootnode
        else:
            R1, W1, R2, W2 = (np.asarray(x, np.float64) for x in (R1, W1, R2, W2))
            if R1.shape[1] != R2.shape[1]:
                raise ValueError("R1 and R2 must have same number of columns")
            if W1.shape[1] != W2.shape[1]:
                raise ValueError("W1 and W2 must have same number of rows")
            h.R1, h.W1, h.R2, h.W2 = R1, W1, R2, W2
            h.rootnode = False if rootnode is None else rootnode
        return h

    @classmethod
    def from_tree(cls, other):
        """Copy a generator tree from any object with the same field names."""
        if other.leafnode:
            if other.rootnode and (other.U is None or other.U.shape[1] == 0):
                return cls.leaf(np.array(other.D, dtype=np.float64), rootnode=True)
            return cls.leaf(np.array(other.D, np.float64), np.array(other.U, np.float64),
                            np.array(other.V, np.float64), rootnode=bool(other.rootnode))
        A11 = cls.from_tree(other.A11)
        A22 = cls.from_tree(other.A22)
        return cls.branch(A11, A22, other.B12, other.B21, other.R1, other.W1, other.R2, other.W2,
                          rootnode=bool(other.rootnode))

    # -- basic queries --------------------------------------------------------
    def isleaf(self):
        return self.leafnode

    def isbranch(self):
        return not self.leafnode

    def size(self, dim=None):
        """``size`` (src/hssmatrix.jl:94-95)."""
        s = self.D.shape if self.leafnode else (self.sz1[0] + self.sz2[0], self.sz1[1] + self.sz2[1])
        return s if dim is None else s[dim - 1]

    @property
    def shape(self):
        return self.size()

    def __repr__(self):
        m, n = self.size()
        return f"{m}x{n} HssMatrix{{Float64}}"

    # -- GPU residency --------------------------------------------------------
    def device(self):
        """The uploaded generator tree (``linalg.DeviceHss``), created on first use."""
        if self._device is None:
            from .linalg import DeviceHss
            self._device = DeviceHss(self)
        return self._device

    def invalidate(self):
        """Drop the uploaded copy after the host generators were modified."""
        self._device = None

    # -- operators mirroring src/matmul.jl:13-15, src/hssmatrix.jl:234 ------
    def __mul__(self, B):
        """``hssA * B``: dense B (src/matmul.jl:13) or an HssMatrix (:65)."""
        from .linalg import hssmul, matmul
        if isinstance(B, HssMatrix):
            return hssmul(self, B)
        return matmul(self, B)

    __matmul__ = __mul__

    # numpy defers A @ hssB and A / hssB to the methods below
    __array_ufunc__ = None

    def __rmul__(self, A):
        """``A * hssB`` for a dense A (src/matmul.jl:14): (hssB' * A')' on the device."""
        from .linalg import rmatmul
        return rmatmul(A, self)

    __rmatmul__ = __rmul__

    def __rtruediv__(self, B):
        """``B / hssA`` for a dense B (src/hssmatrix.jl:236): (hssA' \\ B')'."""
        from .linalg import rdiv
        return rdiv(B, self)

    def __getitem__(self, key):
        """``hssA[i, j]`` (src/hssmatrix.jl:102-114), 0-based, on the device."""
        from .linalg import getindex
        if not isinstance(key, tuple) or len(key) != 2:
            raise IndexError("HssMatrix takes two indices")
        return getindex(self, key[0], key[1])

    def solve(self, b, **kw):
        """``hssA \\ b`` (src/hssmatrix.jl:234; an HssMatrix b: :235)."""
        from .linalg import ldiv
        return ldiv(self, b, **kw)

    def __truediv__(self, other):
        """``hssB / hssA`` for an HssMatrix hssA (src/hssmatrix.jl:237)."""
        from .linalg import rdiv
        if not isinstance(other, HssMatrix):
            return NotImplemented
        return rdiv(self, other)


def gensize(h):
    """``gensize`` (src/hssmatrix.jl:254-262)."""
    if h.leafnode:
        return h.U.shape[1], h.V.shape[1]
    kr, kw = h.R1.shape[1], h.W1.shape[1]
    if kr != h.R2.shape[1]:
        raise ValueError("dimensions of column-translators do not match")
    if kw != h.W2.shape[1]:
        raise ValueError("dimensions of row-translators do not match")
    return kr, kw


def hssrank(h):
    """``hssrank`` (src/hssmatrix.jl:251)."""
    if h.leafnode:
        return 0
    return max(hssrank(h.A11), hssrank(h.A22), *h.B12.shape, *h.B21.shape)


def isleaf(h):
    return h.leafnode


def isbranch(h):
    return not h.leafnode
