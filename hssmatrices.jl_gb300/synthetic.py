"""Seeded synthetic HSS generator trees for benchmarks and the request stream.

On ``bisection_cluster(n, leafsize)`` (src/clustertree.jl:27-35):
leaf ``D = randn(m,m)/sqrt(m) + shift*I``, leaf ``U``, ``V`` orthonormal
``m x min(k, m)`` (Q of a QR of randn); branch ``[R1; R2]`` and ``[W1; W2]``
orthonormal ``(k1+k2) x min(k, k1+k2)``; ``B12``, ``B21 = bscale*randn/sqrt(k)``.
Draws happen in post-order (left subtree, right subtree, then the node).
"""
from __future__ import annotations

import math

import numpy as np

from .hssmatrix import HssMatrix, bisection_cluster


def _orth(rng, m, k):
    if k == 0:
        return np.zeros((m, 0))
    q, _ = np.linalg.qr(rng.standard_normal((m, k)))
    return q[:, :k]


def synthetic_hss(n, leafsize, k, rng, diag_shift=4.0, bscale=0.5):
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


def generator_entries(h):
    """Stored generator entries (D, U, V, R, W, B) of a tree."""
    if h.leafnode:
        return h.D.size + h.U.size + h.V.size
    return (generator_entries(h.A11) + generator_entries(h.A22) + h.B12.size + h.B21.size
            + h.R1.size + h.R2.size + h.W1.size + h.W2.size)
