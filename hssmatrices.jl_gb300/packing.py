"""Packs a generator tree into the node table + FP64 buffer of ``hss_create``.

This is the one walk over the host tree that the Julia shim would do before
``ccall``: nodes are numbered in pre-order (root 0, left subtree first), and
the generator blocks are written column-major into one buffer in level order
-- all leaf ``D`` blocks (the bulk of the bytes) in leaf order, then the leaf
``U`` and ``V`` blocks, then the branch translators ``B12, B21, R1, R2, W1,
W2`` depth by depth -- so that each tree level is one contiguous range.

Works on any object with the reference's field names (``leafnode``, ``D``,
``U``, ``V``, ``A11``, ``A22``, ``B12``, ``B21``, ``R1``, ``W1``, ``R2``,
``W2``), e.g. ``HssMatrix`` here.
"""
from __future__ import annotations

import numpy as np

from ._lib import NODE_FIELDS


def _preorder(h):
    out = []      # (node, depth, parent_index)
    kids = {}
    stack = [(h, 0, -1, None)]
    while stack:
        x, d, par, side = stack.pop()
        idx = len(out)
        out.append((x, d))
        if par >= 0:
            kids.setdefault(par, [None, None])[side] = idx
        if not x.leafnode:
            stack.append((x.A22, d + 1, idx, 1))
            stack.append((x.A11, d + 1, idx, 0))
    return out, kids


def pack(h):
    """Returns (table int64[nnodes, 16], packed float64[total])."""
    nodes, kids = _preorder(h)
    nn = len(nodes)
    table = np.full((nn, NODE_FIELDS), -1, dtype=np.int64)
    table[:, 2:6] = 0
    table[:, 15] = 0
    chunks = []
    off = 0

    def put(a):
        nonlocal off
        a = np.asarray(a, dtype=np.float64)
        if a.size == 0:
            return -1
        o = off
        chunks.append(np.ravel(a, order="F"))
        off += a.size
        return o

    for i, (x, _d) in enumerate(nodes):
        root = i == 0
        if x.leafnode:
            m, n = x.D.shape
            table[i, 2], table[i, 3] = m, n
            if not root:
                table[i, 4], table[i, 5] = x.U.shape[1], x.V.shape[1]
        else:
            table[i, 0], table[i, 1] = kids[i]
            if not root:
                table[i, 4], table[i, 5] = x.R1.shape[1], x.W1.shape[1]
    leaves = [i for i, (x, _d) in enumerate(nodes) if x.leafnode]
    for i in leaves:
        table[i, 6] = put(nodes[i][0].D)
    for i in leaves:
        if i != 0:
            table[i, 7] = put(nodes[i][0].U)
    for i in leaves:
        if i != 0:
            table[i, 8] = put(nodes[i][0].V)
    maxd = max(d for _x, d in nodes)
    for depth in range(maxd + 1):
        for i, (x, d) in enumerate(nodes):
            if d != depth or x.leafnode:
                continue
            table[i, 9] = put(x.B12)
            table[i, 10] = put(x.B21)
            if i != 0:
                table[i, 11] = put(x.R1)
                table[i, 12] = put(x.R2)
                table[i, 13] = put(x.W1)
                table[i, 14] = put(x.W2)
    packed = np.concatenate(chunks) if chunks else np.zeros(0)
    return np.ascontiguousarray(table), np.ascontiguousarray(packed)


def pack_cached(h):
    """``pack`` once per tree object (the serving loop uploads the same matrices again)."""
    cached = getattr(h, "_packed", None)
    if cached is None:
        cached = pack(h)
        try:
            h._packed = cached
        except AttributeError:
            pass
    return cached
