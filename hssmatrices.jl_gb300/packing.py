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


def unpack(table, packed):
    """Inverse of ``pack``: the ``HssMatrix`` of a node table + packed buffer
    (e.g. exported from the device after randomized compression)."""
    from .hssmatrix import HssMatrix
    table = np.asarray(table, dtype=np.int64)
    packed = np.asarray(packed, dtype=np.float64)

    def blk(off, r, c):
        if r * c == 0:
            return np.zeros((r, c))
        return packed[off:off + r * c].reshape((r, c), order="F").copy()

    def build(i, root):
        t = table[i]
        if t[0] < 0:
            D = blk(t[6], t[2], t[3])
            if root:
                return HssMatrix.leaf(D, rootnode=True)
            return HssMatrix.leaf(D, blk(t[7], t[2], t[4]), blk(t[8], t[3], t[5]))
        l, r = int(t[0]), int(t[1])
        A11, A22 = build(l, False), build(r, False)
        ku1, kv1 = table[l, 4], table[l, 5]
        ku2, kv2 = table[r, 4], table[r, 5]
        B12, B21 = blk(t[9], ku1, kv2), blk(t[10], ku2, kv1)
        if root:
            return HssMatrix.branch(A11, A22, B12, B21, rootnode=True)
        ku, kv = t[4], t[5]
        return HssMatrix.branch(A11, A22, B12, B21, blk(t[11], ku1, ku), blk(t[13], kv1, kv),
                                blk(t[12], ku2, ku), blk(t[14], kv2, kv), rootnode=False)

    return build(0, True)
