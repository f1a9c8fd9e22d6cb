"""Generates the golden fixtures in this directory from the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py

Each ``.npz`` holds a packed generator tree (node table + FP64 buffer, the
``hss_create`` layout), seeded inputs, and the oracle's outputs for the HSS
product (src/matmul.jl:18-62), the ULV solve (src/ulvfactor.jl:10-107) and the
per-node ``cols`` bookkeeping (src/ulvfactor.jl:62,76).  ``clusters.npz``
holds ``bisection_cluster`` leaf ranges (src/clustertree.jl:27-35).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import hss_oracle as orc  # noqa: E402


def pack_tree(h):
    """Pre-order node table + column-major packed buffer (same layout as the package's packer)."""
    nodes = []

    def visit(x, d):
        idx = len(nodes)
        nodes.append([x, d, -1, -1])
        if not x.leafnode:
            nodes[idx][2] = visit(x.A11, d + 1)
            nodes[idx][3] = visit(x.A22, d + 1)
        return idx

    visit(h, 0)
    table = np.full((len(nodes), 16), -1, dtype=np.int64)
    table[:, 2:6] = 0
    table[:, 15] = 0
    chunks, off = [], 0

    def put(a):
        nonlocal off
        if a.size == 0:
            return -1
        o = off
        chunks.append(np.ravel(a, order="F"))
        off += a.size
        return o

    for i, (x, _d, l, r) in enumerate(nodes):
        table[i, 0], table[i, 1] = l, r
        if x.leafnode:
            table[i, 2:4] = x.D.shape
            if i:
                table[i, 4], table[i, 5] = x.U.shape[1], x.V.shape[1]
        elif i:
            table[i, 4], table[i, 5] = x.R1.shape[1], x.W1.shape[1]
    leaves = [i for i, n in enumerate(nodes) if n[0].leafnode]
    for i in leaves:
        table[i, 6] = put(nodes[i][0].D)
    for i in leaves:
        if i:
            table[i, 7] = put(nodes[i][0].U)
    for i in leaves:
        if i:
            table[i, 8] = put(nodes[i][0].V)
    for depth in range(max(n[1] for n in nodes) + 1):
        for i, (x, d, _l, _r) in enumerate(nodes):
            if d == depth and not x.leafnode:
                table[i, 9] = put(x.B12)
                table[i, 10] = put(x.B21)
                if i:
                    for f, a in zip(range(11, 15), (x.R1, x.R2, x.W1, x.W2)):
                        table[i, f] = put(a)
    return table, np.concatenate(chunks)


def case(name, h, rng, r):
    m, n = h.size()
    table, packed = pack_tree(h)
    x = rng.standard_normal((n, r))
    b = rng.standard_normal((m, r))
    y = orc.matmul(h, x)
    z = orc.ulvfactsolve(h, b)
    cols = orc.ulv_cols(h)
    flat = np.concatenate([c for c, _mk, _nk in cols])
    lens = np.array([len(c) for c, _mk, _nk in cols], dtype=np.int64)
    mks = np.array([mk for _c, mk, _nk in cols], dtype=np.int64)
    A = orc.full(h)
    z_dense = np.linalg.solve(A, b)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), table=table, packed=packed, x=x, b=b, y=y,
                        z=z, cols=flat, cols_len=lens, cols_mk=mks,
                        size=np.array([m, n], dtype=np.int64))
    print(name, m, n, "nodes", table.shape[0], "packed", packed.size,
          "err vs dense", np.linalg.norm(z - z_dense) / np.linalg.norm(z_dense))


def main():
    rng = np.random.default_rng(20240101)
    # perfect tree, equal ranks
    case("synthetic_perfect", orc.synthetic_hss(512, 64, 12, rng), rng, 3)
    # uneven leaves (2001 / 64 -> leaves of 62 and 63), ranks 20
    case("synthetic_uneven", orc.synthetic_hss(1001, 64, 16, rng), rng, 2)
    # rank >= leaf size at some leaves: the k >= m early exit (src/ulvfactor.jl:32-36)
    case("synthetic_earlyexit", orc.synthetic_hss(320, 40, 48, rng), rng, 2)
    # unbalanced tree (129 -> 65 + 64 with leafsize 64)
    case("synthetic_unbalanced", orc.synthetic_hss(129, 64, 8, rng), rng, 1)
    # single leaf (the whole matrix is dense)
    case("single_leaf", orc.synthetic_hss(40, 64, 8, rng), rng, 2)
    # config 1: Cauchy-type kernel on -1:0.001:1, leafsize 64, compress atol=rtol=1e-6
    A = orc.cauchy_matrix(2001)
    cl = orc.bisection_cluster(2001, 64)
    case("cauchy2001_compress", orc.compress(A, cl, cl, 1e-6, 1e-6), np.random.default_rng(0), 1)
    # cluster trees
    out = {}
    for n, ls in [(10, 3), (2001, 64), (2001, 50), (16384, 128), (65536, 128), (1152, 64), (129, 64),
                  (1, 64), (64, 64), (65, 64)]:
        leaves = orc.cluster_leaves(orc.bisection_cluster(n, ls))
        out[f"n{n}_ls{ls}"] = np.array(leaves, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "clusters.npz"), **out)


if __name__ == "__main__":
    main()
