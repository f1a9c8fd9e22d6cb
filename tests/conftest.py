import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["synthetic_perfect", "synthetic_uneven", "synthetic_earlyexit", "synthetic_unbalanced",
                "single_leaf", "cauchy2001_compress"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def lib(pkg):
    return pkg._lib.load()


@pytest.fixture(scope="session")
def orc():
    from oracle import hss_oracle
    return hss_oracle


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def unpack_tree(table, packed, orc):
    """Rebuild an oracle HssMatrix from the packed layout (inverse of the packer)."""
    def blk(off, r, c):
        if r * c == 0:
            return np.zeros((r, c))
        return packed[off:off + r * c].reshape((r, c), order="F").copy()

    def gens(i):
        if table[i, 0] < 0:
            return table[i, 4], table[i, 5]
        return table[i, 4], table[i, 5]

    def build(i, root):
        t = table[i]
        if t[0] < 0:
            m, n = t[2], t[3]
            D = blk(t[6], m, n)
            if root:
                return orc.HssMatrix.leaf(D, rootnode=True)
            return orc.HssMatrix.leaf(D, blk(t[7], m, t[4]), blk(t[8], n, t[5]))
        l, r = t[0], t[1]
        A11, A22 = build(l, False), build(r, False)
        ku1, kv1 = gens(l)
        ku2, kv2 = gens(r)
        B12, B21 = blk(t[9], ku1, kv2), blk(t[10], ku2, kv1)
        if root:
            return orc.HssMatrix.branch(A11, A22, B12, B21, rootnode=True)
        ku, kv = t[4], t[5]
        return orc.HssMatrix.branch(A11, A22, B12, B21, blk(t[11], ku1, ku), blk(t[13], kv1, kv),
                                    blk(t[12], ku2, ku), blk(t[14], kv2, kv), rootnode=False)

    return build(0, True)
