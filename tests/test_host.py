"""Host-side logic without a GPU: ABI exports, packing, validation, bookkeeping."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden, unpack_tree


def header_symbols():
    src = open(os.path.join(ROOT, "include", "hssgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hss_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib, pkg):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(pkg._lib.EXPORTS) == syms
    assert lib.hss_version() >= 1


def _inspect(lib, table, npacked):
    info = np.zeros((table.shape[0], 13), dtype=np.int64)
    rc = lib.hss_inspect(table.shape[0], table.ctypes.data_as(C.POINTER(C.c_int64)), npacked,
                         info.ctypes.data_as(C.POINTER(C.c_int64)))
    return rc, info


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_packer_matches_golden_layout(pkg, orc, name):
    """The package's packer produces the same table and buffer as the fixture script."""
    g = load_golden(name)
    h = unpack_tree(g["table"], g["packed"], orc)
    table, packed = pkg.pack(pkg.HssMatrix.from_tree(h))
    assert np.array_equal(table, g["table"])
    assert np.array_equal(packed, g["packed"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_inspect_bookkeeping_bit_exact(lib, orc, name):
    """Depth/height/offsets and ULV sizes from the C library equal the oracle's bookkeeping
    (src/ulvfactor.jl:27-28,62,76; src/clustertree.jl:27-35)."""
    g = load_golden(name)
    rc, info = _inspect(lib, g["table"], g["packed"].size)
    assert rc == 0, lib.hss_last_error()
    h = unpack_tree(g["table"], g["packed"], orc)
    cols = orc.ulv_cols(h)   # pre-order, same numbering as the table
    assert len(cols) == info.shape[0]
    for i, (c, mk, nk) in enumerate(cols):
        assert info[i, 5] == len(c), i          # n of the reduce problem = len(cols)
        if i:
            assert info[i, 9] == mk and info[i, 10] == nk, i
    # cols rebuilt from the library's sizes equal the oracle's, element by element
    def rebuild(i):
        t = g["table"][i]
        if t[0] < 0:
            return list(range(info[i, 3], info[i, 3] + info[i, 5]))
        a, b = rebuild(t[0]), rebuild(t[1])
        return a[info[t[0], 10]:] + b[info[t[1], 10]:]
    flat = np.concatenate([np.array(rebuild(i), dtype=np.int64) for i in range(info.shape[0])])
    assert np.array_equal(flat, g["cols"])
    # leaf offsets follow bisection order
    m, _n = g["size"]
    leaves = [i for i in range(info.shape[0]) if info[i, 11]]
    assert sum(g["table"][i, 2] for i in leaves) == m


def test_inspect_rejects_bad_trees(lib, pkg, orc):
    g = load_golden("synthetic_perfect")
    t = g["table"].copy()
    t[1, 4] += 1          # left child's U rank no longer matches its parent's B12/R1
    rc, _ = _inspect(lib, t, g["packed"].size)
    assert rc == pkg._lib.HSS_ERR_BAD_DIMS
    t = g["table"].copy()
    t[1, 1] = -1          # a node with one child
    rc, _ = _inspect(lib, t, g["packed"].size)
    assert rc == pkg._lib.HSS_ERR_BAD_DIMS
    t = g["table"].copy()
    rc, _ = _inspect(lib, t, g["packed"].size - 1)   # last block out of range
    assert rc == pkg._lib.HSS_ERR_BAD_DIMS
    t = g["table"].copy()
    t[2, 0] = 1           # cycle back to an ancestor
    t[2, 1] = 2
    rc, _ = _inspect(lib, t, g["packed"].size)
    assert rc == pkg._lib.HSS_ERR_BAD_DIMS
    # a rectangular (3 x 4) leaf root is a valid operand of the products
    # (src/matmul.jl); only its ULV factorization is refused
    one = np.full((1, 16), -1, dtype=np.int64)
    one[0, 2:6] = [3, 4, 0, 0]
    one[0, 6] = 0
    one[0, 15] = 0
    rc, _ = _inspect(lib, one, 12)
    assert rc == pkg._lib.HSS_OK


def test_host_mirror_api(pkg, orc):
    rng = np.random.default_rng(0)
    h = pkg.HssMatrix.from_tree(orc.synthetic_hss(300, 64, 8, rng))
    assert h.size() == (300, 300) and h.size(1) == 300
    assert pkg.hssrank(h) == 8
    assert pkg.gensize(h.A11) == (8, 8)
    assert repr(h) == "300x300 HssMatrix{Float64}"
    with pytest.raises(ValueError):
        pkg.HssMatrix.leaf(np.zeros((3, 3)), np.zeros((2, 1)), np.zeros((3, 1)))
    o = pkg.HssOptions.current(leafsize=32)
    assert o.leafsize == 32 and pkg.HssOptions.current().leafsize == 64
    with pytest.raises(ValueError):
        pkg.HssOptions.current(atol=-1.0).check()


def test_synthetic_generator_matches_oracle(pkg, orc):
    """The package's benchmark inputs are the same trees the oracle builds from the same seed."""
    a = pkg.synthetic_hss(1152, 64, 48, np.random.default_rng(5))
    b = orc.synthetic_hss(1152, 64, 48, np.random.default_rng(5))
    ta, pa = pkg.pack(a)
    tb, pb = pkg.pack(pkg.HssMatrix.from_tree(b))
    assert np.array_equal(ta, tb) and np.array_equal(pa, pb)
    assert pkg.generator_entries(a) == orc.generator_entries(b) == pa.size


def test_cluster_table_and_validation(pkg, lib):
    """Cluster table of two compatible trees (pre-order, 0-based half-open), and
    hss_rc_create's host-side checks (no GPU needed: they run before any CUDA call)."""
    import ctypes as C
    rcl = pkg.bisection_cluster(10, 3)
    t = pkg.cluster_table(rcl, rcl)
    expect = [[1, 4, 0, 10, 0, 10], [2, 3, 0, 5, 0, 5], [-1, -1, 0, 3, 0, 3], [-1, -1, 3, 5, 3, 5],
              [5, 6, 5, 10, 5, 10], [-1, -1, 5, 8, 5, 8], [-1, -1, 8, 10, 8, 10]]
    assert t.tolist() == expect
    # rectangular: rows and columns from different trees of the same shape
    t2 = pkg.cluster_table(pkg.bisection_cluster(10, 3), pkg.bisection_cluster(12, 3))
    assert t2[0].tolist() == [1, 4, 0, 10, 0, 12]
    with pytest.raises(ValueError):
        pkg.cluster_table(pkg.bisection_cluster(10, 3), pkg.bisection_cluster(10, 5))

    def create(tab):
        tab = np.ascontiguousarray(np.asarray(tab, dtype=np.int64))
        h = C.c_void_p()
        return lib.hss_rc_create(tab.shape[0], tab.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(h))

    bad = [r[:] for r in expect]
    bad[1][3] = 4                      # left child does not end where the right one starts
    assert create(bad) == pkg._lib.HSS_ERR_BAD_DIMS
    bad = [r[:] for r in expect]
    bad[0][1] = -1                     # one child only
    assert create(bad) == pkg._lib.HSS_ERR_BAD_DIMS
    bad = [r[:] for r in expect]
    bad[4][0] = 2                      # node 2 with two parents
    assert create(bad) == pkg._lib.HSS_ERR_BAD_DIMS
    bad = [r[:] for r in expect]
    bad[2][3] = 0                      # empty leaf
    assert create(bad) == pkg._lib.HSS_ERR_BAD_DIMS


def test_sample_argument_checks(pkg, lib):
    import ctypes as C
    # leading dimensions below the sizes are rejected before any device access
    assert lib.hss_sample(None, 5, 10, 4, 0, None, 4, 2, None, 10, 1.0, 0.0, None) == pkg._lib.HSS_ERR_BAD_DIMS
    assert lib.hss_sample(None, 10, 10, 4, 1, None, 4, 2, None, 4, 1.0, 0.0, None) == pkg._lib.HSS_ERR_BAD_DIMS
    assert lib.hss_sample(None, 10, 10, 4, 2, None, 4, 2, None, 10, 1.0, 0.0, None) == pkg._lib.HSS_ERR_BAD_DIMS
    out = C.c_double()
    assert lib.hss_sumsq(None, 3, 5, 1, C.byref(out), None) == pkg._lib.HSS_ERR_BAD_DIMS


def test_unpack_inverts_pack(pkg, orc):
    rng = np.random.default_rng(12)
    h = pkg.HssMatrix.from_tree(orc.synthetic_hss(777, 64, 9, rng))
    table, packed = pkg.pack(h)
    h2 = pkg.unpack(table, packed)
    t2, p2 = pkg.pack(h2)
    assert np.array_equal(table, t2) and np.array_equal(packed, p2)


def test_getindex_index_forms(pkg):
    """hssA[i, j] index normalisation (src/hssmatrix.jl:102-107): ints (also
    negative), ranges, colons and sequences, 0-based; out of range raises."""
    from hssmatrices_gb300.linalg import _index_list
    a, scalar = _index_list(3, 10)
    assert scalar and a.tolist() == [3]
    a, scalar = _index_list(-1, 10)
    assert scalar and a.tolist() == [9]
    a, scalar = _index_list(slice(2, 8, 3), 10)
    assert not scalar and a.tolist() == [2, 5]
    a, _ = _index_list(slice(None), 4)
    assert a.tolist() == [0, 1, 2, 3]
    a, _ = _index_list([7, 1, 7], 10)
    assert a.tolist() == [7, 1, 7]
    for bad in (10, -11, [0, 10], [-1]):
        with pytest.raises(IndexError):
            _index_list(bad, 10)


def test_sample_precision_switch(pkg, lib):
    """The mixed-precision sampling switch: double-float only for matrices
    within float's exponent range, the option reset after the compression."""
    torch = pytest.importorskip("torch")
    comp = pkg.compression
    A = comp.DenseDevice(np.ones((5, 4)), device="cpu")
    with comp._SamplePrecision(A, "df") as sp:
        assert sp.df
    assert not comp._SamplePrecision(A, "fp64").df
    assert not comp._SamplePrecision(comp.DenseDevice(np.full((3, 3), 1e35), device="cpu"), "df").df
    assert not comp._SamplePrecision(comp.DenseDevice(np.zeros((3, 3)), device="cpu"), "df").df
    with pytest.raises(ValueError):
        comp._SamplePrecision(A, "fp32")
    assert lib.hss_set_option(5, 0) == 0


def test_process_options_known(lib):
    """Every process-wide switch of hssgpu.h is accepted (and left at its
    default); an unknown one is rejected."""
    defaults = {1: 0, 2: 0, 3: 0, 4: 0, 5: 0, 6: 1}
    for opt, val in defaults.items():
        assert lib.hss_set_option(opt, val) == 0
    assert lib.hss_set_option(99, 1) != 0


def test_transpose_and_cluster_trees(pkg, orc):
    """transpose (the adjoint of real generators) and the cluster trees read
    back from a generator tree: host only."""
    rng = np.random.default_rng(11)
    for n, ls, k in [(700, 64, 8), (50, 64, 8), (129, 64, 4)]:
        h = orc.synthetic_hss(n, ls, k, rng)
        A = pkg.HssMatrix.from_tree(h)
        At = pkg.transpose(A)
        assert np.abs(orc.full(At) - orc.full(h).T).max() <= 1e-13
        rc, cc = pkg.cluster_trees(A)
        ref = pkg.bisection_cluster(n, ls)

        def same(a, b):
            return (a.lo, a.hi) == (b.lo, b.hi) and a.isleaf() == b.isleaf() and (
                a.isleaf() or (same(a.left, b.left) and same(a.right, b.right)))

        assert same(rc, ref) and same(cc, ref)


def test_hss_division_shape_checks(pkg, orc):
    """hssA \\ hssB and hssB / hssA reject mismatched sizes before any device
    work (host only)."""
    rng = np.random.default_rng(2)
    A = pkg.HssMatrix.from_tree(orc.synthetic_hss(512, 64, 8, rng))
    B = pkg.HssMatrix.from_tree(orc.synthetic_hss(640, 64, 8, rng))
    with pytest.raises(ValueError):
        pkg.hss_ldiv(A, B)
    with pytest.raises(ValueError):
        pkg.rdiv(B, A)


def test_failure_options_validate_arguments(lib, pkg):
    """The fault-injection switches check their values on the host (no GPU needed)."""
    L = pkg._lib
    assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, -1) == L.HSS_ERR_INVALID
    assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, 1 << 33) == L.HSS_ERR_INVALID
    assert lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, -1) == L.HSS_ERR_INVALID
    assert lib.hss_set_option(L.HSS_OPT_POLL_LIMIT, 0) == L.HSS_OK
    assert lib.hss_set_option(L.HSS_OPT_FAIL_ALLOC, 0) == L.HSS_OK
    assert lib.hss_set_option(99, 1) == L.HSS_ERR_INVALID
