"""The oracle pinned to the LAPACK routines the reference calls (CPU).

The oracle restates ``geqlf!``/``ormql!`` as a QR of the reversed matrix and
``gelqf!``/``ormlq!`` as a QR of the transpose.  ``oracle/lapack_ulv.py``
calls ``dgeqlf``, ``dormql``, ``dgelqf``, ``dormlq``, ``dtrsm``, ``dgetrf`` and
``dgetrs`` themselves (OpenBLAS, as Julia's LinearAlgebra links them), in the
order of src/ulvfactor.jl.  These tests check that both give the same
reflectors and the same solutions on every golden fixture.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, unpack_tree

lap = pytest.importorskip("oracle.lapack_ulv")
if not lap.available():
    pytest.skip("SciPy's OpenBLAS does not export the LQ/QL routines here", allow_module_level=True)

REFLECTOR_TOL = 1e-15   # relative, per factor (reflectors and tau)
SOLVE_TOL = 1e-14       # relative, oracle solve vs the LAPACK transcription, for cond(A) <= 45;
                        # above, cond(A) * eps / 4 (rounding differences grow with the conditioning)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("m,k", [(128, 32), (64, 32), (62, 16), (96, 95), (40, 1)])
def test_ql_reflectors_match_dgeqlf(orc, m, k):
    """QLFact (QR of the reversed U) = dgeqlf (src/ulvfactor.jl:39)."""
    rng = np.random.default_rng(m * 1000 + k)
    U = rng.standard_normal((m, k))
    A, tau = lap.geqlf(U)
    q = orc.QLFact(U)
    # QR of J_m U J_k: reflector i of the QR is reflector k-1-i of the QL, rows reversed
    assert _rel(q.qr[::-1, ::-1], A) <= REFLECTOR_TOL
    assert _rel(q.tau[::-1], tau) <= REFLECTOR_TOL
    assert _rel(q.L(), np.tril(A[m - k:, :])) <= REFLECTOR_TOL
    D = rng.standard_normal((m, 7))
    assert _rel(q.apply_qt(D), lap.ormql("L", "T", A, tau, D)) <= 4 * REFLECTOR_TOL


@pytest.mark.parametrize("mk,n", [(96, 128), (32, 64), (46, 62), (1, 5), (30, 30)])
def test_lq_reflectors_match_dgelqf(orc, mk, n):
    """LQFact (QR of the transpose) = dgelqf (src/ulvfactor.jl:44) and its three applications."""
    rng = np.random.default_rng(mk * 1000 + n)
    X = rng.standard_normal((mk, n))
    A, tau = lap.gelqf(X)
    q = orc.LQFact(X)
    r = min(mk, n)
    assert _rel(q.qr[:, :r].T, A[:r, :]) <= REFLECTOR_TOL
    assert _rel(q.tau, tau) <= REFLECTOR_TOL
    assert _rel(q.L(), np.tril(A)[:, :r]) <= REFLECTOR_TOL
    Cr = rng.standard_normal((9, n))
    Cl = rng.standard_normal((n, 6))
    assert _rel(q.apply_right_qt(Cr), lap.ormlq("R", "T", A, tau, Cr)) <= 4 * REFLECTOR_TOL   # :47
    assert _rel(q.apply_left_q(Cl), lap.ormlq("L", "N", A, tau, Cl)) <= 4 * REFLECTOR_TOL     # :50
    assert _rel(q.apply_left_qt(Cl), lap.ormlq("L", "T", A, tau, Cl)) <= 4 * REFLECTOR_TOL    # :102


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_solve_matches_lapack_transcription(orc, case):
    """ulvfactsolve of the oracle = ulvfactor.jl over LAPACK, on every golden fixture."""
    g = load_golden(case)
    h = unpack_tree(g["table"], g["packed"], orc)
    x_lap = lap.ulvfactsolve(h, g["b"])
    x_orc = orc.ulvfactsolve(h, g["b"])
    tol = max(SOLVE_TOL, np.linalg.cond(orc.full(h)) * np.finfo(float).eps / 4)
    assert _rel(x_orc, x_lap) <= tol
    # the fixture's stored solution (from the oracle) is the LAPACK one too
    assert _rel(g["z"], x_lap) <= tol


def test_lapack_transcription_solves_the_system(orc):
    """Against a dense LU solve of full(hssA): the transcription is a solver, not a copy of the oracle."""
    rng = np.random.default_rng(5)
    h = orc.synthetic_hss(1000, 64, 12, rng)
    b = rng.standard_normal((1000, 3))
    x = lap.ulvfactsolve(h, b)
    x0 = np.linalg.solve(orc.full(h), b)
    assert _rel(x, x0) <= 1e-11
