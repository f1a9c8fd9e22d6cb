"""Serving form: continuous batching over resident factorizations (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_against_alone(pkg, orc, reqs):
    factored = {}
    for r in reqs:
        if r.kind == "factor":
            factored[r.matrix] = r.hss
    alone = {}
    for r in reqs:
        if r.kind != "solve":
            continue
        h = factored[r.matrix]
        if r.matrix not in alone:
            alone[r.matrix] = (pkg.HssMatrix.from_tree(h).device().ulvfactor("fp32"), orc.full(h))
        F, A = alone[r.matrix]
        b = r.rhs.cpu().numpy().T
        x_alone = F.solve(b, tol=1e-10)
        x_mix = r.out.cpu().numpy().T
        assert np.linalg.norm(x_mix - x_alone) <= 1e-8 * np.linalg.norm(x_alone)
        res = np.linalg.norm(b - A @ x_mix, axis=0) / np.linalg.norm(b, axis=0)
        assert res.max() <= 2e-10
        assert r.done >= r.arrival


@pytest.mark.parametrize("overlap", [True, False])
def test_served_results_equal_alone(pkg, orc, overlap):
    torch = pytest.importorskip("torch")
    from hssmatrices_gb300 import serve
    reqs, pool = serve.synthetic_requests(n_requests=80, seed=5, rate=4000.0, factor_frac=0.25,
                                          n_range=(300, 1500), k_range=(8, 16), leafsize=64, r_range=(1, 6),
                                          pool_size=4, recent=4)
    # a budget of about two matrices forces evictions and reloads
    need = max(serve.HssServer.estimate_bytes(h, "fp32") for h in pool)
    srv = serve.HssServer(budget_bytes=2 * need + 1, precision="fp32", tol=1e-10, overlap=overlap)
    done = serve.run_stream(srv, reqs, time_scale=1.0)
    assert len(done) == len(reqs) and len({id(r) for r in done}) == len(reqs)
    assert srv.evictions > 0 and srv.batches > 1
    _check_against_alone(pkg, orc, reqs)


def test_requests_arriving_during_a_batch_overlap_it(pkg, orc):
    """Factor requests that arrive while a solve batch runs are factored on the
    factor stream during that batch; every result still equals the solo solve."""
    torch = pytest.importorskip("torch")
    from hssmatrices_gb300 import serve
    reqs, pool = serve.synthetic_requests(n_requests=400, seed=6, rate=1500.0, factor_frac=0.3,
                                          n_range=(2000, 8000), k_range=(8, 24), leafsize=64, r_range=(1, 8),
                                          pool_size=6, recent=4)
    srv = serve.HssServer(budget_bytes=10**11, precision="fp32", tol=1e-10, overlap=True)
    done = serve.run_stream(srv, reqs, time_scale=1.0)
    assert len(done) == len(reqs)
    assert srv.overlapped > 0, "no factor batch was launched while a solve batch ran"
    assert srv.solve_batches > 1 and srv.factor_batches > 1
    _check_against_alone(pkg, orc, reqs)


def test_batcher_rejects_repeated_factor(pkg, orc):
    torch = pytest.importorskip("torch")
    from hssmatrices_gb300 import serve
    h = pkg.HssMatrix.from_tree(orc.synthetic_hss(400, 64, 8, np.random.default_rng(1)))
    b = serve.Batcher()
    (f,) = b.factor([h.device()], "fp64")
    B = torch.randn((2, 400), dtype=torch.float64, device="cuda")
    X = torch.empty_like(B)
    with pytest.raises(ValueError):
        b.solve([f, f], [B, B], [X, X], [400, 400], [2, 2])
