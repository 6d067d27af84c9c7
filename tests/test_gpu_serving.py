"""The continuous-batching conjugate server on the GPU: a request's result is the same alone and
in a mixed batch, matches the per-request host form and the oracle, and the HBM-budget admission
splits work across iterations without changing results."""
import numpy as np
import pytest

from conftest import cm

pytestmark = pytest.mark.gpu


def make_request(rng, n, n0, rid, dataset=None, phi=None, alpha=None, data=None):
    if data is None:
        c = rng.uniform(size=(n, 2))
        X = np.column_stack([np.ones(n), rng.normal(size=n)])
        y = X @ [1.0, -0.5] + np.sin(6 * c[:, 0]) * np.cos(4 * c[:, 1]) + rng.normal(scale=0.3, size=n)
        data = (c, X, y)
    c, X, y = data
    c0 = rng.uniform(size=(n0, 2))
    X0 = np.column_stack([np.ones(n0), rng.normal(size=n0)])
    from spnngp_gb300.serving import ConjRequest

    return ConjRequest(c, X, y, c0, X0, phi if phi is not None else rng.uniform(3, 30),
                       alpha if alpha is not None else rng.uniform(0.05, 2), dataset=dataset, rid=rid)


FIELDS = ("beta_hat", "ab", "bB_inv", "bb", "y0_hat", "y0_hat_var")


@pytest.mark.parametrize("precision", ["fp64", "fp32r"])
def test_same_result_alone_and_in_mix(sp, precision):
    from spnngp_gb300.serving import ConjServer

    rng = np.random.default_rng(5)
    target = make_request(rng, 3000, 700, rid=0, dataset="A")
    alone = ConjServer(precision=precision)
    alone.submit(target)
    ra = alone.step()
    assert len(ra) == 1 and ra[0].error is None
    mix = ConjServer(precision=precision)
    others = [make_request(rng, n, n0, rid=k + 1) for k, (n, n0) in enumerate([(5000, 300), (800, 2000), (12000, 50)])]
    same_ds = make_request(rng, 3000, 400, rid=9, dataset="A", data=(target.coords, target.X, target.y))
    for r in others[:2] + [same_ds, target] + others[2:]:
        mix.submit(r)
    rm = {r.rid: r for r in mix.step()}
    assert len(rm) == 5 and mix.iterations == 1
    for f in FIELDS:
        assert np.array_equal(getattr(ra[0], f), getattr(rm[0], f)), f
    assert mix.stats["hits"] == 1 and mix.stats["misses"] == 4


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32r", 1e-6)])
def test_server_matches_per_request_form(sp, precision, tol):
    from spnngp_gb300.serving import ConjServer, fit_predict_one

    rng = np.random.default_rng(6)
    reqs = [make_request(rng, n, n0, rid=k) for k, (n, n0) in enumerate([(2500, 500), (6000, 1200), (900, 90)])]
    srv = ConjServer(precision=precision)
    for r in reqs:
        srv.submit(r)
    got = {r.rid: r for r in srv.step()}
    for r in reqs:
        ref = fit_predict_one(r, precision="fp64")
        for f in FIELDS:
            a, b = getattr(got[r.rid], f), getattr(ref, f)
            assert np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b))), f


def test_server_matches_oracle(sp, orc):
    from spnngp_gb300.serving import ConjServer

    rng = np.random.default_rng(7)
    req = make_request(rng, 1500, 300, rid=0, phi=8.0, alpha=0.4)
    srv = ConjServer(precision="fp64")
    srv.submit(req)
    got = srv.step()[0]
    o = np.argsort(req.coords[:, 0], kind="stable")
    c, X, y = req.coords[o], req.X[o], req.y[o]
    nn, _, lu = orc.mkNNIndxCB(cm(c), 15)
    nn0, _ = orc.nn2(c, req.coords0, 15)
    ro = orc.cNNGP(y, cm(X), cm(c), [8.0, 0.4], nn, lu, cm(req.X0), cm(req.coords0), cm(nn0), 15, [2.0, 1.0], 0)
    for f, k in (("beta_hat", "beta"), ("ab", "ab"), ("bb", "bb"), ("y0_hat", "y0"), ("y0_hat_var", "y0var")):
        ref = ro[k][:, 0]
        assert np.max(np.abs(getattr(got, f) - ref)) <= 1e-9 * max(1.0, np.max(np.abs(ref))), f


def test_budget_splits_batches_and_rejects_oversized(sp):
    from spnngp_gb300.serving import ConjServer, dataset_bytes, request_bytes, search_bytes

    rng = np.random.default_rng(8)
    reqs = [make_request(rng, 4000, 500, rid=k) for k in range(4)]
    one = dataset_bytes(4000, 2, 15) + request_bytes(4000, 500, 2, 15) + search_bytes(4000, 15)
    big = ConjServer(precision="fp64")
    for r in reqs:
        big.submit(r)
    ref = {r.rid: r for r in big.step()}
    small = ConjServer(precision="fp64", hbm_budget=int(1.5 * one))
    for r in reqs:
        small.submit(r)
    got = {r.rid: r for r in small.drain()}
    assert small.iterations >= 2
    for k in ref:
        for f in FIELDS:
            assert np.array_equal(getattr(ref[k], f), getattr(got[k], f)), f
    tiny = ConjServer(precision="fp64", hbm_budget=one // 2)
    tiny.submit(reqs[0])
    res = tiny.drain()
    assert res[0].error is not None and tiny.stats["rejected"] == 1


def test_serve_replays_stream(sp):
    from spnngp_gb300.serving import ConjServer, serve

    rng = np.random.default_rng(9)
    reqs = [make_request(rng, 2000, 200, rid=k, dataset=k % 3) for k in range(12)]
    data = {}
    for r in reqs:  # requests on one dataset carry the same data
        data.setdefault(r.dataset, (r.coords, r.X, r.y))
        r.coords, r.X, r.y = data[r.dataset]
    t = np.cumsum(rng.exponential(1 / 200.0, size=len(reqs)))
    for r, a in zip(reqs, t):
        r.arrival = float(a)
    out = serve(ConjServer(), reqs)
    assert out["completed"] == 12 and out["failed"] == 0
    assert out["p50_s"] > 0 and out["p99_s"] >= out["p50_s"]


def test_cached_datasets_match_fresh_builds(sp):
    """Datasets a server builds back to back in one batch (torch sorts and gathers the
    coordinates, the library searches neighbors) are identical to fresh builds, and the served
    results equal the per-request form bitwise.  Guards the ordering between torch's work and
    the library's kernels."""
    import torch

    from spnngp_gb300.serving import ConjServer, fit_predict_one

    rng = np.random.default_rng(12)
    reqs = [make_request(rng, n, 2000, rid=k, dataset=k) for k, n in enumerate([60000, 25000, 90000, 40000, 15000])]
    srv = ConjServer(precision="fp64")
    for r in reqs:
        srv.submit(r)
    got = {r.rid: r for r in srv.drain()}
    torch.cuda.synchronize()
    for r in reqs:
        fresh = ConjServer(precision="fp64")
        f = fresh._dataset(r, "fresh")
        torch.cuda.synchronize()
        for name in ("coords", "X", "y", "nn", "lu"):
            assert torch.equal(srv.datasets[r.dataset].tensors[name], f.tensors[name]), (r.rid, name)
        ref = fit_predict_one(r, precision="fp64")
        for fld in FIELDS:
            assert np.array_equal(getattr(got[r.rid], fld), getattr(ref, fld)), (r.rid, fld)
