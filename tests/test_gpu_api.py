"""The R front-end mirror (spnngp_gb300.api) end to end: ordering, neighbor search,
fold selection, posterior summaries and prediction, checked against the same
steps composed from the oracle."""
import numpy as np
import pytest

from conftest import cm

pytestmark = pytest.mark.gpu


def data(n, seed, p=2):
    rng = np.random.default_rng(seed)
    coords = rng.uniform(size=(n, 2))
    X = np.column_stack([np.ones(n)] + [rng.normal(size=n) for _ in range(p - 1)])
    D = np.sqrt(((coords[:, None, :] - coords[None, :, :]) ** 2).sum(-1))
    w = np.linalg.cholesky(np.exp(-6.0 * D) + 1e-9 * np.eye(n)) @ rng.normal(size=n)
    y = X @ np.r_[1.0, -0.5, 0.3][:p] + w + rng.normal(scale=0.3, size=n)
    return coords, X, y


def test_spNNGP_response_matches_oracle_chain(orc):
    from spnngp_gb300 import api

    coords, X, y = data(400, 1)
    starting = {"phi": 6.0, "sigma.sq": 1.0, "tau.sq": 0.1}
    tuning = {"phi": 0.5, "sigma.sq": 0.1, "tau.sq": 0.1}
    priors = {"phi.Unif": [3, 30], "sigma.sq.IG": [2, 1], "tau.sq.IG": [2, 0.1]}
    fit = api.spNNGP(y, X, coords, n_neighbors=10, starting=starting, tuning=tuning, priors=priors,
                     cov_model="exponential", n_samples=300, seed=5, return_neighbor_info=True, fit_rep=True)
    assert fit["p.theta.samples"].shape == (300, 3) and fit["p.beta.samples"].shape == (300, 2)
    assert 0.0 < fit["acceptance"] < 1.0
    assert np.array_equal(fit["coords"], coords) and np.array_equal(fit["y"], y)
    assert fit["y.rep.samples"].shape == (400, len(fit["s.indx"]))
    # the same chain from the oracle with the same streams, in the same NNGP order
    ord_ = fit["neighbor.info"]["ord"]
    c, Xo, yo = coords[ord_], X[ord_], y[ord_]
    o = orc.mkNNIndxCB(cm(c), 10)
    assert np.array_equal(o[0], fit["neighbor.info"]["nn.indx"])
    rep = np.zeros(300, np.int32)
    rep[fit["s.indx"] - 1] = 1
    normals, unifs = api.mcmc_streams(np.random.default_rng(5), 300, 2, 400, 3, [0.1, 0.1, 0.5], rep)
    beta0 = np.linalg.lstsq(Xo, yo, rcond=None)[0]
    r = orc.rNNGP(yo, cm(Xo), 10, cm(c), 0, o[0], o[2], [2, 1], [2, 0.1], [3, 30], [0, 0], beta0,
                  [1.0, 0.1, 6.0], [0.1, 0.1, 0.5], 300, normals, unifs, n_rep=int(rep.sum()), rep_indx=rep)
    assert np.max(np.abs(fit["p.theta.samples"].T - r["theta"]) / r["theta"]) <= 1e-9


def test_spConjNNGP_folds_and_prediction_match_oracle(orc):
    from spnngp_gb300 import api

    coords, X, y = data(600, 2)
    rng = np.random.default_rng(3)
    c0 = rng.uniform(size=(50, 2))
    X0 = np.column_stack([np.ones(50), rng.normal(size=50)])
    ta = np.array([[phi, a] for phi in (3.0, 8.0, 20.0) for a in (0.1, 0.5)])
    k = 4
    folds = [rng.choice(600, 150, replace=False) for _ in range(k)]
    fit = api.spConjNNGP(y, X, coords, n_neighbors=10, theta_alpha=ta, sigma_sq_IG=[2, 1], cov_model="exponential",
                         k_fold=k, score_rule="crps", X_0=X0, coords_0=c0, folds=folds)
    # the fold loop of R/spConjNNGP.R:287-358 composed from the oracle
    ord_ = np.argsort(coords[:, 0], kind="stable")
    c, Xo, yo = coords[ord_], X[ord_], y[ord_]
    scores = np.zeros((len(ta), 2))
    for f in range(k):
        ho = np.sort(folds[f])
        keep = np.ones(600, bool)
        keep[ho] = False
        o = orc.mkNNIndxCB(cm(c[keep]), 10)
        nnh, _ = orc.nn2(c[keep], c[ho], 10)
        r = orc.cNNGP(yo[keep], cm(Xo[keep]), cm(c[keep]), ta.reshape(-1), o[0], o[2], cm(Xo[ho]), cm(c[ho]),
                      cm(nnh), 10, [2, 1], 0)
        for j in range(len(ta)):
            scores[j, 1] += api.crps(yo[ho], r["y0"][:, j], r["y0var"][:, j])
            scores[j, 0] += api.rmspe(yo[ho], r["y0"][:, j])
    scores /= k
    assert np.allclose(fit["k.fold.scores"][:, 2:], scores, rtol=1e-9, atol=1e-12)
    best = ta[np.argmin(scores[:, 1])]
    assert fit["theta.alpha"]["phi"] == best[0] and fit["theta.alpha"]["alpha"] == best[1]
    o = orc.mkNNIndxCB(cm(c), 10)
    nn0, _ = orc.nn2(c, c0, 10)
    r = orc.cNNGP(yo, cm(Xo), cm(c), best, o[0], o[2], cm(X0), cm(c0), cm(nn0), 10, [2, 1], 0)
    assert np.allclose(fit["y.0.hat"], r["y0"][:, 0], rtol=1e-9, atol=1e-10)
    assert np.allclose(fit["beta.hat"], r["beta"][:, 0], rtol=1e-9)
    a, b = r["ab"][:, 0]
    assert fit["sigma.sq.hat"] == pytest.approx(b / (a - 1), rel=1e-9)
    # predict() on a conjugate fit re-runs the fit with the chosen parameters
    pr = api.predict(fit, X0, c0)
    assert np.allclose(pr["y.0.hat"], fit["y.0.hat"], rtol=1e-12)


def test_predict_response(orc):
    from spnngp_gb300 import api

    coords, X, y = data(300, 4)
    fit = api.spNNGP(y, X, coords, n_neighbors=8, starting={"phi": 6, "sigma.sq": 1, "tau.sq": 0.1},
                     tuning={"phi": 0.5, "sigma.sq": 0.1, "tau.sq": 0.1},
                     priors={"phi.Unif": [3, 30], "sigma.sq.IG": [2, 1], "tau.sq.IG": [2, 0.1]},
                     n_samples=100, seed=9)
    rng = np.random.default_rng(10)
    c0 = rng.uniform(size=(20, 2))
    X0 = np.column_stack([np.ones(20), rng.normal(size=20)])
    z = rng.normal(size=20 * 50)
    pr = api.predict(fit, X0, c0, sub_sample={"start": 51, "end": 100}, z=z)
    th = fit["p.theta.samples"][50:100].T
    be = fit["p.beta.samples"][50:100].T
    nn0, _ = orc.nn2(fit["coords"], c0, 8)
    ref, _ = orc.rNNGPPredict(cm(fit["X"]), fit["y"], cm(fit["coords"]), 8, cm(X0), cm(c0), cm(nn0), cm(be), cm(th),
                              0, z)
    assert np.allclose(pr["p.y.0"], ref, rtol=1e-9, atol=1e-9)


def test_unsupported_paths_raise():
    from spnngp_gb300 import api

    coords, X, y = data(50, 5)
    with pytest.raises(NotImplementedError):
        api.spNNGP(y, X, coords, method="latent", starting={}, tuning={}, priors={}, n_samples=1)
    with pytest.raises(ValueError):
        api.spNNGP(y, X, coords, cov_model="cubic", starting={}, tuning={}, priors={}, n_samples=1)


def test_spConjNNGP_posterior_samples_and_replicates():
    """Exact posterior sampling of the conjugate model at one (phi, alpha) (R/spConjNNGP.R:423-436):
    the draws' means match the closed-form posterior means within Monte Carlo error, tau^2 is
    alpha sigma^2, and fit.rep returns one fitted and one replicated draw per sample."""
    from spnngp_gb300 import api

    coords, X, y = data(800, 4)
    ns = 4000
    fit = api.spConjNNGP(y, X, coords, n_neighbors=10, theta_alpha=np.array([[6.0, 0.5]]), sigma_sq_IG=[2, 1],
                         cov_model="exponential", n_samples=ns, fit_rep=True, seed=11)
    d = fit["p.beta.theta.samples"]
    p = X.shape[1]
    assert d.shape == (ns, p + 2)
    assert np.allclose(d[:, p + 1], 0.5 * d[:, p])
    s2 = d[:, p]
    assert abs(s2.mean() - fit["sigma.sq.hat"]) <= 5 * np.sqrt(fit["sigma.sq.var"] / ns)
    sd = np.sqrt(np.diag(fit["beta.var"]))
    assert np.all(np.abs(d[:, :p].mean(axis=0) - fit["beta.hat"]) <= 5 * sd / np.sqrt(ns))
    assert fit["y.hat.samples"].shape == (800, ns) and fit["y.rep.samples"].shape == (800, ns)


def test_conjugate_posterior_samples_on_device(sp):
    """The exact posterior draws of the conjugate model (R/spConjNNGP.R:423-436) made on the device
    from host-fed Gamma(a, 1) variates and normals: each row equals the formula
    sigma^2 = b / g, beta = bB.inv bb + sigma chol(bB.inv) z, tau^2 = alpha sigma^2."""
    rng = np.random.default_rng(81)
    p, ns = 3, 5000
    A = rng.normal(size=(p, p))
    Binv = A @ A.T + p * np.eye(p)
    bb = rng.normal(size=p)
    a, b, alpha = 12.5, 3.25, 0.4
    g = rng.gamma(a, size=ns)
    z = rng.standard_normal(ns * p)
    got = sp.core.conj_posterior_samples(bb, Binv, a, b, alpha, g, z)
    L = np.linalg.cholesky(Binv)
    s2 = b / g
    beta = Binv @ bb + np.sqrt(s2)[:, None] * (z.reshape(ns, p) @ L.T)
    want = np.column_stack([beta, s2, alpha * s2])
    assert got.shape == (ns, p + 2)
    assert np.max(np.abs(got - want) / np.maximum(1.0, np.abs(want))) <= 1e-12
    # the draws' moments match the posterior: E[sigma^2] = b / (a - 1), Var(beta | .) = E[sigma^2] bB.inv
    assert abs(got[:, p].mean() - b / (a - 1)) <= 5 * np.std(got[:, p]) / np.sqrt(ns)
    assert np.allclose(np.cov(got[:, :p].T), b / (a - 1) * Binv, rtol=0.15, atol=0.05)


def test_conjugate_posterior_rejects_non_spd(sp):
    with pytest.raises(sp.NNGPError) as e:
        sp.core.conj_posterior_samples(np.ones(2), -np.eye(2), 3.0, 1.0, 0.5, np.ones(4), np.zeros(8))
    assert e.value.status == 3
