"""Model drivers on the GPU against the reference's own outputs (tests/golden) and
the oracle: MCMC replay with host-fed streams, conjugate fit + prediction,
response prediction, replicated data."""
import numpy as np
import pytest

from conftest import cm, xorder

pytestmark = pytest.mark.gpu

TOL = 1e-9  # FP64 mode; the chain's arithmetic differs from the reference's only in rounding


def mcmc_args(g, model):
    t = f"mc{model}"
    return dict(y=g["mc_y"], X=g["mc_X"], m=10, coords=g["mc_coords"], cov_model=model, nn_indx=g["mc_nnIndx"],
                nn_indx_lu=g["mc_lu"], sigma_sq_IG=[2, 1], tau_sq_IG=[2, 0.1], phi_unif=[3, 30],
                nu_unif=[0.5, 2.5], beta_starting=[1.0, -0.5], theta_starting=g[f"{t}_theta_start"],
                tuning=g[f"{t}_tuning"], n_samples=150, normals=g[f"{t}_normals"], unifs=g[f"{t}_unifs"], n_rep=5,
                rep_indx=g[f"{t}_repindx"])


@pytest.mark.parametrize("model", [0, 2])
def test_rNNGP_replays_reference_chain(sp, golden, model):
    r = sp.rNNGP(**mcmc_args(golden, model), precision="fp64")
    t = f"mc{model}"
    th, gth = r["p.theta.samples"], golden[f"{t}_theta"]
    # identical accept/reject sequence: the chain moves at exactly the same iterations
    moved = np.any(np.diff(th, axis=1) != 0, axis=0)
    gmoved = np.any(np.diff(gth, axis=1) != 0, axis=0)
    assert np.array_equal(moved, gmoved)
    assert np.max(np.abs(th - gth) / np.abs(gth)) <= TOL
    assert np.max(np.abs(r["p.beta.samples"] - golden[f"{t}_beta"])) <= 1e-8
    assert np.max(np.abs(r["y.rep.samples"] - golden[f"{t}_rep"])) <= 1e-8


@pytest.mark.parametrize("model", [0, 2])
def test_rNNGP_fp32r_same_decisions(sp, golden, model):
    a = mcmc_args(golden, model)
    r = sp.rNNGP(**a, precision="fp32r")
    t = f"mc{model}"
    th, gth = r["p.theta.samples"], golden[f"{t}_theta"]
    moved = np.any(np.diff(th, axis=1) != 0, axis=0)
    gmoved = np.any(np.diff(gth, axis=1) != 0, axis=0)
    # log-target error <= 1e-6 relative: decisions agree except on knife-edge uniforms
    assert np.mean(moved == gmoved) >= 0.97
    assert np.allclose(th.mean(axis=1), gth.mean(axis=1), rtol=0.05)


def test_rNNGP_matches_oracle_longer(sp, orc):
    rng = np.random.default_rng(21)
    n, m, p, nS = 1500, 15, 2, 400
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = X @ [1.0, -0.5] + rng.normal(size=n)
    o = orc.mkNNIndxCB(cm(c), m)
    normals = rng.normal(size=nS * 5 + 10)
    unifs = rng.uniform(size=nS + 2)
    args = (y, cm(X), m, cm(c), 0, o[0], o[2], [2, 1], [2, 0.1], [3, 30], [0, 0], [1.0, -0.5], [1.0, 0.2, 6.0],
            [0.1, 0.1, 0.4], nS, normals, unifs)
    ro = orc.rNNGP(*args)
    rg = sp.rNNGP(y, X, m, c, "exponential", o[0], o[2], [2, 1], [2, 0.1], [3, 30], None, [1.0, -0.5],
                  [1.0, 0.2, 6.0], [0.1, 0.1, 0.4], nS, normals, unifs)
    assert rg["accept"] == ro["accept"]
    assert np.max(np.abs(rg["p.theta.samples"] - ro["theta"]) / ro["theta"]) <= TOL


def test_rNNGP_zero_tuning_consumes_no_draw(sp, orc):
    rng = np.random.default_rng(22)
    n, m, nS = 400, 10, 60
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = X @ [1.0, -0.5] + rng.normal(size=n)
    o = orc.mkNNIndxCB(cm(c), m)
    normals = rng.normal(size=nS * 5)
    unifs = rng.uniform(size=nS)
    tun = [0.0, 0.1, 0.3]  # sigma.sq fixed: rnorm(mu, 0) returns mu without a draw
    ro = orc.rNNGP(y, cm(X), m, cm(c), 0, o[0], o[2], [2, 1], [2, 0.1], [3, 30], [0, 0], [1.0, -0.5],
                   [1.0, 0.2, 6.0], tun, nS, normals, unifs)
    rg = sp.rNNGP(y, X, m, c, 0, o[0], o[2], [2, 1], [2, 0.1], [3, 30], None, [1.0, -0.5], [1.0, 0.2, 6.0], tun,
                  nS, normals, unifs)
    assert np.max(np.abs(rg["p.theta.samples"] - ro["theta"]) / ro["theta"]) <= TOL
    assert np.all(rg["p.theta.samples"][0] == 1.0)


def test_rNNGP_stream_too_short_raises(sp, golden):
    a = mcmc_args(golden, 0)
    a["normals"] = a["normals"][:50]
    with pytest.raises(sp.NNGPError) as e:
        sp.rNNGP(**a)
    assert e.value.status == 5


@pytest.mark.parametrize("model", [0, 2])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32r", 1e-5)])
def test_cNNGP_matches_reference(sp, golden, model, precision, tol):
    g = golden
    t = f"cj{model}"
    r = sp.cNNGP(g["mc_y"], g["mc_X"], g["mc_coords"], g[f"{t}_theta_alpha"].T, g["mc_nnIndx"], g["mc_lu"], g["cj_X0"],
                 g["cj_coords0"], g["cj_nnIndx0"], 10, [2.0, 1.0], model, precision=precision)
    for k, ref in (("beta.hat", g[f"{t}_beta"]), ("ab", g[f"{t}_ab"]), ("bb", g[f"{t}_bb"]),
                   ("y.0.hat", g[f"{t}_y0"]), ("y.0.hat.var", g[f"{t}_y0var"])):
        assert np.max(np.abs(r[k] - ref)) <= tol * max(1.0, np.max(np.abs(ref))), k
    p = 2
    for j in range(r["bB.inv"].shape[1]):
        low = np.tril(r["bB.inv"][:, j].reshape(p, p).T)
        ref = np.tril(g[f"{t}_bBInv"][:, j].reshape(p, p).T)
        assert np.max(np.abs(low - ref)) <= tol * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32r", 1e-5)])
def test_rNNGPPredict_matches_reference(sp, golden, precision, tol):
    g = golden
    r = sp.rNNGPPredict(g["mc_X"], g["mc_y"], g["mc_coords"], 10, g["cj_X0"], g["cj_coords0"], g["cj_nnIndx0"],
                        g["pr_beta"], g["pr_theta"], 0, g["pr_z"], precision=precision)
    assert np.max(np.abs(r["p.y.0"] - g["pr_y0"])) <= tol * max(1.0, np.max(np.abs(g["pr_y0"])))


def test_rNNGPReplicated_matches_reference(sp, golden):
    g = golden
    r = sp.rNNGPReplicated(g["mc_X"], 10, g["mc_coords"], 0, g["mc_nnIndx"], g["mc_lu"], g["rp_beta"],
                           g["pr_theta"], g["rp_normals"])
    assert np.max(np.abs(r["y.rep.samples"] - g["rp_yrep"])) <= 1e-9 * max(1.0, np.max(np.abs(g["rp_yrep"])))


@pytest.mark.parametrize("model,theta", [(0, (1.0, 0.1, 6.0)), (2, (1.0, 0.2, 12.0, 1.5))])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32r", 1e-6)])
def test_rNNGPReplicated_dataflow_solve_matches_oracle(sp, orc, model, theta, precision, tol):
    """The dataflow solve (warps take locations in index order and wait for their neighbors)
    against the oracle's sequential recurrence at a size whose neighbor DAG has ~1200 levels."""
    rng = np.random.default_rng(71)
    n, m, p, nS = 20000, 15, 2, 6
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    o = orc.mkNNIndxCB(cm(c), m)
    nT = len(theta)
    th = np.array(theta)[:, None] * rng.uniform(0.8, 1.25, size=(nT, nS))
    beta = rng.normal(size=(nS, p))
    z = rng.normal(size=n * nS)
    r = sp.rNNGPReplicated(X, m, c, model, o[0], o[2], beta, th, z, precision=precision)
    yo, st = orc.rNNGPReplicated(cm(X), m, cm(c), model, o[0], o[2], beta, cm(th), z)
    assert st == 0
    assert np.max(np.abs(r["y.rep.samples"] - yo)) <= tol * max(1.0, np.max(np.abs(yo)))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32r", 1e-6)])
def test_rNNGPReplicated_unordered_locations_match_oracle(sp, orc, precision, tol):
    """Locations in no spatial order (brute-force neighbor lists): index order is still a
    topological order of the neighbor DAG, so the dataflow solve needs no ordering."""
    rng = np.random.default_rng(74)
    n, m, p, nS = 3000, 10, 2, 3
    c = rng.uniform(size=(n, 2))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    o = orc.mkNNIndx(cm(c), m)
    th = np.array([1.0, 0.1, 6.0])[:, None] * rng.uniform(0.8, 1.25, size=(3, nS))
    beta = rng.normal(size=(nS, p))
    z = rng.normal(size=n * nS)
    r = sp.rNNGPReplicated(X, m, c, 0, o[0], o[2], beta, th, z, precision=precision)
    yo, st = orc.rNNGPReplicated(cm(X), m, cm(c), 0, o[0], o[2], beta, cm(th), z)
    assert st == 0
    assert np.max(np.abs(r["y.rep.samples"] - yo)) <= tol * max(1.0, np.max(np.abs(yo)))


def test_rNNGPReplicated_rejects_non_predecessor_neighbors(sp, orc):
    """A neighbor list naming a later location is refused by the replicate solve's own check."""
    rng = np.random.default_rng(72)
    n, m = 500, 10
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    o = orc.mkNNIndxCB(cm(c), m)
    nn = o[0].copy()
    lu = o[2]
    nn[lu[300]] = 400  # location 300's first neighbor: a successor
    with pytest.raises(sp.NNGPError) as e:
        sp.rNNGPReplicated(X, m, c, 0, nn, lu, rng.normal(size=(2, 2)), np.array([[1.0, 1.0], [0.1, 0.1], [6.0, 6.0]]),
                           rng.normal(size=2 * n))
    assert e.value.status == 1


def test_rNNGP_replicates_match_oracle_at_scale(sp, orc):
    """fit.rep in the response MCMC: the recorded draws, made after the chain by the level
    solve, against the oracle's in-chain sequential recurrence."""
    rng = np.random.default_rng(73)
    n, m, p, nS, nR = 6000, 15, 2, 40, 4
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = X @ [1.0, -0.5] + rng.normal(size=n)
    o = orc.mkNNIndxCB(cm(c), m)
    ri = np.zeros(nS, np.int32)
    ri[[5, 17, 30, 39]] = 1
    normals = rng.normal(size=nS * 5 + nR * n + 8)
    unifs = rng.uniform(size=nS + 2)
    args = (y, cm(X), m, cm(c), 0, o[0], o[2], [2, 1], [2, 0.1], [3, 30], [0, 0], [1.0, -0.5], [1.0, 0.2, 6.0],
            [0.1, 0.1, 0.4], nS, normals, unifs)
    ro = orc.rNNGP(*args, n_rep=nR, rep_indx=ri)
    rg = sp.rNNGP(y, X, m, c, 0, o[0], o[2], [2, 1], [2, 0.1], [3, 30], None, [1.0, -0.5], [1.0, 0.2, 6.0],
                  [0.1, 0.1, 0.4], nS, normals, unifs, n_rep=nR, rep_indx=ri)
    assert rg["accept"] == ro["accept"]
    assert np.max(np.abs(rg["y.rep.samples"] - ro["rep"])) <= 1e-9 * max(1.0, np.max(np.abs(ro["rep"])))


def test_cNNGP_many_grid_points_match_oracle(sp, orc):
    rng = np.random.default_rng(31)
    n, m, p, n0 = 3000, 15, 3, 300
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=(n, p - 1))])
    y = X @ np.arange(1, p + 1) + rng.normal(size=n)
    c0 = rng.uniform(size=(n0, 2))
    X0 = np.column_stack([np.ones(n0), rng.normal(size=(n0, p - 1))])
    o = orc.mkNNIndxCB(cm(c), m)
    nn0, _ = orc.nn2(c, c0, m)
    ta = np.array([[phi, a] for phi in np.linspace(3, 30, 8) for a in np.linspace(0.05, 2, 5)]).T
    ro = orc.cNNGP(y, cm(X), cm(c), ta.T.reshape(-1), o[0], o[2], cm(X0), cm(c0), cm(nn0), m, [2, 1], 0)
    rg = sp.cNNGP(y, X, c, ta, o[0], o[2], X0, c0, nn0, m, [2, 1], "exponential")
    assert np.max(np.abs(rg["beta.hat"] - ro["beta"])) <= 1e-9
    assert np.max(np.abs(rg["y.0.hat"] - ro["y0"])) <= 1e-9
    assert np.max(np.abs(rg["y.0.hat.var"] - ro["y0var"]) / ro["y0var"]) <= 1e-9


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32r", 1e-6)])
def test_cNNGP_multi_matches_single_problem_runs(sp, orc, precision, tol):
    from spnngp_gb300 import api

    rng = np.random.default_rng(41)
    problems, singles = [], []
    ta = np.array([[phi, a] for phi in (3.0, 9.0, 25.0) for a in (0.1, 0.8)]).T
    for k, n in enumerate((1200, 2500, 1800)):  # uneven folds
        c = xorder(rng.uniform(size=(n, 2)))
        X = np.column_stack([np.ones(n), rng.normal(size=n)])
        y = X @ [1.0, -0.5] + rng.normal(size=n)
        n0 = 150 + 40 * k
        c0 = rng.uniform(size=(n0, 2))
        X0 = np.column_stack([np.ones(n0), rng.normal(size=n0)])
        y0 = X0 @ [1.0, -0.5] + rng.normal(size=n0)
        o = orc.mkNNIndxCB(cm(c), 12)
        nn0, _ = orc.nn2(c, c0, 12)
        P = {"y": y, "X": X, "coords": c, "nn_indx": o[0], "nn_indx_lu": o[2], "theta_alpha": ta, "X0": X0,
             "coords0": c0, "nn_indx0": nn0, "y0_true": y0}
        problems.append(P)
        singles.append(sp.cNNGP(y, X, c, ta, o[0], o[2], X0, c0, nn0, 12, [2, 1], "exponential",
                                precision=precision))
    outs = sp.cNNGP_multi(problems, 12, [2, 1], "exponential", precision=precision)
    for P, o, s in zip(problems, outs, singles):
        for k in ("beta.hat", "ab", "bb", "y.0.hat", "y.0.hat.var"):
            assert np.allclose(o[k], s[k], rtol=tol, atol=tol), k
        for j in range(ta.shape[1]):
            assert o["crps"][j] == pytest.approx(api.crps(P["y0_true"], s["y.0.hat"][:, j], s["y.0.hat.var"][:, j]),
                                                 rel=1e-9)
            assert o["rmspe"][j] == pytest.approx(api.rmspe(P["y0_true"], s["y.0.hat"][:, j]), rel=1e-9)


def _chain(sp, rng, n, m, model, nS, p=2):
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n)] + [rng.normal(size=n) for _ in range(p - 1)])
    y = X @ np.linspace(1.0, -0.5, p) + rng.normal(size=n)
    knn = sp.mkNNIndxCB(c, m)
    nn, lu = knn["nnIndx"], knn["nnIndxLU"]
    nTheta = 4 if model == 2 else 3
    return {"y": y, "X": X, "coords": c, "nn_indx": nn, "nn_indx_lu": lu, "m": m, "cov_model": model,
            "sigma_sq_IG": [2, 1], "tau_sq_IG": [2, 0.1], "phi_unif": [3, 30], "nu_unif": [0.2, 2.0],
            "beta_starting": np.linspace(1.0, -0.5, p), "theta_starting": [1.0, 0.2, 6.0, 0.8][:nTheta],
            "tuning": [0.1, 0.1, 0.4, 0.1][:nTheta], "n_samples": nS,
            "normals": rng.normal(size=nS * (p + nTheta) + 5), "unifs": rng.uniform(size=nS + 1)}


@pytest.mark.parametrize("precision", ["fp64", "fp32r"])
def test_rNNGP_batch_same_as_each_chain_alone(sp, precision):
    """Chains of uneven size, both neighbor classes and all four models, advanced together, give
    exactly the draws each gives alone."""
    rng = np.random.default_rng(31)
    specs = [(700, 10, 0, 40), (1800, 15, 1, 25), (450, 20, 2, 30), (1200, 32, 3, 40), (900, 5, 0, 0),
             (2500, 16, 2, 35)]
    chains = [_chain(sp, rng, *s) for s in specs]
    batch = sp.rNNGP_batch(chains, precision=precision)
    for P, r in zip(chains, batch):
        if P["n_samples"] == 0:
            assert r["accept"] == 0 and r["p.theta.samples"].size == 0
            continue
        a = sp.rNNGP(P["y"], P["X"], P["m"], P["coords"], P["cov_model"], P["nn_indx"], P["nn_indx_lu"],
                     P["sigma_sq_IG"], P["tau_sq_IG"], P["phi_unif"], P["nu_unif"] if P["cov_model"] == 2 else None,
                     P["beta_starting"], P["theta_starting"], P["tuning"], P["n_samples"], P["normals"], P["unifs"],
                     precision=precision)
        assert r["accept"] == a["accept"]
        assert np.array_equal(r["p.theta.samples"], a["p.theta.samples"])
        assert np.array_equal(r["p.beta.samples"], a["p.beta.samples"])


def test_rNNGP_batch_matches_oracle(sp, orc):
    rng = np.random.default_rng(32)
    chains = [_chain(sp, rng, 800, 12, 0, 60), _chain(sp, rng, 600, 20, 3, 60)]
    batch = sp.rNNGP_batch(chains)
    for P, r in zip(chains, batch):
        ro = orc.rNNGP(P["y"], cm(P["X"]), P["m"], cm(P["coords"]), P["cov_model"], P["nn_indx"], P["nn_indx_lu"],
                       P["sigma_sq_IG"], P["tau_sq_IG"], P["phi_unif"], [0, 0], P["beta_starting"],
                       P["theta_starting"], P["tuning"], P["n_samples"], P["normals"], P["unifs"])
        assert r["accept"] == ro["accept"]
        assert np.max(np.abs(r["p.theta.samples"] - ro["theta"]) / ro["theta"]) <= TOL


@pytest.fixture(scope="module")
def config0():
    import os

    from conftest import ROOT

    return np.load(os.path.join(ROOT, "tests", "golden", "config0_golden.npz"))


def test_config0_chain_replays_reference(sp, config0):
    """The n = 2000, m = 15 response model, 2000 samples, against the reference's own chain
    (tests/golden/config0_golden.npz): bit-exact neighbor lists, then the FP64 chain moves at
    exactly the reference's iterations with theta and beta equal to rounding."""
    g = config0
    knn = sp.mkNNIndxCB(g["coords"], 15)
    assert np.array_equal(knn["nnIndx"], g["nnIndx"]) and np.array_equal(knn["nnIndxLU"], g["lu"])
    assert np.array_equal(knn["nnDist"], g["nnDist"])
    r = sp.rNNGP(g["y"], g["X"], 15, g["coords"], "exponential", g["nnIndx"], g["lu"], [2, 1], [2, 0.1], [3, 30],
                 None, [1.0, -0.5], g["theta_start"], g["tuning"], 2000, g["normals"], g["unifs"], precision="fp64")
    th, gth = r["p.theta.samples"], g["theta"]
    moved = np.any(np.diff(th, axis=1) != 0, axis=0)
    gmoved = np.any(np.diff(gth, axis=1) != 0, axis=0)
    assert np.array_equal(moved, gmoved)
    assert np.max(np.abs(th - gth) / np.abs(gth)) <= TOL
    assert np.max(np.abs(r["p.beta.samples"] - g["beta"])) <= 1e-8


def test_config0_chain_fp32r_posterior(sp, config0):
    """The same chain in FP32R: log-target error <= 1e-6 relative, so the decisions agree with the
    reference's except on knife-edge uniforms, and the posterior means agree within Monte Carlo
    error (the batch-means standard error of the reference's chain, after 500 burn-in samples)."""
    g = config0
    r = sp.rNNGP(g["y"], g["X"], 15, g["coords"], "exponential", g["nnIndx"], g["lu"], [2, 1], [2, 0.1], [3, 30],
                 None, [1.0, -0.5], g["theta_start"], g["tuning"], 2000, g["normals"], g["unifs"], precision="fp32r")
    th, gth = r["p.theta.samples"], g["theta"]
    moved = np.any(np.diff(th, axis=1) != 0, axis=0)
    gmoved = np.any(np.diff(gth, axis=1) != 0, axis=0)
    assert np.mean(moved == gmoved) >= 0.97
    keep = slice(500, None)
    for a, b in ((th, gth), (r["p.beta.samples"], g["beta"])):
        batches = b[:, keep].reshape(b.shape[0], 15, -1).mean(axis=2)
        se = batches.std(axis=1, ddof=1) / np.sqrt(15)
        assert np.all(np.abs(a[:, keep].mean(axis=1) - b[:, keep].mean(axis=1)) <= 3 * se + 1e-12)


@pytest.mark.parametrize("model,phi,alpha,nu", [(0, 6.0, 0.3, 0.0), (2, 9.0, 0.5, 1.2)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32r", 1e-6)])
def test_updateConjBF_matches_reference(sp, orc, model, phi, alpha, nu, precision, tol):
    """updateConjBF (sigma^2 = 1, nugget alpha, src/cNNGP.cpp:24-69) through its own C-ABI entry
    point, against the oracle's updateBF at theta = (1, alpha, phi[, nu]): the conjugate form is
    the response form at unit variance."""
    rng = np.random.default_rng(61)
    n, m = 3000, 15
    c = xorder(rng.uniform(size=(n, 2)))
    o = orc.mkNNIndxCB(cm(c), m)
    B, F = sp.updateConjBF(c, o[0], o[2], m, model, phi, alpha, nu, precision=precision)
    Bo, Fo, _, st = orc.updateBF(cm(c), o[0], o[2], m, model, 1.0, alpha, phi, nu)
    assert st == 0
    assert np.max(np.abs(B - Bo)) <= tol * max(1.0, np.max(np.abs(Bo)))
    assert np.max(np.abs(F - Fo) / Fo) <= tol
