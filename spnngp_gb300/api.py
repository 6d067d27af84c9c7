"""Host-side mirror of spNNGP's R front-ends for the response and conjugate models.

``spNNGP(method="response")`` (R/spNNGP.R:1-504), ``spConjNNGP`` (R/spConjNNGP.R:1-522)
and ``predict`` (predict.NNGP, R/generics.R:532-683) keep the reference's argument
names (dots become underscores), defaults, checks and return objects; a formula is
replaced by ``y`` and ``X`` (the model matrix, intercept included when wanted).
Everything numeric runs on the GB300 through the C ABI.

Random numbers: the reference draws from R's global generator.  Here every call
takes ``seed`` (or a ``numpy.random.Generator`` as ``rng``) and builds the
host-fed streams in the reference's consumption order; an R binding fills the
same streams from R's generator (norm_rand / unif_rand, in the same order) instead.
"""
from __future__ import annotations

import math
import time
import warnings

import numpy as np

from . import core
from ._lib import Context

COV_MODELS = core.COV_MODELS


def _rng(seed=None, rng=None) -> np.random.Generator:
    if rng is not None:
        return rng
    return np.random.default_rng(seed)


def _lower(d) -> dict:
    return {str(k).lower().replace("_", "."): v for k, v in (d or {}).items()}


def _as_X(X, n) -> np.ndarray:
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X[:, None]
    if X.shape[0] != n:
        raise ValueError("error: X must have one row per observation")
    return X


def _coords(coords, n) -> np.ndarray:
    c = np.asarray(coords, dtype=np.float64)
    if c.ndim != 2 or c.shape[0] != n or c.shape[1] != 2:
        raise ValueError("error: either coords has more than two columns or the number of rows is different "
                         "than data used in the model formula")
    return c


def _quants(a) -> np.ndarray:
    return np.quantile(a, [0.5, 0.05, 0.975], axis=1).T


def mk_n_indx_list(nn_indx, n, m):
    """1-based neighbor lists per location, as R/util.R:272-279 (first entry NA -> None)."""
    out = [None]
    for i in range(1, n):
        if i < m:
            off, cnt = int(i / 2 * (i - 1)), i
        else:
            off, cnt = int(m / 2 * (m - 1) + (i - m) * m), m
        out.append(np.asarray(nn_indx[off:off + cnt]) + 1)
    return out


# ------------------------------------------------------------------- response

def mcmc_streams(rng, n_samples, p, n, n_theta, tuning, rep_indx=None):
    """Normal and uniform streams in the order rNNGP consumes R's generator
    (src/rNNGP.cpp:294,309-313,327-333,349)."""
    n_prop = sum(1 for t in tuning[:n_theta] if t != 0)
    n_rep = int(np.sum(rep_indx)) if rep_indx is not None else 0
    normals = rng.standard_normal(n_samples * (p + n_prop) + n_rep * n)
    unifs = rng.uniform(size=n_samples)
    return normals, unifs


def spNNGP(y, X, coords, method="response", family="gaussian", n_neighbors=15, starting=None, tuning=None,
           priors=None, cov_model="exponential", n_samples=None, n_omp_threads=1, search_type="cb", ord=None,
           return_neighbor_info=False, neighbor_info=None, fit_rep=False, sub_sample=None, verbose=False,
           n_report=100, seed=None, rng=None, normals=None, unifs=None, precision="fp64",
           ctx: Context | None = None, **kw):
    """Response NNGP model (R/spNNGP.R).  Returns the reference's NNGP object as a dict."""
    for k in kw:
        warnings.warn(f"'{k}' is not an argument")
    method = str(method).lower()
    if method not in ("response", "latent"):
        raise ValueError(f"error: specified method '{method}' is not a valid option; choose from response, latent.")
    if method == "latent":
        raise NotImplementedError("method='latent' (the sequential latent Gibbs sweep) is outside this build's "
                                  "hot path; only the response and conjugate models run on the GB300")
    if str(family).lower() != "gaussian":
        raise ValueError("error: only the latent method can be used with non-Gaussain family.")
    y = np.asarray(y, dtype=np.float64).reshape(-1)
    n = len(y)
    X = _as_X(X, n)
    p = X.shape[1]
    coords = _coords(coords, n)
    cov_model = str(cov_model).lower()
    if cov_model not in COV_MODELS:
        raise ValueError(f"error: specified cov.model '{cov_model}' is not a valid option; choose from "
                         + ", ".join(COV_MODELS) + ".")
    cov_idx = COV_MODELS.index(cov_model)
    matern = cov_model == "matern"

    # neighbors and ordering (R/spNNGP.R:97-146)
    provided = neighbor_info is not None
    if provided:
        warnings.warn("Using user defined neighbor.info. No checks are done on the supplied neighbor information.")
        ni = neighbor_info
        if not all(k in ni for k in ("n.neighbors", "nn.indx", "nn.indx.lu", "ord")):
            raise ValueError("The supplied neighbor.info is malformed.")
        nn_indx, nn_indx_lu, ord_ = ni["nn.indx"], ni["nn.indx.lu"], np.asarray(ni["ord"])
        n_neighbors = int(ni["n.neighbors"])
        nn_run_time = ni.get("nn.indx.run.time")
    else:
        if ord is None:
            ord_ = np.argsort(coords[:, 0], kind="stable")
        else:
            ord_ = np.asarray(ord)
            if len(ord_) != n:
                raise ValueError("error: supplied order vector ord must be of length n")
    coords_o, X_o, y_o = coords[ord_], X[ord_], y[ord_]

    # priors (R/spNNGP.R:183-224)
    if priors is None:
        raise ValueError("error: prior list for the parameters must be specified")
    pr = _lower(priors)
    sig_ig = np.asarray(pr.get("sigma.sq.ig", None) if "sigma.sq.ig" in pr else None, dtype=float) \
        if "sigma.sq.ig" in pr else None
    if sig_ig is None:
        raise ValueError("error: sigma.sq.IG must be specified")
    if sig_ig.size != 2 or np.any(sig_ig <= 0):
        raise ValueError("error: sigma.sq.IG must be a positive vector of length 2")
    if "tau.sq.ig" not in pr:
        raise ValueError("error: tau.sq.IG must be specified")
    tau_ig = np.asarray(pr["tau.sq.ig"], dtype=float)
    if tau_ig.size != 2 or np.any(tau_ig <= 0):
        raise ValueError("error: tau.sq.IG must be a positive vector of length 2")
    if "phi.unif" not in pr:
        raise ValueError("error: phi.Unif must be specified")
    phi_u = np.asarray(pr["phi.unif"], dtype=float)
    if phi_u.size != 2 or np.any(phi_u <= 0) or phi_u[0] >= phi_u[1]:
        raise ValueError("error: phi.Unif must be a positive vector of length 2 with element 1 < element 2")
    nu_u = np.zeros(2)
    if matern:
        if "nu.unif" not in pr:
            raise ValueError("error: nu.Unif must be specified")
        nu_u = np.asarray(pr["nu.unif"], dtype=float)
        if nu_u.size != 2 or np.any(nu_u <= 0) or nu_u[0] >= nu_u[1]:
            raise ValueError("error: nu.Unif must be a positive vector of length 2 with element 1 < element 2")

    # starting and tuning (R/spNNGP.R:229-299)
    if starting is None:
        raise ValueError("error: starting value list for the parameters must be specified")
    st = _lower(starting)
    if "beta" not in st:
        beta_start = np.linalg.lstsq(X_o, y_o, rcond=None)[0]
    else:
        beta_start = np.asarray(st["beta"], dtype=float).reshape(-1)
        if len(beta_start) != p:
            raise ValueError("error: supplied beta.starting is the wrong length")
    for k in ("sigma.sq", "tau.sq", "phi") + (("nu",) if matern else ()):
        if k not in st:
            raise ValueError(f"error: {k} must be specified in starting value list")
    theta_start = [float(np.ravel(st["sigma.sq"])[0]), float(np.ravel(st["tau.sq"])[0]), float(np.ravel(st["phi"])[0])]
    if matern:
        theta_start.append(float(np.ravel(st["nu"])[0]))
    if tuning is None:
        raise ValueError("error: tuning value vector for the spatial parameters must be specified")
    tu = _lower(tuning)
    for k in ("sigma.sq", "tau.sq", "phi") + (("nu",) if matern else ()):
        if k not in tu:
            raise ValueError(f"error: {k} must be specified in tuning value list")
    tun = [float(np.ravel(tu["sigma.sq"])[0]), float(np.ravel(tu["tau.sq"])[0]), float(np.ravel(tu["phi"])[0])]
    if matern:
        tun.append(float(np.ravel(tu["nu"])[0]))
    if n_samples is None:
        raise ValueError("error: n.samples must be specified")

    # neighbor search (R/spNNGP.R:304-351)
    if not provided:
        if search_type not in ("brute", "cb"):
            raise ValueError(f"error: specified search.type '{search_type}' is not a valid option; choose from "
                             "brute, cb.")
        idx = (core.mkNNIndx if search_type == "brute" else core.mkNNIndxCB)(coords_o, n_neighbors, ctx=ctx)
        nn_indx, nn_indx_lu, nn_run_time = idx["nnIndx"], idx["nnIndxLU"], idx["run.time"]

    # fitted / replicated samples (R/spNNGP.R:356-380)
    n_rep, rep_indx, s_indx = 0, None, None
    if fit_rep:
        ss = dict(sub_sample or {})
        start = ss.get("start", math.floor(0.5 * n_samples))
        end = ss.get("end", n_samples)
        thin = ss.get("thin", 1)
        if start >= n_samples:
            raise ValueError("error: in sub.sample, invalid start")
        if end > n_samples:
            raise ValueError("error: in sub.sample, invalid end")
        if thin >= n_samples:
            raise ValueError("error: in sub.sample, invalid thin")
        s_indx = np.arange(int(start), int(end) + 1, int(thin))  # 1-based sample numbers
        sub_sample = {"start": start, "end": end, "thin": thin}
        n_rep = len(s_indx)
        rep_indx = np.zeros(n_samples, np.int32)
        rep_indx[s_indx - 1] = 1

    if normals is None or unifs is None:
        normals, unifs = mcmc_streams(_rng(seed, rng), n_samples, p, n, len(theta_start), tun, rep_indx)

    t0 = time.perf_counter()
    out = core.rNNGP(y_o, X_o, n_neighbors, coords_o, cov_idx, nn_indx, nn_indx_lu, sig_ig, tau_ig, phi_u, nu_u,
                     beta_start, theta_start, tun, n_samples, normals, unifs, n_rep=n_rep, rep_indx=rep_indx,
                     precision=precision, ctx=ctx)
    res = {"run.time": time.perf_counter() - t0}
    col = ["sigma.sq", "tau.sq", "phi"] + (["nu"] if matern else [])
    res["p.theta.samples"] = out["p.theta.samples"].T  # n.samples x nTheta (coda::mcmc layout)
    res["p.beta.samples"] = out["p.beta.samples"].T
    res["theta.names"] = col
    res["acceptance"] = out["accept"] / max(n_samples, 1)
    if return_neighbor_info:
        res["neighbor.info"] = {"n.neighbors": n_neighbors, "n.indx": mk_n_indx_list(nn_indx, n, n_neighbors),
                                "nn.indx": nn_indx, "nn.indx.lu": nn_indx_lu, "ord": ord_,
                                "nn.indx.run.time": nn_run_time}
    inv = np.argsort(ord_, kind="stable")
    res["coords"], res["y"], res["X"] = coords_o[inv], y_o[inv], X_o[inv]
    if fit_rep:
        beta_sub = res["p.beta.samples"][s_indx - 1]
        res["y.hat.samples"] = res["X"] @ beta_sub.T
        res["y.hat.quants"] = _quants(res["y.hat.samples"])
        res["y.rep.samples"] = out["y.rep.samples"][inv]
        res["y.rep.quants"] = _quants(res["y.rep.samples"])
        res["sub.sample"] = sub_sample
        res["s.indx"] = s_indx
    res.update({"n.neighbors": n_neighbors, "cov.model": cov_model, "cov.model.indx": cov_idx,
                "starting": starting, "priors": priors, "tuning": tuning, "type": ("response", "gaussian"),
                "class": "NNGP", "precision": precision})
    return res


# ------------------------------------------------------------------ conjugate

def crps(y, y_hat, y_var):
    """R/util.R:247-251 (negatively oriented, lower is better)."""
    from math import erf, pi, sqrt

    sd = np.sqrt(y_var)
    z = (y - y_hat) / sd
    pdf = np.exp(-0.5 * z * z) / np.sqrt(2 * pi)
    cdf = 0.5 * (1 + np.vectorize(erf)(z / sqrt(2)))
    return float(np.mean(-sd * (1 / np.sqrt(pi) - 2 * pdf - z * (2 * cdf - 1))))


def rmspe(y, y_hat):
    """R/util.R:253-255."""
    return float(np.sqrt(np.mean((y - y_hat) ** 2)))


def _theta_alpha_matrix(theta_alpha, matern):
    """Returns (g x nTheta array with columns phi, alpha[, nu], single_set)."""
    if isinstance(theta_alpha, dict):
        cols = {str(k).lower(): np.atleast_1d(np.asarray(v, dtype=float)) for k, v in theta_alpha.items()}
        for need in ("phi", "alpha") + (("nu",) if matern else ()):
            if need not in cols:
                raise ValueError(f"error: column name {need} must be specified in theta.alpha")
        g = len(cols["phi"])
        ta = np.column_stack([cols["phi"], cols["alpha"]] + ([cols["nu"]] if matern else []))
        single = g == 1 and all(np.ndim(v) == 0 for v in theta_alpha.values())
        return ta, single
    ta = np.asarray(theta_alpha, dtype=float)
    single = ta.ndim == 1
    ta = np.atleast_2d(ta)
    if ta.shape[1] != (3 if matern else 2):
        raise ValueError("error: theta.alpha needs columns (phi, alpha[, nu])")
    return ta, single


def spConjNNGP(y, X, coords, knots=None, n_neighbors=15, theta_alpha=None, sigma_sq_IG=None,
               cov_model="exponential", k_fold=5, score_rule="crps", X_0=None, coords_0=None, n_omp_threads=1,
               search_type="cb", ord=None, return_neighbor_info=True, neighbor_info=None, fit_rep=False,
               n_samples=None, verbose=False, seed=None, rng=None, folds=None, precision="fp64",
               ctx: Context | None = None, **kw):
    """Conjugate NNGP with k-fold selection of (phi, alpha[, nu]) (R/spConjNNGP.R).

    ``folds`` (an extension for replay) is a list of k hold-out index arrays (0-based,
    in the NNGP order); by default each fold draws floor(n/k) indices independently
    without replacement, as R/spConjNNGP.R:289 does."""
    for k in kw:
        if k != "n_report":
            warnings.warn(f"'{k}' is not an argument")
    if knots is not None:
        raise NotImplementedError("knots= (the low-rank SLGP variant) is outside this build's hot path")
    gen = _rng(seed, rng)
    y = np.asarray(y, dtype=np.float64).reshape(-1)
    n = len(y)
    X = _as_X(X, n)
    p = X.shape[1]
    coords = _coords(coords, n)
    cov_model = str(cov_model).lower()
    if cov_model not in COV_MODELS:
        raise ValueError(f"error: specified cov.model '{cov_model}' is not a valid option; choose from "
                         + ", ".join(COV_MODELS) + ".")
    cov_idx = COV_MODELS.index(cov_model)
    matern = cov_model == "matern"
    if fit_rep and n_samples is None:
        raise ValueError("error: if fit.rep=TRUE, specify the number of fitted and replicated samples to generate "
                         "using the n.samples argument.")
    n_samples = 0 if n_samples is None else int(n_samples)

    provided = neighbor_info is not None
    if provided:
        ni = neighbor_info
        if not all(k in ni for k in ("n.neighbors", "nn.indx", "nn.indx.lu", "ord")):
            raise ValueError("The supplied neighbor.info is malformed.")
        nn_indx, nn_indx_lu, ord_ = ni["nn.indx"], ni["nn.indx.lu"], np.asarray(ni["ord"])
        n_neighbors = int(ni["n.neighbors"])
        nn_run_time = ni.get("nn.indx.run.time")
        warnings.warn("Using user defined neighbor.info, no checks are done on the supplied neighbor information.")
    else:
        ord_ = np.argsort(coords[:, 0], kind="stable") if ord is None else np.asarray(ord)
        if len(ord_) != n:
            raise ValueError("error: supplied order vector ord must be of length n")
    coords_o, X_o, y_o = coords[ord_], X[ord_], y[ord_]

    n0 = 0
    nn0 = None
    if X_0 is not None:
        X_0 = np.atleast_2d(np.asarray(X_0, dtype=float))
        if X_0.shape[1] != p:
            raise ValueError(f"error: X.0 must n.0-by-{p} matrix")
        n0 = X_0.shape[0]
        if coords_0 is None:
            raise ValueError("error: coords.0 must specified")
        coords_0 = np.atleast_2d(np.asarray(coords_0, dtype=float))
        if coords_0.shape != (n0, 2):
            raise ValueError("error: either coords.0 has more than two columns or the number of rows is different "
                             "than X.0")
        nn0, _ = core.nn2(coords_o, coords_0, n_neighbors, ctx=ctx)

    ta, single = _theta_alpha_matrix(theta_alpha, matern)
    if not single and (k_fold is None or k_fold < 2 or k_fold >= n):
        raise ValueError("error: k.fold must be greater than 1 and less than n")
    if sigma_sq_IG is None:
        raise ValueError("error: sigma.sq.IG must be specified")
    sig_ig = np.asarray(sigma_sq_IG, dtype=float)
    if sig_ig.size != 2 or np.any(sig_ig <= 0):
        raise ValueError("error: sigma.sq.IG must be a positive vector of length 2")

    if not provided:
        if search_type not in ("brute", "cb"):
            raise ValueError(f"error: specified search.type '{search_type}' is not a valid option; choose from "
                             "brute, cb.")
        idx = (core.mkNNIndx if search_type == "brute" else core.mkNNIndxCB)(coords_o, n_neighbors, ctx=ctx)
        nn_indx, nn_indx_lu, nn_run_time = idx["nnIndx"], idx["nnIndxLU"], idx["run.time"]

    t0 = time.perf_counter()
    res = {}
    if not single:
        if score_rule not in ("rmspe", "crps"):
            raise ValueError(f"error: specified score.rule '{score_rule}' is not a valid option; choose from "
                             "rmspe, crps.")
        scores = np.zeros((ta.shape[0], 2))  # columns rmspe, crps
        problems = []
        for f in range(int(k_fold)):
            if folds is not None:
                ho = np.sort(np.asarray(folds[f]))
            else:
                ho = np.sort(gen.choice(n, size=n // int(k_fold), replace=False))
            keep = np.ones(n, bool)
            keep[ho] = False
            cm_, Xm, ym = coords_o[keep], X_o[keep], y_o[keep]
            ch, Xh, yh = coords_o[ho], X_o[ho], y_o[ho]
            idx = (core.mkNNIndx if search_type == "brute" else core.mkNNIndxCB)(cm_, n_neighbors, ctx=ctx)
            nnh, _ = core.nn2(cm_, ch, n_neighbors, ctx=ctx)
            problems.append({"y": ym, "X": Xm, "coords": cm_, "nn_indx": idx["nnIndx"], "nn_indx_lu": idx["nnIndxLU"],
                             "theta_alpha": ta.T, "X0": Xh, "coords0": ch, "nn_indx0": nnh, "y0_true": yh})
        # every fold x every parameter set in one fused launch, scored on the device
        outs = core.cNNGP_multi(problems, n_neighbors, sig_ig, cov_idx, precision=precision, want_pred=False,
                                ctx=ctx)
        for o in outs:
            scores[:, 1] += o["crps"]
            scores[:, 0] += o["rmspe"]
        scores /= int(k_fold)
        col = 1 if score_rule == "crps" else 0
        best = int(np.argmin(scores[:, col]))
        res["k.fold.scores"] = np.column_stack([ta, scores])
        ta = ta[best:best + 1]

    out = core.cNNGP(y_o, X_o, coords_o, ta.T, nn_indx, nn_indx_lu, X_0, coords_0, nn0, n_neighbors, sig_ig,
                     cov_idx, precision=precision, ctx=ctx)
    res["run.time"] = time.perf_counter() - t0
    names = ["phi", "alpha"] + (["nu"] if matern else [])
    res["theta.alpha"] = dict(zip(names, ta[0]))
    a, b = out["ab"][0, 0], out["ab"][1, 0]
    res["ab"] = out["ab"]
    res["sigma.sq.hat"] = b / (a - 1)
    res["sigma.sq.var"] = b ** 2 / ((a - 1) ** 2 * (a - 2))
    res["beta.hat"] = out["beta.hat"][:, 0]
    Binv = out["bB.inv"][:, 0].reshape(p, p).T  # column-major p x p, lower valid
    Binv = np.tril(Binv) + np.tril(Binv, -1).T
    res["bB.inv"] = out["bB.inv"]
    res["bb"] = out["bb"][:, 0]
    res["beta.var"] = b * Binv / (a - 1)
    if n0:
        res["y.0.hat"] = out["y.0.hat"][:, 0]
        res["y.0.hat.var"] = out["y.0.hat.var"][:, 0]
    res.update({"sigma.sq.IG": sig_ig, "n.neighbors": n_neighbors, "cov.model": cov_model,
                "cov.model.indx": cov_idx, "search.type": search_type})
    if return_neighbor_info:
        res["neighbor.info"] = {"n.neighbors": n_neighbors, "n.indx": mk_n_indx_list(nn_indx, n, n_neighbors),
                                "nn.indx": nn_indx, "nn.indx.lu": nn_indx_lu, "ord": ord_,
                                "nn.indx.run.time": nn_run_time}
    # exact posterior sampling (R/spConjNNGP.R:423-436): sigma^2 ~ IG(a, b), beta | sigma^2 ~
    # N(bB.inv bb, sigma^2 bB.inv), tau^2 = alpha sigma^2, on the device from host-fed Gamma(a, 1)
    # variates and normals (one gamma and p normals per sample)
    if n_samples > 0:
        alpha = ta[0, 1]
        draws = core.conj_posterior_samples(res["bb"], Binv, a, b, alpha, gen.gamma(a, size=n_samples),
                                            gen.standard_normal(n_samples * p), ctx=ctx)
        res["p.beta.theta.samples"] = draws
        if fit_rep:
            inv_o = np.argsort(ord_, kind="stable")
            beta = draws[:, :p]
            res["y.hat.samples"] = (X_o @ beta.T)[inv_o]
            res["y.hat.quants"] = _quants(res["y.hat.samples"])
            th = np.column_stack([draws[:, p], draws[:, p + 1], np.full(n_samples, ta[0, 0])] +
                                 ([np.full(n_samples, ta[0, 2])] if matern else []))
            zn = gen.standard_normal(n * n_samples)
            rep = core.rNNGPReplicated(X_o, n_neighbors, coords_o, cov_idx, nn_indx, nn_indx_lu, beta, th.T, zn,
                                       precision=precision, ctx=ctx)
            res["y.rep.samples"] = rep["y.rep.samples"][inv_o]
            res["y.rep.quants"] = _quants(res["y.rep.samples"])
            res["sub.sample"] = {"start": 1, "end": n_samples, "thin": 1}
            res["s.indx"] = np.arange(1, n_samples + 1)
    inv = np.argsort(ord_, kind="stable")
    res["coords"], res["y"], res["X"] = coords_o[inv], y_o[inv], X_o[inv]
    res["type"] = ("conjugate", "gaussian")
    res["class"] = "NNGP"
    res["precision"] = precision
    return res


# -------------------------------------------------------------------- predict

def predict(obj: dict, X_0, coords_0, sub_sample=None, n_omp_threads=1, verbose=False, n_report=100, seed=None,
            rng=None, z=None, precision=None, ctx: Context | None = None):
    """predict.NNGP (R/generics.R:532-683) for response and conjugate fits."""
    if obj.get("class") != "NNGP":
        raise ValueError("error: requires an output object of class NNGP")
    precision = precision or obj.get("precision", "fp64")
    X_0 = np.atleast_2d(np.asarray(X_0, dtype=float))
    coords_0 = np.atleast_2d(np.asarray(coords_0, dtype=float))
    out = {"type": obj["type"]}
    t0 = time.perf_counter()
    if obj["type"][0] == "conjugate":
        if sub_sample is not None:
            warnings.warn("'sub.sample' is not an argument for prediction using a conjugate model.")
        r = spConjNNGP(obj["y"], obj["X"], obj["coords"], n_neighbors=obj["n.neighbors"],
                       theta_alpha=obj["theta.alpha"], sigma_sq_IG=obj["sigma.sq.IG"], cov_model=obj["cov.model"],
                       X_0=X_0, coords_0=coords_0, search_type=obj["search.type"], precision=precision, ctx=ctx)
        out.update(r)
    else:
        X, y, coords = obj["X"], obj["y"], obj["coords"]
        n, p = X.shape
        if X_0.shape[1] != p:
            raise ValueError(f"error: X.0 must have {p} columns")
        if coords_0.shape[1] != 2:
            raise ValueError("error: coords.0 must have two columns")
        th, be = obj["p.theta.samples"], obj["p.beta.samples"]
        n_s = th.shape[0]
        ss = dict(sub_sample or {})
        start, end, thin = ss.get("start", 1), ss.get("end", n_s), ss.get("thin", 1)
        if start >= n_s:
            raise ValueError("invalid start")
        if end > n_s:
            raise ValueError("invalid end")
        if thin >= n_s:
            raise ValueError("invalid thin")
        s_indx = np.arange(int(start), int(end) + 1, int(thin)) - 1
        q = X_0.shape[0]
        nn0, _ = core.nn2(coords, coords_0, obj["n.neighbors"], ctx=ctx)
        if z is None:
            z = _rng(seed, rng).standard_normal(q * len(s_indx))
        r = core.rNNGPPredict(X, y, coords, obj["n.neighbors"], X_0, coords_0, nn0, be[s_indx].T, th[s_indx].T,
                              obj["cov.model.indx"], z, precision=precision, ctx=ctx)
        out["p.y.0"] = r["p.y.0"]
        out["sub.sample"] = {"start": start, "end": end, "thin": thin}
    out["run.time"] = time.perf_counter() - t0
    out["class"] = "predict.NNGP"
    return out
