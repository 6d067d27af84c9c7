"""Low-level entry points, one per native routine of spNNGP's hot path.

Each function mirrors the R-level wrapper that calls the reference routine
(names and argument meaning as in R/nn.R and the .Call sites), returns numpy
arrays, and runs on the GB300 through the C ABI.  Coordinates may be given as an
n x 2 array (one row per location, the R ``coords`` matrix) or as the
column-major flat vector the .Call layer receives.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from ._lib import FP32R, FP64, ConjProblem, Context, MCMCProblem, NNGPError, default_context, dptr, f64, i32, iptr, n_indx

COV_MODELS = ("exponential", "spherical", "matern", "gaussian")  # R/spNNGP.R:172


def cov_model_index(cov_model) -> int:
    if isinstance(cov_model, (int, np.integer)):
        if not 0 <= int(cov_model) < 4:
            raise ValueError("cov.model index must be 0..3")
        return int(cov_model)
    name = str(cov_model).lower()
    if name not in COV_MODELS:
        raise ValueError(f"error: specified cov.model '{cov_model}' is not a valid option; choose from "
                         + ", ".join(COV_MODELS) + ".")
    return COV_MODELS.index(name)


def precision_code(precision) -> int:
    if precision in (FP64, "fp64", "FP64", None):
        return FP64
    if precision in (FP32R, "fp32r", "FP32R", "fp32", "mixed"):
        return FP32R
    raise ValueError("precision must be 'fp64' or 'fp32r'")


def coords_cm(coords) -> np.ndarray:
    """Column-major flat copy (x then y) of an n x 2 coordinate matrix."""
    a = np.asarray(coords, dtype=np.float64)
    if a.ndim == 2:
        if a.shape[1] != 2:
            raise ValueError("coords must be an n x 2 matrix")
        return np.ascontiguousarray(a.T).reshape(-1)
    return f64(a)


def _ctx(ctx: Context | None) -> Context:
    return ctx if ctx is not None else default_context()


# ------------------------------------------------------------------ neighbors

def mkNNIndxCB(coords, m: int, n_omp_threads: int = 1, ctx: Context | None = None) -> dict:
    """Ordered kNN by the code-book search (R/nn.R:53-76 -> src/nn.cpp:213-258)."""
    c = coords_cm(coords)
    n = len(c) // 2
    nI = n_indx(n, m)
    nnIndx = np.zeros(max(nI, 0), np.int32)
    nnDist = np.zeros(max(nI, 0), np.float64)
    lu = np.zeros(2 * n, np.int32)
    t0 = time.perf_counter()
    _ctx(ctx).call("nngp_mkNNIndxCB", n, m, dptr(c), iptr(nnIndx), dptr(nnDist), iptr(lu))
    return {"run.time": time.perf_counter() - t0, "nnIndx": nnIndx, "nnDist": nnDist, "nnIndxLU": lu}


def mkNNIndx(coords, m: int, n_omp_threads: int = 1, ctx: Context | None = None) -> dict:
    """Ordered kNN by exhaustive scan (R/nn.R:27-51 -> src/nn.cpp:63-111)."""
    c = coords_cm(coords)
    n = len(c) // 2
    nI = n_indx(n, m)
    nnIndx = np.zeros(max(nI, 0), np.int32)
    nnDist = np.zeros(max(nI, 0), np.float64)
    lu = np.zeros(2 * n, np.int32)
    t0 = time.perf_counter()
    _ctx(ctx).call("nngp_mkNNIndx", n, m, dptr(c), iptr(nnIndx), dptr(nnDist), iptr(lu))
    return {"run.time": time.perf_counter() - t0, "nnIndx": nnIndx, "nnDist": nnDist, "nnIndxLU": lu}


def mkUIndx(n: int, m: int, nn_indx, nn_indx_lu, search_type: int = 2, ctx: Context | None = None) -> dict:
    """Reverse neighbor index (R/nn.R:1-24 -> src/nn.cpp:25-56)."""
    nI = n_indx(n, m)
    nn, lu = i32(nn_indx), i32(nn_indx_lu)
    u = np.zeros(nI, np.int32)
    ulu = np.zeros(2 * n, np.int32)
    ui = np.zeros(nI, np.int32)
    t0 = time.perf_counter()
    _ctx(ctx).call("nngp_mkUIndx", n, m, iptr(nn), iptr(u), iptr(ulu), iptr(ui), iptr(lu), int(search_type))
    return {"run.time": time.perf_counter() - t0, "u.indx": u, "u.indx.lu": ulu, "ui.indx": ui}


def nn2(data, query, k: int, ctx: Context | None = None):
    """Exact kNN of query points among data points: (n0 x k 0-based indices, distances).
    Stands in for RANN::nn2 at R/spConjNNGP.R:158,311 and R/generics.R:642 (which add 1)."""
    c = coords_cm(data)
    c0 = coords_cm(query)
    n, n0 = len(c) // 2, len(c0) // 2
    idx = np.zeros(n0 * k, np.int32)
    dist = np.zeros(n0 * k, np.float64)
    if n0:
        _ctx(ctx).call("nngp_nn2", n, dptr(c), n0, dptr(c0), k, iptr(idx), dptr(dist))
    return idx.reshape(k, n0).T.copy(), dist.reshape(k, n0).T.copy()


# ---------------------------------------------------------------- B, F and Q

def _theta_vec(theta, model: int) -> np.ndarray:
    t = list(np.asarray(theta, np.float64).reshape(-1))
    need = 4 if model == 2 else 3
    if len(t) < need:
        raise ValueError("theta must be (sigma.sq, tau.sq, phi[, nu])")
    return f64(t + [0.0] * (4 - len(t)))


def updateBF(coords, nn_indx, nn_indx_lu, m: int, cov_model, theta, precision="fp64",
             ctx: Context | None = None):
    """B, F and sum(log F) at theta = (sigma.sq, tau.sq, phi[, nu]) (src/rNNGP.cpp:46-101)."""
    c = coords_cm(coords)
    n = len(c) // 2
    model = cov_model_index(cov_model)
    th = _theta_vec(theta, model)
    B = np.zeros(max(n_indx(n, m), 1))
    F = np.zeros(n)
    ld = np.zeros(1)
    _ctx(ctx).call("nngp_updateBF", n, m, dptr(c), iptr(i32(nn_indx)), iptr(i32(nn_indx_lu)), model, dptr(th),
                   precision_code(precision), dptr(B), dptr(F), dptr(ld))
    return B[: n_indx(n, m)], F, float(ld[0])


def updateConjBF(coords, nn_indx, nn_indx_lu, m: int, cov_model, phi, alpha, nu=0.0, precision="fp64",
                 ctx: Context | None = None):
    """B and F of the conjugate model (sigma^2 = 1, nugget alpha) (src/cNNGP.cpp:24-69)."""
    c = coords_cm(coords)
    n = len(c) // 2
    model = cov_model_index(cov_model)
    B = np.zeros(max(n_indx(n, m), 1))
    F = np.zeros(n)
    _ctx(ctx).call("nngp_updateConjBF", n, m, dptr(c), iptr(i32(nn_indx)), iptr(i32(nn_indx_lu)), model,
                   float(phi), float(alpha), float(nu), precision_code(precision), dptr(B), dptr(F))
    return B[: n_indx(n, m)], F


def Q(B, F, u, v, nn_indx, nn_indx_lu, ctx: Context | None = None) -> float:
    """u'(I-B)'F^-1(I-B)v (src/util.cpp:261-280)."""
    F = f64(F)
    out = np.zeros(1)
    Bf = f64(B) if len(B) else np.zeros(1)
    _ctx(ctx).call("nngp_Q", dptr(Bf), dptr(F), dptr(f64(u)), dptr(f64(v)), len(F), iptr(i32(nn_indx)),
                   iptr(i32(nn_indx_lu)), dptr(out))
    return float(out[0])


def loglik_gram(coords, nn_indx, nn_indx_lu, m: int, V, cov_model, theta, precision="fp64",
                ctx: Context | None = None):
    """(sum log F, V'(I-B)'F^-1(I-B)V) for V = [X y] (n x nv) in one fused pass."""
    c = coords_cm(coords)
    n = len(c) // 2
    V = np.asarray(V, np.float64)
    if V.ndim == 1:
        V = V[:, None]
    nv = V.shape[1]
    Vc = f64(np.asarray(V).T.reshape(-1))
    model = cov_model_index(cov_model)
    th = _theta_vec(theta, model)
    ld = np.zeros(1)
    G = np.zeros(nv * nv)
    _ctx(ctx).call("nngp_loglik_gram", n, m, nv, dptr(c), iptr(i32(nn_indx)), iptr(i32(nn_indx_lu)), dptr(Vc),
                   model, dptr(th), precision_code(precision), dptr(ld), dptr(G))
    return float(ld[0]), G.reshape(nv, nv)


# ------------------------------------------------------------------ drivers

def rNNGP(y, X, m: int, coords, cov_model, nn_indx, nn_indx_lu, sigma_sq_IG, tau_sq_IG, phi_unif, nu_unif,
          beta_starting, theta_starting, tuning, n_samples: int, normals, unifs, n_rep: int = 0, rep_indx=None,
          precision="fp64", ctx: Context | None = None) -> dict:
    """Response-model MCMC, the .Call("rNNGP", ...) routine (src/rNNGP.cpp:103-421).

    theta_starting / tuning are (sigma.sq, tau.sq, phi[, nu]).  normals / unifs are the host-fed
    streams consumed in the reference's order (p normals for beta, n for a replicate draw, one per
    proposal with non-zero tuning, one uniform per iteration).  Returns p.beta.samples (p x n),
    p.theta.samples (nTheta x n), y.rep.samples (n x n.rep) and the acceptance count."""
    y = f64(y)
    n = len(y)
    Xa = np.asarray(X, np.float64)
    Xc = f64(Xa.T.reshape(-1)) if Xa.ndim == 2 else f64(Xa)
    p = len(Xc) // n
    c = coords_cm(coords)
    model = cov_model_index(cov_model)
    nTheta = 4 if model == 2 else 3
    ts = f64(list(np.asarray(theta_starting, np.float64).reshape(-1)[:nTheta]) + [0.0] * (4 - nTheta))
    tu = f64(list(np.asarray(tuning, np.float64).reshape(-1)[:nTheta]) + [0.0] * (4 - nTheta))
    nu_u = f64(nu_unif if nu_unif is not None else [0.0, 0.0])
    normals, unifs = f64(normals), f64(unifs)
    ri = i32(rep_indx if rep_indx is not None else np.zeros(max(1, n_samples), np.int32))
    beta_s = np.zeros(max(1, p * n_samples))
    theta_s = np.zeros(max(1, nTheta * n_samples))
    rep = np.zeros(max(1, n * n_rep))
    acc = np.zeros(1, np.int32)
    _ctx(ctx).call("nngp_rNNGP", dptr(y), dptr(Xc), p, n, m, dptr(c), model, iptr(i32(nn_indx)),
                   iptr(i32(nn_indx_lu)), dptr(f64(sigma_sq_IG)), dptr(f64(tau_sq_IG)), dptr(f64(phi_unif)),
                   dptr(nu_u), dptr(f64(beta_starting)), dptr(ts), dptr(tu), int(n_samples), int(n_rep), iptr(ri),
                   dptr(normals), len(normals), dptr(unifs), len(unifs), precision_code(precision), dptr(beta_s),
                   dptr(theta_s), dptr(rep), iptr(acc))
    out = {"p.beta.samples": beta_s[: p * n_samples].reshape(n_samples, p).T,
           "p.theta.samples": theta_s[: nTheta * n_samples].reshape(n_samples, nTheta).T,
           "accept": int(acc[0])}
    if n_rep:
        out["y.rep.samples"] = rep[: n * n_rep].reshape(n_rep, n).T
    return out


def cNNGP(y, X, coords, theta_alpha, nn_indx, nn_indx_lu, X0, coords0, nn_indx0, m: int, sigma_sq_IG, cov_model,
          precision="fp64", ctx: Context | None = None) -> dict:
    """Conjugate NNGP over the columns of theta_alpha (nTheta x g, rows phi, alpha[, nu]) with prediction at
    coords0 -- the .Call("cNNGP", ...) routine (src/cNNGP.cpp:73-358).  nn_indx0 is n0 x m, 0-based."""
    y = f64(y)
    n = len(y)
    Xa = np.asarray(X, np.float64)
    Xc = f64(Xa.T.reshape(-1)) if Xa.ndim == 2 else f64(Xa)
    p = len(Xc) // n
    c = coords_cm(coords)
    model = cov_model_index(cov_model)
    nTheta = 3 if model == 2 else 2
    ta = np.asarray(theta_alpha, np.float64)
    ta = f64(ta.T.reshape(-1)) if ta.ndim == 2 else f64(ta)
    g = len(ta) // nTheta
    if coords0 is not None and len(np.asarray(coords0)):
        c0 = coords_cm(coords0)
        n0 = len(c0) // 2
        X0a = np.asarray(X0, np.float64)
        X0c = f64(X0a.T.reshape(-1)) if X0a.ndim == 2 else f64(X0a)
        nn0 = np.asarray(nn_indx0)
        nn0 = i32(nn0.T.reshape(-1)) if nn0.ndim == 2 else i32(nn0)
    else:
        n0, c0, X0c, nn0 = 0, np.zeros(2), np.zeros(1), np.zeros(1, np.int32)
    beta = np.zeros(p * g)
    ab = np.zeros(2 * g)
    bBInv = np.zeros(p * p * g)
    bb = np.zeros(p * g)
    y0 = np.zeros(max(1, n0 * g))
    y0v = np.zeros(max(1, n0 * g))
    _ctx(ctx).call("nngp_cNNGP", dptr(y), dptr(Xc), p, n, dptr(c), dptr(ta), iptr(i32(nn_indx)), iptr(i32(nn_indx_lu)),
                   dptr(X0c), dptr(c0), n0, iptr(nn0), g, m, dptr(f64(sigma_sq_IG)), model, precision_code(precision),
                   dptr(beta), dptr(ab), dptr(bBInv), dptr(bb), dptr(y0), dptr(y0v))
    out = {"beta.hat": beta.reshape(g, p).T, "ab": ab.reshape(g, 2).T, "bB.inv": bBInv.reshape(g, p * p).T,
           "bb": bb.reshape(g, p).T}
    if n0:
        out["y.0.hat"] = y0[: n0 * g].reshape(g, n0).T
        out["y.0.hat.var"] = y0v[: n0 * g].reshape(g, n0).T
    return out


def rNNGPPredict(X, y, coords, m: int, X0, coords0, nn_indx0, beta_samples, theta_samples, cov_model, z,
                 precision="fp64", ctx: Context | None = None) -> dict:
    """Posterior predictive draws (src/rNNGPPredict.cpp:25-223).  beta_samples p x nS, theta_samples
    nTheta x nS, z q*nS normals with z[i*nS + s] for (point i, sample s).  Returns p.y.0 (q x nS)."""
    y = f64(y)
    n = len(y)
    Xa = np.asarray(X, np.float64)
    Xc = f64(Xa.T.reshape(-1)) if Xa.ndim == 2 else f64(Xa)
    p = len(Xc) // n
    c = coords_cm(coords)
    c0 = coords_cm(coords0)
    q = len(c0) // 2
    X0a = np.asarray(X0, np.float64)
    X0c = f64(X0a.T.reshape(-1)) if X0a.ndim == 2 else f64(X0a)
    nn0 = np.asarray(nn_indx0)
    nn0 = i32(nn0.T.reshape(-1)) if nn0.ndim == 2 else i32(nn0)
    bs = np.asarray(beta_samples, np.float64)
    nS = bs.size // p
    bsc = f64(bs.T.reshape(-1)) if bs.ndim == 2 else f64(bs)
    ts = np.asarray(theta_samples, np.float64)
    tsc = f64(ts.T.reshape(-1)) if ts.ndim == 2 else f64(ts)
    y0 = np.zeros(max(1, q * nS))
    _ctx(ctx).call("nngp_rNNGPPredict", dptr(Xc), dptr(y), dptr(c), n, p, m, dptr(X0c), dptr(c0), q, iptr(nn0),
                   dptr(bsc), dptr(tsc), nS, cov_model_index(cov_model), dptr(f64(z)), precision_code(precision),
                   dptr(y0))
    return {"p.y.0": y0[: q * nS].reshape(nS, q).T}


def rNNGPReplicated(X, m: int, coords, cov_model, nn_indx, nn_indx_lu, beta, theta, normals, precision="fp64",
                    ctx: Context | None = None) -> dict:
    """Replicated data at every sample (src/rNNGPReplicated.cpp:74-244).  beta nS x p, theta nTheta x nS,
    normals n*nS consumed sample by sample.  Returns y.rep.samples (n x nS)."""
    c = coords_cm(coords)
    n = len(c) // 2
    Xa = np.asarray(X, np.float64)
    Xc = f64(Xa.T.reshape(-1)) if Xa.ndim == 2 else f64(Xa)
    p = len(Xc) // n
    b = np.asarray(beta, np.float64)
    nS = b.shape[0]
    ts = np.asarray(theta, np.float64)
    tsc = f64(ts.T.reshape(-1)) if ts.ndim == 2 else f64(ts)
    yr = np.zeros(n * nS)
    _ctx(ctx).call("nngp_rNNGPReplicated", dptr(Xc), p, n, m, dptr(c), cov_model_index(cov_model),
                   iptr(i32(nn_indx)), iptr(i32(nn_indx_lu)), dptr(f64(b.T.reshape(-1))), dptr(tsc), nS,
                   dptr(f64(normals)), precision_code(precision), dptr(yr))
    return {"y.rep.samples": yr.reshape(nS, n).T}


def conj_posterior_samples(bb, bB_inv, a: float, b: float, alpha: float, gammas, normals,
                           ctx: Context | None = None) -> np.ndarray:
    """Exact posterior draws of the conjugate model (R/spConjNNGP.R:423-436) on the device: rows
    (beta, sigma.sq, tau.sq), one per Gamma(a, 1) variate in gammas; normals holds p standard
    normals per sample.  bB_inv is p x p (its lower triangle is read)."""
    bb = f64(bb)
    p = len(bb)
    g = f64(gammas)
    ns = len(g)
    Bl = f64(np.asarray(bB_inv, np.float64).T.reshape(-1))  # column-major
    out = np.zeros(max(ns * (p + 2), 1))
    _ctx(ctx).call("nngp_conj_posterior_samples", p, dptr(bb), dptr(Bl), float(a), float(b), float(alpha), ns,
                   dptr(g), dptr(f64(normals)), dptr(out))
    return out[: ns * (p + 2)].reshape(p + 2, ns).T


def cNNGP_multi(problems, m: int, sigma_sq_IG, cov_model, precision="fp64", want_pred=True,
                ctx: Context | None = None) -> list:
    """Batched conjugate fits (nngp_cNNGP_multi): every (problem, parameter set) in one fused
    launch.  Each problem is a dict with y, X (n x p), coords (n x 2), nn_indx, nn_indx_lu,
    theta_alpha (nTheta x g) and optionally X0, coords0, nn_indx0 (n0 x m) and y0_true (held-out
    responses: the problem is then scored by CRPS and RMSPE per parameter set, R/util.R:247-255).
    Returns one dict per problem with beta.hat, ab, bB.inv, bb[, y.0.hat, y.0.hat.var][, crps, rmspe]."""
    model = cov_model_index(cov_model)
    nTheta = 3 if model == 2 else 2
    keep = []  # arrays must outlive the call
    structs = (ConjProblem * len(problems))()
    outs = []
    p = None
    for k, P in enumerate(problems):
        y = f64(P["y"])
        n = len(y)
        Xa = np.asarray(P["X"], np.float64)
        Xa = Xa[:, None] if Xa.ndim == 1 else Xa
        p = Xa.shape[1] if p is None else p
        Xc = f64(Xa.T.reshape(-1))
        c = coords_cm(P["coords"])
        ta = np.asarray(P["theta_alpha"], np.float64)
        ta = f64(ta.T.reshape(-1)) if ta.ndim == 2 else f64(ta)
        g = len(ta) // nTheta
        nn, lu = i32(P["nn_indx"]), i32(P["nn_indx_lu"])
        o = {"beta.hat": np.zeros(p * g), "ab": np.zeros(2 * g), "bB.inv": np.zeros(p * p * g), "bb": np.zeros(p * g)}
        st = structs[k]
        st.n, st.g = n, g
        st.y, st.X, st.coords, st.nnIndx, st.nnIndxLU, st.thetaAlpha = (a.ctypes.data for a in (y, Xc, c, nn, lu, ta))
        keep += [y, Xc, c, nn, lu, ta]
        if P.get("coords0") is not None and len(P["coords0"]):
            c0 = coords_cm(P["coords0"])
            n0 = len(c0) // 2
            X0 = np.asarray(P["X0"], np.float64)
            X0c = f64((X0[:, None] if X0.ndim == 1 else X0).T.reshape(-1))
            nn0 = np.asarray(P["nn_indx0"])
            nn0 = i32(nn0.T.reshape(-1)) if nn0.ndim == 2 else i32(nn0)
            st.n0 = n0
            st.X0, st.coords0, st.nnIndx0 = X0c.ctypes.data, c0.ctypes.data, nn0.ctypes.data
            keep += [X0c, c0, nn0]
            if want_pred:
                o["y.0.hat"], o["y.0.hat.var"] = np.zeros(n0 * g), np.zeros(n0 * g)
                st.y0Hat, st.y0HatVar = o["y.0.hat"].ctypes.data, o["y.0.hat.var"].ctypes.data
            if P.get("y0_true") is not None:
                yt = f64(P["y0_true"])
                keep.append(yt)
                st.y0True = yt.ctypes.data
                o["crps"], o["rmspe"] = np.zeros(g), np.zeros(g)
                st.crps, st.rmspe = o["crps"].ctypes.data, o["rmspe"].ctypes.data
        st.betaHat, st.ab, st.bBInv, st.bb = (o[k2].ctypes.data for k2 in ("beta.hat", "ab", "bB.inv", "bb"))
        outs.append((o, n, g, st.n0))
    _ctx(ctx).call("nngp_cNNGP_multi", len(problems), C.cast(structs, C.c_void_p), p, m, dptr(f64(sigma_sq_IG)),
                   model, precision_code(precision), 0)
    res = []
    for o, n, g, n0 in outs:
        r = {"beta.hat": o["beta.hat"].reshape(g, p).T, "ab": o["ab"].reshape(g, 2).T,
             "bB.inv": o["bB.inv"].reshape(g, p * p).T, "bb": o["bb"].reshape(g, p).T}
        if "y.0.hat" in o:
            r["y.0.hat"] = o["y.0.hat"].reshape(g, n0).T
            r["y.0.hat.var"] = o["y.0.hat.var"].reshape(g, n0).T
        if "crps" in o:
            r["crps"], r["rmspe"] = o["crps"], o["rmspe"]
        res.append(r)
    return res


def rNNGP_batch(chains, precision="fp64", ctx: Context | None = None) -> list:
    """Independent response-model chains advanced together (nngp_rNNGP_batch).  Each chain is a dict
    with the arguments of rNNGP that may differ between chains (y, X, coords, nn_indx, nn_indx_lu, m,
    cov_model, sigma_sq_IG, tau_sq_IG, phi_unif[, nu_unif], beta_starting, theta_starting, tuning,
    n_samples, normals, unifs); all chains share p.  No replicate draws.  Returns one dict per chain with
    p.beta.samples, p.theta.samples and accept -- each identical to what rNNGP gives that chain alone."""
    structs = (MCMCProblem * len(chains))()
    keep, outs = [], []
    p = None
    for k, P in enumerate(chains):
        y = f64(P["y"])
        n = len(y)
        Xa = np.asarray(P["X"], np.float64)
        Xa = Xa[:, None] if Xa.ndim == 1 else Xa
        if p is None:
            p = Xa.shape[1]
        elif Xa.shape[1] != p:
            raise ValueError("all chains of a batch must share p")
        model = cov_model_index(P["cov_model"])
        nTheta = 4 if model == 2 else 3
        nS = int(P["n_samples"])
        arrs = {"y": y, "X": f64(Xa.T.reshape(-1)), "coords": coords_cm(P["coords"]),
                "nnIndx": i32(P["nn_indx"]), "nnIndxLU": i32(P["nn_indx_lu"]),
                "sigmaSqIG": f64(P["sigma_sq_IG"]), "tauSqIG": f64(P["tau_sq_IG"]), "phiUnif": f64(P["phi_unif"]),
                "nuUnif": f64(P.get("nu_unif") if P.get("nu_unif") is not None else [0.0, 0.0]),
                "betaStarting": f64(P["beta_starting"]),
                "thetaStarting": f64(list(np.asarray(P["theta_starting"], np.float64).reshape(-1)[:nTheta])
                                     + [0.0] * (4 - nTheta)),
                "tuning": f64(list(np.asarray(P["tuning"], np.float64).reshape(-1)[:nTheta]) + [0.0] * (4 - nTheta)),
                "normals": f64(P["normals"]), "unifs": f64(P["unifs"]),
                "betaSamples": np.zeros(max(1, p * nS)), "thetaSamples": np.zeros(max(1, nTheta * nS))}
        st = structs[k]
        st.n, st.m, st.covModel, st.nSamples = n, int(P["m"]), model, nS
        for name, a in arrs.items():
            setattr(st, name, a.ctypes.data)
        st.nNormals, st.nUnifs = len(arrs["normals"]), len(arrs["unifs"])
        keep.append(arrs)
        outs.append((arrs, nS, nTheta))
    _ctx(ctx).call("nngp_rNNGP_batch", len(chains), C.cast(structs, C.c_void_p), p, precision_code(precision), 0)
    return [{"p.beta.samples": a["betaSamples"][: p * nS].reshape(nS, p).T,
             "p.theta.samples": a["thetaSamples"][: nT * nS].reshape(nS, nT).T,
             "accept": int(structs[k].nAccept)} for k, (a, nS, nT) in enumerate(outs)]


__all__ = ["mkNNIndxCB", "mkNNIndx", "mkUIndx", "nn2", "updateBF", "updateConjBF", "Q", "loglik_gram",
           "rNNGP", "rNNGP_batch", "cNNGP", "cNNGP_multi", "rNNGPPredict", "rNNGPReplicated", "cov_model_index", "precision_code", "coords_cm", "NNGPError", "Context", "COV_MODELS"]
