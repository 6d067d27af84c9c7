"""Low-level entry points, one per native routine of spNNGP's hot path.

Each function mirrors the R-level wrapper that calls the reference routine
(names and argument meaning as in R/nn.R and the .Call sites), returns numpy
arrays, and runs on the GB300 through the C ABI.  Coordinates may be given as an
n x 2 array (one row per location, the R ``coords`` matrix) or as the
column-major flat vector the .Call layer receives.
"""
from __future__ import annotations

import time

import numpy as np

from ._lib import FP32R, FP64, Context, NNGPError, default_context, dptr, f64, i32, iptr, n_indx

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


__all__ = ["mkNNIndxCB", "mkNNIndx", "mkUIndx", "nn2", "updateBF", "updateConjBF", "Q", "loglik_gram",
           "cov_model_index", "precision_code", "coords_cm", "NNGPError", "Context", "COV_MODELS"]
