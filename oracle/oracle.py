"""TEST ORACLE ONLY: ctypes access to the CPU restatement of the spNNGP hot path
(``_build/libnngp_oracle.so``, built from ``nngp_oracle.c``) and, where it was
built, to the reference package's own sources compiled against the R-API
stand-in (``_ref/libspnngp_ref.so``).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module; the product package never does.

All arrays follow the reference's conventions: column-major FP64 matrices,
0-based int32 indices, ``nnIndxLU = [offsets | counts]`` of length 2n, theta
= (sigma^2, tau^2, phi[, nu]) for the response model and (phi, alpha[, nu])
per column of ``theta_alpha`` for the conjugate model.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libnngp_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libspnngp_ref.so")
RCALL_SO = os.path.join(HERE, "_build", "libspnngp_rcall.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

COV_MODELS = ("exponential", "spherical", "matern", "gaussian")


def build(ref: bool = False, rcall: bool = False) -> None:
    """Compile the restatement (and, with ref=True, the shim build of the reference; with
    rcall=True, this project's .Call layer against the same R-API stand-in)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    if rcall:
        subprocess.run(["make", "-s", "-C", HERE, "rcall"], check=True)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def n_indx(n: int, m: int) -> int:
    return int((1 + m) / 2 * m + (n - m - 1) * m)


def cov_index(name_or_int) -> int:
    return name_or_int if isinstance(name_or_int, int) else COV_MODELS.index(name_or_int)


class _Lib:
    def __init__(self, path):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)


class Oracle(_Lib):
    """The C restatement (nngp_oracle.c)."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build()
        super().__init__(path)
        L = self.lib
        L.or_spcor.restype = C.c_double
        L.or_spcor.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        L.or_bessel_k.restype = C.c_double
        L.or_bessel_k.argtypes = [C.c_double, C.c_double]
        L.or_updateBF.restype = C.c_int
        L.or_Q.restype = C.c_double
        L.or_n_indx.restype = C.c_long
        L.or_stream_set.argtypes = [_dp, C.c_long, _dp, C.c_long]

    # --- streams
    def set_streams(self, normals, unifs):
        self._norm = f64(normals)
        self._unif = f64(unifs)
        self.lib.or_stream_set(_d(self._norm), len(self._norm), _d(self._unif), len(self._unif))

    def stream_used(self):
        a, b, o = C.c_long(), C.c_long(), C.c_int()
        self.lib.or_stream_used(C.byref(a), C.byref(b), C.byref(o))
        return a.value, b.value, bool(o.value)

    # --- scalar helpers
    def spcor(self, d, phi, nu, model):
        return self.lib.or_spcor(float(d), float(phi), float(nu), cov_index(model))

    def bessel_k(self, x, nu):
        return self.lib.or_bessel_k(float(x), float(nu))

    def rsort_with_index(self, x, idx):
        x = f64(x).copy()
        idx = i32(idx).copy()
        self.lib.or_rsort_with_index(_d(x), _i(idx), len(x))
        return x, idx

    # --- neighbor search
    def mkNNIndxCB(self, coords, m, threads=1):
        coords = f64(np.asarray(coords).T.reshape(-1)) if np.asarray(coords).ndim == 2 else f64(coords)
        n = len(coords) // 2
        nI = n_indx(n, m)
        nnIndx = np.zeros(nI, np.int32)
        nnDist = np.zeros(nI, np.float64)
        lu = np.zeros(2 * n, np.int32)
        self.lib.or_mkNNIndxCB(n, m, _d(coords), _i(nnIndx), _d(nnDist), _i(lu), threads)
        return nnIndx, nnDist, lu

    def mkNNIndx(self, coords, m, threads=1):
        coords = f64(np.asarray(coords).T.reshape(-1)) if np.asarray(coords).ndim == 2 else f64(coords)
        n = len(coords) // 2
        nI = n_indx(n, m)
        nnIndx = np.zeros(nI, np.int32)
        nnDist = np.zeros(nI, np.float64)
        lu = np.zeros(2 * n, np.int32)
        self.lib.or_mkNNIndx(n, m, _d(coords), _i(nnIndx), _d(nnDist), _i(lu), threads)
        return nnIndx, nnDist, lu

    def mkUIndx(self, n, m, nnIndx, nnIndxLU, search_type=2):
        nI = n_indx(n, m)
        u = np.zeros(nI, np.int32)
        ulu = np.zeros(2 * n, np.int32)
        ui = np.zeros(nI, np.int32)
        nnIndx, nnIndxLU = i32(nnIndx), i32(nnIndxLU)
        self.lib.or_mkUIndx(n, m, _i(nnIndx), _i(nnIndxLU), _i(u), _i(ulu), _i(ui), search_type)
        return u, ulu, ui

    def nn2(self, coords, coords0, k, threads=1):
        c = f64(np.asarray(coords).T.reshape(-1))
        c0 = f64(np.asarray(coords0).T.reshape(-1))
        n, n0 = len(c) // 2, len(c0) // 2
        idx = np.zeros(n0 * k, np.int32)
        dist = np.zeros(n0 * k, np.float64)
        self.lib.or_nn2(n, _d(c), n0, _d(c0), k, _i(idx), _d(dist), threads)
        return idx.reshape(k, n0).T.copy(), dist.reshape(k, n0).T.copy()

    # --- B/F, Q
    def updateBF(self, coords_cm, nnIndx, nnIndxLU, m, model, sigma_sq, tau_sq, phi, nu=0.0, threads=1):
        coords_cm = f64(coords_cm)
        n = len(coords_cm) // 2
        B = np.zeros(n_indx(n, m), np.float64)
        F = np.zeros(n, np.float64)
        ld = C.c_double()
        nnIndx, nnIndxLU = i32(nnIndx), i32(nnIndxLU)
        st = self.lib.or_updateBF(n, m, _d(coords_cm), _i(nnIndx), _i(nnIndxLU), cov_index(model),
                                  C.c_double(sigma_sq), C.c_double(tau_sq), C.c_double(phi), C.c_double(nu),
                                  _d(B), _d(F), C.byref(ld), threads)
        return B, F, ld.value, st

    def Q(self, B, F, u, v, nnIndx, nnIndxLU, threads=1):
        B, F, u, v = f64(B), f64(F), f64(u), f64(v)
        nnIndx, nnIndxLU = i32(nnIndx), i32(nnIndxLU)
        return self.lib.or_Q(_d(B), _d(F), _d(u), _d(v), len(F), _i(nnIndx), _i(nnIndxLU), threads)

    # --- drivers
    def rNNGP(self, y, X, m, coords_cm, model, nnIndx, nnIndxLU, sigma_sq_IG, tau_sq_IG, phi_unif, nu_unif,
              beta_start, theta_start, tuning, n_samples, normals, unifs, threads=1, n_rep=0, rep_indx=None):
        y, X, coords_cm = f64(y), f64(X), f64(coords_cm)
        n = len(y)
        p = X.size // n
        model = cov_index(model)
        nTheta = 4 if model == 2 else 3
        beta_s = np.zeros(p * n_samples)
        theta_s = np.zeros(nTheta * n_samples)
        rep = np.zeros(max(1, n * n_rep))
        ri = i32(rep_indx if rep_indx is not None else np.zeros(max(1, n_samples), np.int32))
        acc = C.c_int()
        self.set_streams(normals, unifs)
        args = [f64(a) for a in (sigma_sq_IG, tau_sq_IG, phi_unif, nu_unif, beta_start, theta_start, tuning)]
        nnIndx, nnIndxLU = i32(nnIndx), i32(nnIndxLU)
        st = self.lib.or_rNNGP(_d(y), _d(X), p, n, m, _d(coords_cm), model, _i(nnIndx), _i(nnIndxLU),
                               *[_d(a) for a in args], n_samples, threads, n_rep, _i(ri),
                               _d(beta_s), _d(theta_s), _d(rep), C.byref(acc))
        return dict(status=st, beta=beta_s.reshape(n_samples, p).T, theta=theta_s.reshape(n_samples, nTheta).T,
                    rep=rep[: n * n_rep].reshape(n_rep, n).T if n_rep else None, accept=acc.value,
                    used=self.stream_used())

    def cNNGP(self, y, X, coords_cm, theta_alpha, nnIndx, nnIndxLU, X0, coords0_cm, nnIndx0, m, sigma_sq_IG,
              model, threads=1):
        y, X, coords_cm = f64(y), f64(X), f64(coords_cm)
        n = len(y)
        p = X.size // n
        model = cov_index(model)
        ta = f64(theta_alpha)
        nTheta = 3 if model == 2 else 2
        g = ta.size // nTheta
        X0 = f64(X0) if X0 is not None else np.zeros(1)
        c0 = f64(coords0_cm) if coords0_cm is not None else np.zeros(2)
        n0 = X0.size // p if coords0_cm is not None else 0
        nn0 = i32(nnIndx0) if nnIndx0 is not None else np.zeros(1, np.int32)
        out = dict(beta=np.zeros(p * g), ab=np.zeros(2 * g), bBInv=np.zeros(p * p * g), bb=np.zeros(p * g),
                   y0=np.zeros(max(1, n0 * g)), y0var=np.zeros(max(1, n0 * g)))
        nnIndx, nnIndxLU = i32(nnIndx), i32(nnIndxLU)
        st = self.lib.or_cNNGP(_d(y), _d(X), p, n, _d(coords_cm), _d(ta), _i(nnIndx), _i(nnIndxLU), _d(X0), _d(c0),
                               n0, _i(nn0), g, m, _d(f64(sigma_sq_IG)), model, threads,
                               *[_d(out[k]) for k in ("beta", "ab", "bBInv", "bb", "y0", "y0var")])
        out["status"] = st
        out["beta"] = out["beta"].reshape(g, p).T
        out["ab"] = out["ab"].reshape(g, 2).T
        out["bBInv"] = out["bBInv"].reshape(g, p * p).T
        out["bb"] = out["bb"].reshape(g, p).T
        out["y0"] = out["y0"][: n0 * g].reshape(g, n0).T
        out["y0var"] = out["y0var"][: n0 * g].reshape(g, n0).T
        return out

    def rNNGPPredict(self, X, y, coords_cm, m, X0, coords0_cm, nnIndx0, beta, theta, model, z, threads=1):
        X, y, coords_cm, X0, coords0_cm = f64(X), f64(y), f64(coords_cm), f64(X0), f64(coords0_cm)
        n = len(y)
        p = X.size // n
        q = X0.size // p
        beta = f64(beta)
        nS = beta.size // p
        y0 = np.zeros(q * nS)
        st = self.lib.or_rNNGPPredict(_d(X), _d(y), _d(coords_cm), n, p, m, _d(X0), _d(coords0_cm), q,
                                      _i(i32(nnIndx0)), _d(beta), _d(f64(theta)), nS, cov_index(model),
                                      _d(f64(z)), threads, _d(y0))
        return y0.reshape(nS, q).T, st

    def rNNGPReplicated(self, X, m, coords_cm, model, nnIndx, nnIndxLU, beta_sp, theta, normals, threads=1):
        X, coords_cm = f64(X), f64(coords_cm)
        n = len(coords_cm) // 2
        p = X.size // n
        beta_sp = np.asarray(beta_sp, np.float64)
        nS = beta_sp.shape[0]
        yr = np.zeros(n * nS)
        self.set_streams(normals, np.zeros(1))
        st = self.lib.or_rNNGPReplicated(_d(X), p, n, m, _d(coords_cm), cov_index(model), _i(i32(nnIndx)),
                                         _i(i32(nnIndxLU)), _d(f64(beta_sp.T.reshape(-1))), _d(f64(theta)), nS,
                                         threads, _d(yr))
        return yr.reshape(nS, n).T, st


class Reference(_Lib):
    """The reference's own src/*.cpp compiled against the R-API stand-in (oracle/_ref).  With
    path=RCALL_SO the same drivers call this project's .Call layer (src/) instead: every method
    below except spcor, updateBF, updateConjBF and Q then runs through the SEXP routines of
    src/nngp_call.cpp."""

    def __init__(self, path=REF_SO):
        super().__init__(path)
        L = self.lib
        L.ref_last_error.restype = C.c_char_p
        L.ref_stream_set.argtypes = [_dp, C.c_long, _dp, C.c_long]
        if hasattr(L, "ref_spCor"):  # absent from the .Call-layer build
            L.ref_spCor.restype = C.c_double
            L.ref_spCor.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
            L.ref_Q.restype = C.c_double
            L.ref_updateBF.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _dp, C.c_int, C.c_double, C.c_int, _dp,
                                       _dp, _dp]
            L.ref_updateConjBF.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, C.c_double, C.c_double, C.c_double,
                                           C.c_int, C.c_int, _dp, _dp]

    def error(self):
        return self.lib.ref_last_error().decode()

    def set_streams(self, normals, unifs):
        self._norm = f64(normals)
        self._unif = f64(unifs)
        self.lib.ref_stream_set(_d(self._norm), len(self._norm), _d(self._unif), len(self._unif))

    def stream_used(self):
        a, b, o = C.c_long(), C.c_long(), C.c_int()
        self.lib.ref_stream_used(C.byref(a), C.byref(b), C.byref(o))
        return a.value, b.value, bool(o.value)

    def spcor(self, d, phi, nu, model):
        return self.lib.ref_spCor(float(d), float(phi), float(nu), cov_index(model))

    def mkNNIndxCB(self, coords_cm, m, threads=1):
        coords_cm = f64(coords_cm)
        n = len(coords_cm) // 2
        nI = n_indx(n, m)
        # one guard slot in front: the reference reads nnDist[-1] for the location whose list is empty
        nnIndx = np.zeros(nI + 1, np.int32)
        nnDist = np.zeros(nI + 1, np.float64)
        lu = np.zeros(2 * n, np.int32)
        st = self.lib.ref_mkNNIndxCB(n, m, _d(coords_cm), _i(nnIndx[1:]), _d(nnDist[1:]), _i(lu), threads)
        return nnIndx[1:].copy(), nnDist[1:].copy(), lu, st

    def mkNNIndx(self, coords_cm, m, threads=1):
        coords_cm = f64(coords_cm)
        n = len(coords_cm) // 2
        nI = n_indx(n, m)
        nnIndx = np.zeros(nI, np.int32)
        nnDist = np.zeros(nI, np.float64)
        lu = np.zeros(2 * n, np.int32)
        st = self.lib.ref_mkNNIndx(n, m, _d(coords_cm), _i(nnIndx), _d(nnDist), _i(lu), threads)
        return nnIndx, nnDist, lu, st

    def mkUIndx(self, n, m, nnIndx, nnIndxLU, search_type=2):
        nI = n_indx(n, m)
        u = np.zeros(nI, np.int32)
        ulu = np.zeros(2 * n, np.int32)
        ui = np.zeros(nI, np.int32)
        st = self.lib.ref_mkUIndx(n, m, _i(i32(nnIndx)), _i(u), _i(ulu), _i(ui), _i(i32(nnIndxLU)), search_type)
        return u, ulu, ui, st

    def updateBF(self, coords_cm, nnIndx, nnIndxLU, m, model, theta, nu_unif_b=0.0, threads=1):
        coords_cm = f64(coords_cm)
        n = len(coords_cm) // 2
        B = np.zeros(n_indx(n, m))
        F = np.zeros(n)
        ld = np.zeros(1)
        st = self.lib.ref_updateBF(n, m, _d(coords_cm), _i(i32(nnIndx)), _i(i32(nnIndxLU)), _d(f64(theta)),
                                   cov_index(model), nu_unif_b, threads, _d(B), _d(F), _d(ld))
        return B, F, ld[0], st

    def Q(self, B, F, u, v, nnIndx, nnIndxLU):
        return self.lib.ref_Q(_d(f64(B)), _d(f64(F)), _d(f64(u)), _d(f64(v)), len(F), _i(i32(nnIndx)),
                              _i(i32(nnIndxLU)))

    def rNNGP(self, y, X, m, coords_cm, model, nnIndx, nnIndxLU, sigma_sq_IG, tau_sq_IG, phi_unif, nu_unif,
              beta_start, theta_start, tuning, n_samples, normals, unifs, threads=1, n_rep=0, rep_indx=None):
        y, X, coords_cm = f64(y), f64(X), f64(coords_cm)
        n = len(y)
        p = X.size // n
        model = cov_index(model)
        nTheta = 4 if model == 2 else 3
        th = list(theta_start) + [0.0] * (4 - len(theta_start))
        tu = list(tuning) + [0.0] * (4 - len(tuning))
        beta_s = np.zeros(p * n_samples)
        theta_s = np.zeros(nTheta * n_samples)
        rep = np.zeros(max(1, n * n_rep))
        ri = i32(rep_indx if rep_indx is not None else np.zeros(max(1, n_samples), np.int32))
        self.set_streams(normals, unifs)
        L = self.lib
        st = L.ref_rNNGP(_d(y), _d(X), p, n, m, _d(coords_cm), model, _i(i32(nnIndx)), _i(i32(nnIndxLU)),
                         _d(f64(sigma_sq_IG)), _d(f64(tau_sq_IG)), _d(f64(phi_unif)), _d(f64(nu_unif)),
                         _d(f64(beta_start)), C.c_double(th[0]), C.c_double(th[1]), C.c_double(th[2]),
                         C.c_double(th[3]), C.c_double(tu[0]), C.c_double(tu[1]), C.c_double(tu[2]),
                         C.c_double(tu[3]), n_samples, threads, n_rep, _i(ri), _d(beta_s), _d(theta_s), _d(rep))
        return dict(status=st, beta=beta_s.reshape(n_samples, p).T, theta=theta_s.reshape(n_samples, nTheta).T,
                    rep=rep[: n * n_rep].reshape(n_rep, n).T if n_rep else None, used=self.stream_used())

    def cNNGP(self, y, X, coords_cm, theta_alpha, nnIndx, nnIndxLU, X0, coords0_cm, nnIndx0, m, sigma_sq_IG,
              model, threads=1):
        y, X, coords_cm = f64(y), f64(X), f64(coords_cm)
        n = len(y)
        p = X.size // n
        model = cov_index(model)
        ta = f64(theta_alpha)
        nTheta = 3 if model == 2 else 2
        g = ta.size // nTheta
        X0 = f64(X0) if X0 is not None else np.zeros(1)
        c0 = f64(coords0_cm) if coords0_cm is not None else np.zeros(2)
        n0 = X0.size // p if coords0_cm is not None else 0
        nn0 = i32(nnIndx0) if nnIndx0 is not None else np.zeros(1, np.int32)
        out = dict(beta=np.zeros(p * g), ab=np.zeros(2 * g), bBInv=np.zeros(p * p * g), bb=np.zeros(p * g),
                   y0=np.zeros(max(1, n0 * g)), y0var=np.zeros(max(1, n0 * g)))
        st = self.lib.ref_cNNGP(_d(y), _d(X), p, n, _d(coords_cm), _d(ta), _i(i32(nnIndx)), _i(i32(nnIndxLU)),
                                _d(X0), _d(c0), n0, _i(nn0), g, m, _d(f64(sigma_sq_IG)), model, threads,
                                *[_d(out[k]) for k in ("beta", "ab", "bBInv", "bb", "y0", "y0var")])
        out["status"] = st
        out["beta"] = out["beta"].reshape(g, p).T
        out["ab"] = out["ab"].reshape(g, 2).T
        out["bBInv"] = out["bBInv"].reshape(g, p * p).T
        out["bb"] = out["bb"].reshape(g, p).T
        out["y0"] = out["y0"][: n0 * g].reshape(g, n0).T
        out["y0var"] = out["y0var"][: n0 * g].reshape(g, n0).T
        return out

    def rNNGPPredict(self, X, y, coords_cm, m, X0, coords0_cm, nnIndx0, beta, theta, model, z):
        """Runs with one thread (the reference's z pairing races with more)."""
        X, y, coords_cm, X0, coords0_cm = f64(X), f64(y), f64(coords_cm), f64(X0), f64(coords0_cm)
        n = len(y)
        p = X.size // n
        q = X0.size // p
        beta = f64(beta)
        nS = beta.size // p
        y0 = np.zeros(q * nS)
        self.set_streams(z, np.zeros(1))
        st = self.lib.ref_rNNGPPredict(_d(X), _d(y), _d(coords_cm), n, p, m, _d(X0), _d(coords0_cm), q,
                                       _i(i32(nnIndx0)), _d(beta), _d(f64(theta)), nS, cov_index(model), 1,
                                       _d(y0))
        return y0.reshape(nS, q).T, st

    def rNNGPReplicated(self, X, m, coords_cm, model, nnIndx, nnIndxLU, beta_sp, theta, normals, threads=1):
        X, coords_cm = f64(X), f64(coords_cm)
        n = len(coords_cm) // 2
        p = X.size // n
        beta_sp = np.asarray(beta_sp, np.float64)
        nS = beta_sp.shape[0]
        yr = np.zeros(n * nS)
        self.set_streams(normals, np.zeros(1))
        st = self.lib.ref_rNNGPReplicated(_d(X), p, n, m, _d(coords_cm), cov_index(model), _i(i32(nnIndx)),
                                          _i(i32(nnIndxLU)), _d(f64(beta_sp.T.reshape(-1))), _d(f64(theta)), nS,
                                          threads, _d(yr))
        return yr.reshape(nS, n).T, st
