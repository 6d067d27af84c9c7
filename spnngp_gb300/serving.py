"""Continuous-batching server for conjugate NNGP fit + predict requests on one GB300.

A request is one spConjNNGP fit at a fixed (phi, alpha) followed by prediction
at its own point set -- the work R/spConjNNGP.R:149-216 and :359-403 do per
call: order the data by the first coordinate, find the m ordered neighbors
(src/nn.cpp:213-258) and the prediction neighbors (RANN::nn2,
R/spConjNNGP.R:158), then src/cNNGP.cpp:73-358 at one parameter set.

The server keeps each dataset's ordered coordinates, covariates and neighbor
index resident in HBM (the neighbor.info reuse of R/spConjNNGP.R:416-420), so a
second request on the same dataset skips the upload and the search.  Requests
are admitted while the bytes they need fit the HBM budget (least recently used
idle datasets are evicted to make room; a request too large for the budget on
its own is rejected).  Every iteration of the serving loop fits and predicts
all admitted requests in one nngp_cNNGP_multi call: one fused likelihood launch
over every request's locations, then the per-request prediction solves.  A
request's result does not depend on what else is in its batch: each request is
a separate job of the fused launch with its own fixed-order reductions.

Latency of a request = completion time - arrival time; ``serve`` replays a
timed arrival stream in real time and reports throughput and latency
percentiles.  ``serve_per_request`` replays the same stream through the plain
per-request form (host entry points, one request at a time) for comparison.
"""
from __future__ import annotations

import collections
import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import ConjProblem, Context, NNGPError, default_context, n_indx
from .core import coords_cm, cov_model_index, mkNNIndxCB, nn2, precision_code, cNNGP


@dataclass
class ConjRequest:
    """One fit + predict request.  coords n x 2 (any order), X n x p, y n, coords0 n0 x 2,
    X0 n0 x p.  Requests naming the same ``dataset`` key share its resident state, so they
    must carry the same coords, X and y."""

    coords: np.ndarray
    X: np.ndarray
    y: np.ndarray
    coords0: np.ndarray
    X0: np.ndarray
    phi: float
    alpha: float
    nu: float = 0.0
    dataset: object = None
    rid: int = 0
    arrival: float = 0.0


@dataclass
class ConjResult:
    rid: int
    beta_hat: np.ndarray = None
    ab: np.ndarray = None
    bB_inv: np.ndarray = None
    bb: np.ndarray = None
    y0_hat: np.ndarray = None
    y0_hat_var: np.ndarray = None
    error: str | None = None
    arrival: float = 0.0
    done: float = 0.0
    batch: int = 0

    @property
    def latency(self) -> float:
        return self.done - self.arrival


@dataclass
class _Dataset:
    n: int
    nbytes: int
    tensors: dict = field(default_factory=dict)
    busy: int = 0


def dataset_bytes(n: int, p: int, m: int) -> int:
    """HBM held by one resident dataset: ordered coords, X, y, nnIndx, nnIndxLU."""
    return 16 * n + 8 * n * p + 8 * n + 4 * max(n_indx(n, m), 0) + 8 * n


def search_bytes(n: int, m: int) -> int:
    """Transient HBM of one neighbor search: nnDist plus the sorted views and sort scratch."""
    return 8 * max(n_indx(n, m), 0) + 96 * n


def request_bytes(n: int, n0: int, p: int, m: int) -> int:
    """HBM one request needs while it is in a batch, besides its dataset: prediction inputs,
    neighbors and outputs, plus the fit's per-location temporaries (split coordinates, the
    [X y] matrix) and the prediction temporaries."""
    return 16 * n0 + 8 * n0 * p + 4 * n0 * m + 8 * n0 * m + 32 * n0 + 32 * n + 8 * n * (p + 1) + 4096


class ConjServer:
    """Serving loop state: queue, resident datasets, HBM accounting."""

    def __init__(self, m: int = 15, cov_model="exponential", sigma_sq_IG=(2.0, 1.0), precision="fp32r",
                 hbm_budget: float = 150e9, max_batch: int = 512, ctx: Context | None = None, cache: bool = True):
        import torch

        self.torch = torch
        self.ctx = ctx or default_context()
        self.dev = torch.device("cuda", self.ctx.device)
        # one stream for the server's torch work (uploads, ordering, output buffers) and the
        # library's kernels, so each sees the other's results in order
        self.stream = torch.cuda.Stream(self.dev)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.m = m
        self.model = cov_model_index(cov_model)
        self.sigma_sq_IG = np.ascontiguousarray(sigma_sq_IG, np.float64)
        self.prec = precision_code(precision)
        self.budget = int(hbm_budget)
        self.max_batch = max_batch
        self.cache = cache
        self.queue = collections.deque()
        self.datasets: "collections.OrderedDict[object, _Dataset]" = collections.OrderedDict()
        self.resident = 0
        self.iterations = 0
        self.stats = {"hits": 0, "misses": 0, "evictions": 0, "rejected": 0}

    # ------------------------------------------------------------- admission
    def submit(self, req: ConjRequest):
        self.queue.append(req)

    def _p(self, req):
        X = np.asarray(req.X)
        return 1 if X.ndim == 1 else X.shape[1]

    def _evict_for(self, need: int, pinned: set) -> bool:
        while self.resident + need > self.budget:
            victim = next((k for k, d in self.datasets.items() if d.busy == 0 and k not in pinned), None)
            if victim is None:
                return False
            d = self.datasets.pop(victim)
            self.resident -= d.nbytes
            d.tensors.clear()
            self.stats["evictions"] += 1
        return True

    def _admit(self):
        batch, pinned = [], set()
        while self.queue and len(batch) < self.max_batch:
            req = self.queue[0]
            n, p, n0 = len(req.y), self._p(req), len(req.coords0)
            key = req.dataset if (self.cache and req.dataset is not None) else ("req", req.rid)
            need_ds = 0 if key in self.datasets or key in pinned else dataset_bytes(n, p, self.m)
            need = need_ds + request_bytes(n, n0, p, self.m)
            peak = need + (search_bytes(n, self.m) if need_ds else 0)
            if dataset_bytes(n, p, self.m) + request_bytes(n, n0, p, self.m) + search_bytes(n, self.m) > self.budget:
                self.queue.popleft()
                self.stats["rejected"] += 1
                batch.append((req, None, "request exceeds the HBM budget"))
                continue
            if not self._evict_for(peak, pinned | {key}):
                break  # wait for the running batch's memory (FIFO: no overtaking)
            self.queue.popleft()
            self.resident += need
            pinned.add(key)
            batch.append((req, key, None))
        return batch

    # ------------------------------------------------------------ preparation
    def _dataset(self, req, key):
        # torch's work and the library's neighbor search must share the server's stream
        self.ctx.set_stream(self.stream.cuda_stream)
        with self.torch.cuda.stream(self.stream):
            return self._dataset_on_stream(req, key)

    def _dataset_on_stream(self, req, key):
        torch = self.torch
        d = self.datasets.get(key)
        if d is not None:
            self.datasets.move_to_end(key)
            self.stats["hits"] += 1
            return d
        self.stats["misses"] += 1
        n, p, m = len(req.y), self._p(req), self.m
        # the reference orders the data by the first coordinate (R/spConjNNGP.R:149-152)
        c = torch.from_numpy(np.ascontiguousarray(req.coords, np.float64)).to(self.dev, non_blocking=True)
        X = torch.from_numpy(np.ascontiguousarray(np.asarray(req.X, np.float64).reshape(n, p))).to(self.dev)
        y = torch.from_numpy(np.ascontiguousarray(req.y, np.float64)).to(self.dev)
        ord_ = torch.argsort(c[:, 0], stable=True)
        ccm = c.index_select(0, ord_).t().contiguous()
        Xcm = X.index_select(0, ord_).t().contiguous()
        ys = y.index_select(0, ord_).contiguous()
        nI = max(n_indx(n, m), 1)
        nn = torch.empty(nI, dtype=torch.int32, device=self.dev)
        dist = torch.empty(nI, dtype=torch.float64, device=self.dev)
        lu = torch.empty(2 * n, dtype=torch.int32, device=self.dev)
        self.ctx.call("nngp_mkNNIndxCB_dev", n, m, ccm.data_ptr(), nn.data_ptr(), dist.data_ptr(), lu.data_ptr())
        del dist
        d = _Dataset(n=n, nbytes=dataset_bytes(n, p, m), tensors={"coords": ccm, "X": Xcm, "y": ys, "nn": nn, "lu": lu})
        self.datasets[key] = d
        return d

    # -------------------------------------------------------------- iteration
    def step(self, now=time.perf_counter) -> list:
        """One serving iteration: admit, prepare, one batched fit + predict, retire."""
        self.ctx.set_stream(self.stream.cuda_stream)  # the context may be shared with other callers
        with self.torch.cuda.stream(self.stream):
            return self._step(now)

    def _step(self, now) -> list:
        torch = self.torch
        batch = self._admit()
        if not batch:
            return []
        self.iterations += 1
        done, live = [], []
        for req, key, err in batch:
            if err is not None:
                done.append(ConjResult(rid=req.rid, error=err, arrival=req.arrival, done=now(),
                                       batch=self.iterations))
                continue
            live.append((req, key))
        if not live:
            return done
        structs = (ConjProblem * len(live))()
        keep, outs = [], []
        for j, (req, key) in enumerate(live):
            d = self._dataset(req, key)
            d.busy += 1
            n, p, n0, m = d.n, self._p(req), len(req.coords0), self.m
            c0 = torch.from_numpy(coords_cm(req.coords0)).to(self.dev)
            X0 = torch.from_numpy(np.ascontiguousarray(np.asarray(req.X0, np.float64).reshape(n0, p).T)
                                  .reshape(-1)).to(self.dev)
            nn0 = torch.empty(max(n0 * m, 1), dtype=torch.int32, device=self.dev)
            if n0:
                self.ctx.call("nngp_nn2_dev", n, d.tensors["coords"].data_ptr(), n0, c0.data_ptr(), m,
                              nn0.data_ptr(), None)
            ta = np.array([req.phi, req.alpha] + ([req.nu] if self.model == 2 else []), np.float64)
            o = {k: torch.empty(s, dtype=torch.float64, device=self.dev)
                 for k, s in (("beta", p), ("ab", 2), ("bBInv", p * p), ("bb", p), ("y0", max(n0, 1)),
                              ("y0v", max(n0, 1)))}
            st = structs[j]
            st.n, st.n0, st.g = n, n0, 1
            st.y, st.X, st.coords = (d.tensors[k].data_ptr() for k in ("y", "X", "coords"))
            st.nnIndx, st.nnIndxLU = d.tensors["nn"].data_ptr(), d.tensors["lu"].data_ptr()
            st.X0, st.coords0, st.nnIndx0 = X0.data_ptr(), c0.data_ptr(), nn0.data_ptr()
            st.thetaAlpha = ta.ctypes.data
            st.betaHat, st.ab, st.bBInv, st.bb = (o[k].data_ptr() for k in ("beta", "ab", "bBInv", "bb"))
            if n0:
                st.y0Hat, st.y0HatVar = o["y0"].data_ptr(), o["y0v"].data_ptr()
            keep.append((c0, X0, nn0, ta))
            outs.append((req, key, o, n, p, n0))
        err = None
        try:
            self.ctx.call("nngp_cNNGP_multi", len(live), C.cast(structs, C.c_void_p), outs[0][4], self.m,
                          self.sigma_sq_IG.ctypes.data_as(C.POINTER(C.c_double)), self.model, self.prec, 1)
        except NNGPError as e:
            err = str(e)
        t = now()
        for req, key, o, n, p, n0 in outs:
            r = ConjResult(rid=req.rid, arrival=req.arrival, batch=self.iterations, error=err)
            if err is None:
                host = {k: v.cpu().numpy() for k, v in o.items()}
                r.beta_hat, r.ab, r.bB_inv, r.bb = host["beta"], host["ab"], host["bBInv"].reshape(p, p).T, host["bb"]
                if n0:
                    r.y0_hat, r.y0_hat_var = host["y0"], host["y0v"]
                t = now()
            r.done = t
            done.append(r)
            d = self.datasets.get(key)
            if d is not None:
                d.busy -= 1
                if not self.cache or (isinstance(key, tuple) and key and key[0] == "req"):
                    self.datasets.pop(key)
                    self.resident -= d.nbytes
            self.resident -= request_bytes(n, n0, p, self.m)
        return done

    def drain(self) -> list:
        out = []
        while self.queue:
            out += self.step()
        return out


def serve(server: ConjServer, requests, realtime: bool = True) -> dict:
    """Replays requests (sorted by ``arrival``, seconds from start) in real time through the server:
    each loop iteration submits every request that has arrived and runs one batched step."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    results, i = [], 0
    while i < len(reqs) or server.queue:
        now = clock()
        while i < len(reqs) and (reqs[i].arrival <= now or not realtime):
            server.submit(reqs[i])
            i += 1
        if not server.queue:
            time.sleep(max(0.0, min(reqs[i].arrival - clock(), 0.05)))
            continue
        results += server.step(now=clock)
    return summarize(results)


def serve_per_request(requests, m: int = 15, cov_model="exponential", sigma_sq_IG=(2.0, 1.0), precision="fp32r",
                      ctx: Context | None = None) -> dict:
    """The plain per-request form on the same arrival stream: one request at a time, in arrival
    order, through the host entry points (order, neighbor search, nn2, cNNGP), as a loop over
    spConjNNGP calls does it."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    results = []
    for req in reqs:
        wait = req.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        results.append(fit_predict_one(req, m, cov_model, sigma_sq_IG, precision, ctx,
                                       clock=lambda: time.perf_counter() - t0))
    return summarize(results)


def fit_predict_one(req: ConjRequest, m: int = 15, cov_model="exponential", sigma_sq_IG=(2.0, 1.0),
                    precision="fp32r", ctx: Context | None = None, clock=time.perf_counter) -> ConjResult:
    """One request through the host entry points alone."""
    n = len(req.y)
    X = np.asarray(req.X, np.float64).reshape(n, -1)
    ord_ = np.argsort(np.asarray(req.coords)[:, 0], kind="stable")
    c, Xs, ys = np.asarray(req.coords)[ord_], X[ord_], np.asarray(req.y)[ord_]
    nb = mkNNIndxCB(c, m, ctx=ctx)
    nn0, _ = nn2(c, req.coords0, m, ctx=ctx)
    model = cov_model_index(cov_model)
    ta = np.array([[req.phi], [req.alpha]] + ([[req.nu]] if model == 2 else []))
    r = ConjResult(rid=req.rid, arrival=req.arrival)
    try:
        out = cNNGP(ys, Xs, c, ta, nb["nnIndx"], nb["nnIndxLU"], req.X0, req.coords0, nn0, m, sigma_sq_IG, model,
                    precision=precision, ctx=ctx)
        r.beta_hat, r.ab, r.bb = out["beta.hat"][:, 0], out["ab"][:, 0], out["bb"][:, 0]
        p = len(r.beta_hat)
        r.bB_inv = out["bB.inv"][:, 0].reshape(p, p).T
        if "y.0.hat" in out:
            r.y0_hat, r.y0_hat_var = out["y.0.hat"][:, 0], out["y.0.hat.var"][:, 0]
    except NNGPError as e:
        r.error = str(e)
    r.done = clock()
    return r


def summarize(results) -> dict:
    ok = [r for r in results if r.error is None]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(0)
    span = (max(r.done for r in results) - min(r.arrival for r in results)) if results else 0.0
    return {"results": results, "completed": len(ok), "failed": len(results) - len(ok),
            "throughput_rps": len(ok) / span if span > 0 else None,
            "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "iterations": len({r.batch for r in results}),
            "mean_batch": len(results) / max(len({r.batch for r in results}), 1) if results else None}


__all__ = ["ConjRequest", "ConjResult", "ConjServer", "serve", "serve_per_request", "fit_predict_one",
           "dataset_bytes", "request_bytes", "search_bytes"]
