"""Benchmark of the NNGP B/F neighborhood-solve pass on one GB300.

Headline metric: B/F neighborhood solves/s at n = 1e6, m = 15.  One step is
one fused likelihood pass (updateBF + log-likelihood: sum log F_i and the Gram
of [X y], so Q(X beta - y) for any beta) over all n locations at a fixed
theta, in the FP32 + FP64-refinement form.  Workload: n = 1e6 locations
uniform on the unit square in the reference's x-ordering, m = 15 code-book
neighbors, exponential covariance with sigma^2 = 1, tau^2 = 0.1, phi = 59.91
(effective range 0.05), X = [1, N(0,1)], synthetic y.

Reported beside it: the plain FP64 form's throughput and the log-likelihood
error of the FP32R form against it, the e2e throughput through the C ABI with
host buffers (copies inside the timed region), the dominant kernel's roofline
fraction against the measured FP32 pipe peak (and its HBM bytes against the
measured copy bandwidth), the autotuned launch shape, and the CPU baseline (the
oracle's C port of the reference loop, OpenMP on all host cores).  Sections
(--sections): accuracy (FP32R vs FP64 at n = 1e6 for m = 15 and 32, three
models at two ranges), mcmc (the batched multi-instance chains), conj (the
spConjNNGP k-fold grid sweep) and serve (the request loop's p50/p99).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

Under torchrun (N > 1) every rank runs the same workload on its own GPU
(replicas: the pass does not exchange data) and value is the sum of solves
over all ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N = 1_000_000
M = 15
THETA = (1.0, 0.1, 59.91)  # sigma^2, tau^2, phi (effective range 0.05)
COV = "exponential"
METRIC = "B/F neighborhood solves/s at n=1e6 m=15 (FP32+FP64-refine fused updateBF+loglik)"
UNIT = "solves/s"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def workload(n=N, seed=2024):
    rng = np.random.default_rng(seed)
    c = rng.uniform(size=(n, 2))
    c = c[np.argsort(c[:, 0], kind="stable")]
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = X @ np.array([1.0, -0.5]) + rng.normal(size=n)
    return c, X, y


def algorithmic_flops(m):
    """Per-solve flop counts of the minimal algorithm: covariance build (8 per entry), Cholesky,
    two triangular solves and F (the FP64 form), plus the refinement of the FP32R form (the
    residual c - C b and the two correction solves)."""
    P = m * (m + 1) / 2
    base = 8 * P + m ** 3 / 3 + m ** 2 / 2 + m / 6 + 2 * m ** 2 + 2 * m
    refine = 2 * m ** 2 + m + 2 * m ** 2
    return base, base + refine


def algorithmic_bytes(m, nv):
    """Compulsory HBM bytes per solve of the fused pass: the neighbor list (4m), the location's
    split coordinates (16) and its row of V as float pairs (8 nv); neighbor coordinates and V
    rows are L2-resident gathers."""
    return 4 * m + 16 + 8 * nv


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:  # sampling must cover the timed region
                time.sleep(0.05)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x: float, device=None) -> float:
    """The largest x over the ranks of the job (x itself for a single process): every rank
    reports the slowest rank's time."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, max_ms: float, world_size: int) -> float:
    """Units per second of the whole job: every rank processes units_per_rank (replicas) and
    the job takes the slowest rank's time."""
    return world_size * units_per_rank / (max_ms * 1e-3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def bench_config():
    """The workload both arms run (the same string on both lines)."""
    return {"workload": f"n={N} uniform [0,1]^2 x-ordered (seed 2024), m={M} code-book neighbors, {COV} "
                        f"sigma2={THETA[0]} tau2={THETA[1]} phi={THETA[2]}, X=[1,N(0,1)], one fused "
                        f"updateBF + log-likelihood pass per step",
            "l2": "GPU arm: flushed between timed steps (512 MB write), inputs ~100 MB; CPU arm: host memory"}


def cpu_step_oracle(orc, ccm, nn, lu, Xcm, y, threads, n, keep=False):
    """One reference-path step on the host: updateBF (potrf/potri/symv per location) plus the
    log-likelihood quadratic form Q(X beta - y), as src/rNNGP.cpp:306-317 computes them.  orc is
    the oracle port or the reference's own build (oracle.Reference); keep=True also returns B
    and F."""
    from oracle.oracle import Reference

    if isinstance(orc, Reference):
        B, F, ld, st = orc.updateBF(ccm, nn, lu, M, 0, np.array(THETA), threads=threads)
        r = Xcm[:n] * 1.0 + Xcm[n:] * -0.5 - y
        q = orc.Q(B, F, r, r, nn, lu)
    else:
        B, F, ld, st = orc.updateBF(ccm, nn, lu, M, 0, *THETA, 0.0, threads=threads)
        r = Xcm[:n] * 1.0 + Xcm[n:] * -0.5 - y
        q = orc.Q(B, F, r, r, nn, lu, threads=threads)
    ll = -0.5 * (ld + q)
    return (ll, B, F) if keep else ll


def cpu_reference_impl():
    """The CPU implementation the reference arm and cpu_baseline time: the reference's own
    src/*.cpp compiled through the R-API stand-in (oracle/_ref) where that build exists -- it
    is compiled from the spNNGP sources, which only the build host has -- else the oracle's C
    port of the same routines (bit-identical results to the reference build at this workload;
    the same speed on the build host)."""
    from oracle.oracle import Oracle, Reference, build

    build()
    try:
        return Reference(), "reference", "the reference's own src/rNNGP.cpp updateBF and src/util.cpp Q " \
                                         "(compiled unmodified against an R-API stand-in)"
    except Exception as e:
        why = f"reference build not present on this host ({type(e).__name__})"
        return Oracle(), "port", f"the oracle's C port of src/rNNGP.cpp:46-101 and src/util.cpp:261-280; {why}"


def nngp_draw(sp, ctx, c, nn, lu, m, model, theta, rng):
    """One draw of w ~ NNGP(0, sigma^2 R(phi[, nu])) on the given neighbor sets: B and F from
    the library's FP64 updateBF (tau^2 = 0, a 1e-6 nugget for the gaussian model), then the
    sparse unit lower-triangular solve (I - B) w = F^(1/2) z."""
    import scipy.sparse as sps
    from scipy.sparse.linalg import spsolve_triangular

    n = len(c)
    tau = 1e-6 if model == 3 else 0.0
    B, F, _ = sp.updateBF(c, nn, lu, m, model, [theta[0], tau, theta[2]] + list(theta[3:]), ctx=ctx)
    rows = np.repeat(np.arange(n), lu[n:])
    L = sps.csr_matrix((-B, (rows, nn)), shape=(n, n)) + sps.identity(n, format="csr")
    return spsolve_triangular(L.tocsr(), np.sqrt(F) * rng.normal(size=n), lower=True, unit_diagonal=True)


def section_mcmc_batch(sp, ctx, dev, iters, n_inst=256, seed=77):
    """Uneven multi-instance rNNGP: n_inst independent datasets, n log-uniform in [500, 50000],
    m cycling 10/15/20, cov.model cycling exponential/spherical/gaussian/matern (nu 0.5/1.5/2.5,
    held fixed: tuning 0 on nu), priors sigma.sq IG(2,1), tau.sq IG(2,0.1), phi Unif(3,30).
    One step = one Metropolis-within-Gibbs iteration of every chain."""
    import ctypes as C

    import torch
    from spnngp_gb300._lib import MCMCProblem

    rng = np.random.default_rng(seed)
    models = ["exponential", "spherical", "gaussian", "matern"]
    probs = (MCMCProblem * n_inst)()
    keep, total_n, ns = [], 0, []
    t0 = time.perf_counter()
    for k in range(n_inst):
        n = int(np.exp(rng.uniform(np.log(500), np.log(50000))))
        m = (10, 15, 20)[k % 3]
        model = k % 4
        nu = (0.5, 1.5, 2.5)[(k // 4) % 3]
        c = rng.uniform(size=(n, 2))
        c = c[np.argsort(c[:, 0], kind="stable")]
        X = np.column_stack([np.ones(n), rng.normal(size=n)])
        nb = sp.mkNNIndxCB(c, m, ctx=ctx)
        nn, lu = nb["nnIndx"], nb["nnIndxLU"]
        theta = [1.0, 0.1, 6.0] + ([nu] if model == 2 else [])
        w = nngp_draw(sp, ctx, c, nn, lu, m, model, theta, rng)
        y = X @ np.array([1.0, -0.5]) + w + rng.normal(scale=np.sqrt(0.1), size=n)
        nT = 4 if model == 2 else 3
        tun = [0.1, 0.1, 0.5, 0.0][:nT]
        nNorm = iters * (2 + 3) + 8
        dev_arrays = {
            "y": torch.from_numpy(y).to(dev), "X": torch.from_numpy(np.ascontiguousarray(X.T).reshape(-1)).to(dev),
            "coords": torch.from_numpy(np.ascontiguousarray(c.T).reshape(-1)).to(dev),
            "nnIndx": torch.from_numpy(nn).to(dev), "nnIndxLU": torch.from_numpy(lu).to(dev),
            "normals": torch.from_numpy(rng.normal(size=nNorm)).to(dev),
            "unifs": torch.from_numpy(rng.uniform(size=iters + 1)).to(dev),
            "betaSamples": torch.zeros(2 * iters, dtype=torch.float64, device=dev),
            "thetaSamples": torch.zeros(nT * iters, dtype=torch.float64, device=dev)}
        host_arrays = {"sigmaSqIG": np.array([2.0, 1.0]), "tauSqIG": np.array([2.0, 0.1]),
                       "phiUnif": np.array([3.0, 30.0]), "nuUnif": np.array([0.1, 3.0]),
                       "betaStarting": np.array([1.0, -0.5]),
                       "thetaStarting": np.array(theta + [0.0] * (4 - nT)),
                       "tuning": np.array(tun + [0.0] * (4 - nT))}
        P = probs[k]
        P.n, P.m, P.covModel, P.nSamples = n, m, model, iters
        for name, t in dev_arrays.items():
            setattr(P, name, t.data_ptr())
        for name, a in host_arrays.items():
            setattr(P, name, a.ctypes.data)
        P.nNormals, P.nUnifs = nNorm, iters + 1
        keep.append((dev_arrays, host_arrays, (c, X, y, nn, lu)))
        total_n += n
        ns.append(n)
    gen_s = time.perf_counter() - t0

    def run(resident, n_iter):
        for P in probs:
            P.nSamples = n_iter
        ctx.call("nngp_rNNGP_batch", n_inst, C.cast(probs, C.c_void_p), 2, 1, resident)

    run(1, 3)  # warm-up: kernels loaded, tuning, allocator pool
    torch.cuda.synchronize()
    # a short call: its time is the one-off cost of a call (plans, graph capture, first passes)
    # plus its few iterations, which the long call's per-iteration time separates out
    short = 10
    t0 = time.perf_counter()
    run(1, short)
    dt_short = time.perf_counter() - t0
    e2e_iters = min(iters, 200)
    run(1, e2e_iters)
    acc_e2e = [P.nAccept for P in probs]
    ctx.reset_launches()
    t0 = time.perf_counter()
    run(1, iters)
    dt = time.perf_counter() - t0
    launches = ctx.launches
    acc = [P.nAccept for P in probs]
    per_iter = (dt - dt_short) / max(iters - short, 1)
    setup = max(dt_short - short * per_iter, 0.0)
    # the same chains through the host-memory form of the call (uploads and sample readback inside)
    hprobs = (MCMCProblem * n_inst)()
    hkeep = []
    for k in range(n_inst):
        dev_arrays, host_arrays, (c, X, y, nn, lu) = keep[k]
        src = probs[k]
        H = hprobs[k]
        C.memmove(C.addressof(H), C.addressof(src), C.sizeof(MCMCProblem))
        nT = 4 if src.covModel == 2 else 3
        H.nSamples = e2e_iters
        ha = {"y": y, "X": np.ascontiguousarray(X.T).reshape(-1), "coords": np.ascontiguousarray(c.T).reshape(-1),
              "nnIndx": nn, "nnIndxLU": lu, "normals": dev_arrays["normals"].cpu().numpy(),
              "unifs": dev_arrays["unifs"].cpu().numpy(), "betaSamples": np.zeros(2 * e2e_iters),
              "thetaSamples": np.zeros(nT * e2e_iters)}
        for name, a in ha.items():
            setattr(H, name, a.ctypes.data)
        hkeep.append(ha)
    h2d = sum(a.nbytes for ha in hkeep for nm, a in ha.items() if nm not in ("betaSamples", "thetaSamples"))
    d2h = sum(ha["betaSamples"].nbytes + ha["thetaSamples"].nbytes for ha in hkeep)
    t0 = time.perf_counter()
    ctx.call("nngp_rNNGP_batch", n_inst, C.cast(hprobs, C.c_void_p), 2, 1, 0)
    e2e_dt = time.perf_counter() - t0
    same = all(hprobs[k].nAccept == acc_e2e[k] for k in range(n_inst))
    return {
        "workload": f"{n_inst} independent response-model chains, n log-uniform [500, 50000] (total {total_n}), "
                    "m cycling 10/15/20, cov.model cycling exponential/spherical/gaussian/matern(nu 0.5/1.5/2.5 "
                    "fixed), y = X beta + w + eps with w an NNGP draw, FP32R",
        "iterations": iters, "seconds": dt, "iterations_per_s": iters / dt, "ms_per_iteration": dt * 1e3 / iters,
        "solves_per_s": total_n * iters / dt,
        "replay_ms_per_iteration": per_iter * 1e3, "replay_solves_per_s": total_n / per_iter,
        "call_setup_s": setup,
        "gpu_launches": int(launches), "launches_per_iteration": launches / iters,
        "mean_accept_rate": float(np.mean(acc)) / iters,
        "e2e": {"iterations": e2e_iters, "seconds": e2e_dt, "iterations_per_s": e2e_iters / e2e_dt,
                "h2d_bytes": int(h2d), "d2h_bytes": int(d2h), "same_accept_counts_as_resident": same},
        "data_generation_s": gen_s,
        "note": "seconds: one call running every chain for all iterations (plans, graph capture and the "
                "per-iteration graph replays); replay_ms_per_iteration and call_setup_s split it using a "
                f"{short}-iteration call",
    }


def section_parity(sp, ctx, c, nbr, ll_cpu, B_cpu, F_cpu, ll64, ll32, threads, kind):
    """Parity at the headline workload itself (n = 1e6, m = 15) against the CPU implementation:
    the oracle's code-book neighbor search compared bit for bit with the GPU's lists and
    distances, the CPU log-likelihood against the GPU's FP64 and FP32R fused passes, and the
    CPU B and F against the GPU's FP64 and FP32R updateBF (host-pointer entry point)."""
    from oracle.oracle import Oracle

    ccm = np.ascontiguousarray(c.T).reshape(-1)
    t0 = time.perf_counter()
    nn_o, d_o, lu_o = Oracle().mkNNIndxCB(ccm, M, threads=threads)
    knn_cpu_s = time.perf_counter() - t0
    out = {"n": N, "m": M, "checked_against": kind,
           "nn_bitexact": bool(np.array_equal(nn_o, nbr["nnIndx"]) and np.array_equal(lu_o, nbr["nnIndxLU"])),
           "nn_dist_bitexact": bool(np.array_equal(d_o, nbr["nnDist"])),
           "oracle_knn_seconds": knn_cpu_s,
           "loglik_cpu": ll_cpu,
           "fp64_loglik_rel_err_vs_cpu": abs(ll64 - ll_cpu) / abs(ll_cpu),
           "fp32r_loglik_rel_err_vs_cpu": abs(ll32 - ll_cpu) / abs(ll_cpu)}
    scale = max(1.0, float(np.max(np.abs(B_cpu))))
    for prec in ("fp64", "fp32r"):
        B, F, _ = sp.updateBF(c, nbr["nnIndx"], nbr["nnIndxLU"], M, COV, THETA, prec, ctx=ctx)
        out[f"{prec}_B_max_err_rel_max_abs_vs_cpu"] = float(np.max(np.abs(B - B_cpu)) / scale)
        out[f"{prec}_F_max_rel_err_vs_cpu"] = float(np.max(np.abs(F - F_cpu) / F_cpu))
        del B, F
    out["fp64_within_1e-10"] = bool(out["fp64_loglik_rel_err_vs_cpu"] <= 1e-10 and
                                    out["fp64_B_max_err_rel_max_abs_vs_cpu"] <= 1e-10 and
                                    out["fp64_F_max_rel_err_vs_cpu"] <= 1e-10)
    out["fp32r_within_1e-6"] = bool(out["fp32r_loglik_rel_err_vs_cpu"] <= 1e-6 and
                                    out["fp32r_B_max_err_rel_max_abs_vs_cpu"] <= 1e-6 and
                                    out["fp32r_F_max_rel_err_vs_cpu"] <= 1e-6)
    return out


# Config-1 models at effective ranges 0.05 and 0.5 (the distance where the correlation falls to
# 0.05): exponential phi = 2.9957 / range, Matern nu = 1.5 phi = 4.7439 / range, gaussian
# phi = 1.7308 / range with a 1e-6 nugget (the ill-conditioned case).
ACCURACY_CASES = [("exponential", 0.05, (1.0, 0.1, 59.91)), ("exponential", 0.5, (1.0, 0.1, 5.991)),
                  ("matern", 0.05, (1.0, 0.1, 94.88, 1.5)), ("matern", 0.5, (1.0, 0.1, 9.488, 1.5)),
                  ("gaussian", 0.05, (1.0, 1e-6, 34.62)), ("gaussian", 0.5, (1.0, 1e-6, 3.462))]


def section_accuracy(sp, ctx, dev, n=N, ms=(15, 20, 32), seed=2024, reps=3):
    """Plain method at scale, FP64 vs FP32 + refinement: n = 1e6 uniform locations, the code-book
    neighbor search, then one updateBF and one fused log-likelihood at fixed theta for each
    model and range; errors of the FP32R form against the FP64 form (itself pinned to the oracle
    to 1e-10 by the tests), the time of the whole fused pass (device-resident inputs; FP32R:
    primary kernel, the double-float and FP64 re-solves of the flagged locations, the sums)
    after one untimed call (which also tunes a new kernel class), and how many locations the
    FP32R pass re-solved in each tier.  m = 15 runs the register kernel, 20 and 32 the
    warp-per-location kernel (bounds 24 and 32)."""
    import torch

    from spnngp_gb300._lib import _dp

    c, X, y = workload(n, seed)
    V = np.column_stack([X, y])
    nv = V.shape[1]
    beta = np.array([1.0, -0.5])
    rows = []
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_c, d_V = t(np.ascontiguousarray(c.T).reshape(-1)), t(np.ascontiguousarray(V.T).reshape(-1))
    d_ld = torch.zeros(1, dtype=torch.float64, device=dev)
    d_G = torch.zeros(nv * nv, dtype=torch.float64, device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def ll_of(ld, G):
        return -0.5 * (ld + beta @ G[:2, :2] @ beta - 2 * beta @ G[:2, 2] + G[2, 2])

    for m in ms:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nb = sp.mkNNIndxCB(c, m, ctx=ctx)
        knn_s = time.perf_counter() - t0
        nn, lu = nb["nnIndx"], nb["nnIndxLU"]
        d_nn, d_lu = t(nn), t(lu)
        for model, rng_eff, theta in ACCURACY_CASES:
            res = {}
            th = np.array(list(theta) + [0.0] * (4 - len(theta)))
            code = sp.cov_model_index(model)
            for prec, pc in (("fp64", 0), ("fp32r", 1)):
                def run():
                    ctx.call("nngp_loglik_gram_dev", n, m, nv, d_c.data_ptr(), d_nn.data_ptr(), d_lu.data_ptr(),
                             d_V.data_ptr(), code, th.ctypes.data_as(_dp), pc, d_ld.data_ptr(), d_G.data_ptr())
                run()  # untimed: plan, tuning
                torch.cuda.synchronize()
                ctx.call("nngp_set_kernel_timing", 1)
                ctx.call("nngp_kernel_time", None, None)
                ev0.record()
                for _ in range(reps):
                    run()
                ev1.record()
                torch.cuda.synchronize()
                kms = C.c_double()
                ctx.call("nngp_kernel_time", C.byref(kms), None)
                ctx.call("nngp_set_kernel_timing", 0)
                resolved = ctx.fp32r_resolved()[0] if pc else 0
                tiers = ctx.fp32r_tiers() if pc else (0, 0)
                ll = ll_of(d_ld.item(), d_G.cpu().numpy().reshape(nv, nv))
                B, F, _ = sp.updateBF(c, nn, lu, m, model, theta, prec, ctx=ctx)
                res[prec] = (ll, B, F, ev0.elapsed_time(ev1) / reps, kms.value / reps, resolved, tiers)
            ll64, B64, F64, p64, _, _, _ = res["fp64"]
            ll32, B32, F32, p32, k32, nres, ntiers = res["fp32r"]
            rows.append({"m": m, "model": model, "range": rng_eff, "theta": list(theta),
                         "loglik_rel_err": abs(ll32 - ll64) / abs(ll64),
                         "F_max_rel_err": float(np.max(np.abs(F32 - F64) / F64)),
                         "B_max_err_rel_max_abs": float(np.max(np.abs(B32 - B64)) / max(1.0, np.max(np.abs(B64)))),
                         "pass_ms_fp64": p64, "pass_ms_fp32r": p32, "fp32r_speedup": p64 / p32,
                         "fp32r_primary_kernel_ms": k32, "fp32r_resolved": nres,
                         "fp32r_resolved_double_float": ntiers[0], "fp32r_resolved_fp64": ntiers[1],
                         "knn_seconds": knn_s})
            del B64, F64, B32, F32
        del d_nn, d_lu
    worst = max(r["loglik_rel_err"] for r in rows)
    worst_f = max(r["F_max_rel_err"] for r in rows)
    return {"workload": f"n={n} uniform [0,1]^2 x-ordered, X=[1,N(0,1)], code-book neighbors, one fused "
                        f"loglik pass and one updateBF per (m, model, range), FP32R vs FP64",
            "cases": rows, "max_loglik_rel_err": worst, "max_F_rel_err": worst_f,
            "max_B_err": max(r["B_max_err_rel_max_abs"] for r in rows),
            "within_1e-6": bool(worst <= 1e-6 and worst_f <= 1e-6),
            "note": "pass_ms: the whole fused likelihood pass timed with CUDA events on the launching stream "
                    f"(mean of {reps}); fp32r_primary_kernel_ms: its FP32R kernel alone; the gaussian cases "
                    "(1e-6 nugget) are too ill-conditioned for a float factor: their flagged locations are "
                    "re-solved in double-float on the FP32 pipe for m <= 16 and in FP64 for m > 16 "
                    "(fp32r_resolved_double_float / fp32r_resolved_fp64)"}


def section_config0(sp, ctx, skip_cpu=False):
    """The plain response model at its CPU-sized configuration (n = 2000, m = 15, exponential,
    2000 samples; inputs, host-fed streams and the reference's own chain from
    tests/golden/config0_golden.npz): MCMC iterations/s of the GPU chain (FP64 and FP32R,
    through the public rNNGP call with host data) against the CPU implementation on all host
    cores with the same streams, and whether each chain moves at the reference's iterations."""
    from oracle.oracle import Oracle, build

    g = np.load(os.path.join(HERE, "tests", "golden", "config0_golden.npz"))
    nS = g["theta"].shape[1]
    args = (g["y"], g["X"], 15, g["coords"], "exponential", g["nnIndx"], g["lu"], [2, 1], [2, 0.1], [3, 30], None,
            [1.0, -0.5], g["theta_start"], g["tuning"], nS, g["normals"], g["unifs"])
    gmoved = np.any(np.diff(g["theta"], axis=1) != 0, axis=0)
    out = {"workload": "n=2000 uniform, X=[1,N(0,1)], w from a dense exponential GP (sigma2=1, phi=6), tau2=0.1, "
                       "m=15, priors sigma.sq IG(2,1) tau.sq IG(2,0.1) phi U(3,30), 2000 samples, host-fed streams",
           "samples": int(nS)}
    for prec in ("fp64", "fp32r"):
        sp.rNNGP(*args[:14], 50, *args[15:], precision=prec, ctx=ctx)  # warm-up: plan, graph capture
        t0 = time.perf_counter()
        r = sp.rNNGP(*args, precision=prec, ctx=ctx)
        dt = time.perf_counter() - t0
        moved = np.any(np.diff(r["p.theta.samples"], axis=1) != 0, axis=0)
        out[prec] = {"seconds": dt, "iterations_per_s": nS / dt,
                     "same_decisions_as_reference": float(np.mean(moved == gmoved)),
                     "theta_max_rel_err_vs_reference": float(np.max(np.abs(r["p.theta.samples"] - g["theta"]) /
                                                                    np.abs(g["theta"])))}
    if not skip_cpu:
        build()
        orc = Oracle()
        thr = os.cpu_count() or 1
        ccm = lambda a: np.ascontiguousarray(np.asarray(a).T).reshape(-1)  # noqa: E731
        t0 = time.perf_counter()
        ro = orc.rNNGP(g["y"], ccm(g["X"]), 15, ccm(g["coords"]), 0, g["nnIndx"], g["lu"], [2, 1], [2, 0.1], [3, 30],
                       [0.5, 2.5], [1.0, -0.5], g["theta_start"], g["tuning"], nS, g["normals"], g["unifs"],
                       threads=thr)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": nS / dt, "unit": "iterations/s", "cores": thr, "kind": "port",
                               "identical_chain_to_reference": bool(np.array_equal(ro["theta"], g["theta"])),
                               "sample": "the oracle's C port of rNNGP (src/rNNGP.cpp:103-421), the full 2000 "
                                         "samples, OpenMP over locations"}
        out["gpu_fp64_over_cpu"] = out["fp64"]["iterations_per_s"] / out["cpu_baseline"]["value"]
    return out


def section_replicate(sp, ctx, n=N, n_samples=100, skip_cpu=False, seed=404):
    """Replicated data (rNNGPReplicated, the y_rep of fit.rep / fitted.NNGP) at n = 1e6, m = 15,
    exponential, n_samples parameter sets scattered around the headline theta: the
    dataflow GPU solve through the public call (host data in and out), FP32R and FP64,
    against the oracle's sequential recurrence on a two-sample slice of the same inputs."""
    rng = np.random.default_rng(seed)
    c, X, _ = workload(n)
    nb = sp.mkNNIndxCB(c, M, ctx=ctx)
    nn, lu = nb["nnIndx"], nb["nnIndxLU"]
    th = np.array(THETA)[:, None] * rng.uniform(0.8, 1.25, size=(3, n_samples))
    beta = rng.normal(size=(n_samples, 2))
    z = rng.standard_normal(size=n * n_samples)
    out = {"workload": f"n={n} uniform x-ordered, m={M}, exponential, {n_samples} samples (theta within x0.8-1.25 "
                       f"of sigma2={THETA[0]} tau2={THETA[1]} phi={THETA[2]}), X=[1,N(0,1)]",
           "samples": n_samples}
    res = {}
    for prec in ("fp32r", "fp64"):
        sp.rNNGPReplicated(X, M, c, COV, nn, lu, beta[:2], th[:, :2], z[: 2 * n], precision=prec, ctx=ctx)  # warm
        t0 = time.perf_counter()
        r = sp.rNNGPReplicated(X, M, c, COV, nn, lu, beta, th, z, precision=prec, ctx=ctx)["y.rep.samples"]
        dt = time.perf_counter() - t0
        res[prec] = r[:, :2].copy()
        out[prec] = {"seconds": dt, "samples_per_s": n_samples / dt, "solves_per_s": n * n_samples / dt,
                     "h2d_bytes": int(z.nbytes + X.nbytes + c.nbytes + nn.nbytes + lu.nbytes),
                     "d2h_bytes": int(8 * n * n_samples)}
        del r
    if not skip_cpu:
        from oracle.oracle import Oracle, build

        build()
        thr = os.cpu_count() or 1
        ccm = np.ascontiguousarray(c.T).reshape(-1)
        Xcm = np.ascontiguousarray(X.T).reshape(-1)
        t0 = time.perf_counter()
        yo, st = Oracle().rNNGPReplicated(Xcm, M, ccm, 0, nn, lu, beta[:2], np.ascontiguousarray(th[:, :2].T).reshape(-1),
                                          z[: 2 * n], threads=thr)
        dt = time.perf_counter() - t0
        scale = max(1.0, float(np.max(np.abs(yo))))
        out["cpu_baseline"] = {"value": 2 / dt, "unit": "samples/s", "cores": thr, "kind": "port",
                               "sample": "the oracle's C port of rNNGPReplicated (src/rNNGPReplicated.cpp:183-205: "
                                         "updateBF with OpenMP, then the sequential recurrence) on the first 2 samples"}
        out["fp64_max_err_vs_cpu"] = float(np.max(np.abs(res["fp64"] - yo)) / scale)
        out["fp32r_max_err_vs_cpu"] = float(np.max(np.abs(res["fp32r"] - yo)) / scale)
        out["gpu_fp32r_over_cpu"] = out["fp32r"]["samples_per_s"] / out["cpu_baseline"]["value"]
    return out


def clustered_coords(rng, n, blobs=20, sd=0.03, uniform_frac=0.2):
    """Mixture of Gaussian blobs (clipped to the unit square) plus a uniform share."""
    nu = int(round(uniform_frac * n))
    centers = rng.uniform(0.1, 0.9, size=(blobs, 2))
    lab = rng.integers(0, blobs, size=n - nu)
    c = np.vstack([np.clip(centers[lab] + rng.normal(scale=sd, size=(n - nu, 2)), 0.0, 1.0),
                   rng.uniform(size=(nu, 2))])
    return c[rng.permutation(n)]


def section_conj_sweep(sp, ctx, orc=None, n=200_000, seed=91):
    """Batched spConjNNGP: n clustered locations (20 blobs, sd 0.03, plus 20% uniform), p = 3
    covariates N(0,1), y = X beta + w + eps with w an NNGP draw at phi = 10, sigma^2 = 1 and
    tau^2 = 0.2; grid 50 phi in [3,30] x 20 alpha in [0.05,2]; 5 uneven random folds; m = 15."""
    from spnngp_gb300.api import spConjNNGP

    rng = np.random.default_rng(seed)
    c = clustered_coords(rng, n)
    X = np.column_stack([np.ones(n), rng.normal(size=n), rng.normal(size=n)])
    o = np.argsort(c[:, 0], kind="stable")
    co = c[o]
    nb = sp.mkNNIndxCB(co, M, ctx=ctx)
    w = np.empty(n)
    w[o] = nngp_draw(sp, ctx, co, nb["nnIndx"], nb["nnIndxLU"], M, 0, [1.0, 0.0, 10.0], rng)
    y = X @ np.array([1.0, 0.5, -0.5]) + w + rng.normal(scale=np.sqrt(0.2), size=n)
    phis, alphas = np.linspace(3, 30, 50), np.linspace(0.05, 2, 20)
    ta = np.array([[ph, al] for ph in phis for al in alphas])
    perm = rng.permutation(n)
    cuts = np.cumsum((np.array([0.12, 0.16, 0.20, 0.24, 0.28]) * n).astype(int))[:-1]
    folds = np.split(perm, cuts)  # uneven folds, indices in the NNGP (x) order
    g = len(ta)
    solves = sum((n - len(f)) * g + len(f) * g for f in folds) + n
    res = {}
    for prec in ("fp32r", "fp64"):
        t0 = time.perf_counter()
        r = spConjNNGP(y, X, c, n_neighbors=M, theta_alpha=ta, sigma_sq_IG=[2.0, 1.0],
                              cov_model="exponential", k_fold=5, folds=folds, precision=prec, ctx=ctx,
                              return_neighbor_info=False)
        res[prec] = (time.perf_counter() - t0, r)
    t32, r32 = res["fp32r"]
    t64, r64 = res["fp64"]
    s32, s64 = r32["k.fold.scores"][:, 2:], r64["k.fold.scores"][:, 2:]
    out = {
        "workload": f"spConjNNGP k-fold sweep: n={n} clustered (20 blobs sd 0.03 + 20% uniform), p=3, "
                    f"{g}-point (phi, alpha) grid, 5 uneven folds, m={M}, exponential, CRPS selection",
        "seconds_fp32r": t32, "seconds_fp64": t64, "solves": int(solves),
        "solves_per_s_fp32r": solves / t32, "solves_per_s_fp64": solves / t64,
        "selected_fp32r": r32["theta.alpha"], "selected_fp64": r64["theta.alpha"],
        "same_selection": r32["theta.alpha"] == r64["theta.alpha"],
        "score_max_rel_err_fp32r_vs_fp64": float(np.max(np.abs(s32 - s64) / np.abs(s64))),
        "note": "timed through the public spConjNNGP call (host data in, per-fold neighbor searches, "
                "one fused launch over all folds x grid points, device scoring, final fit)",
    }
    if orc is not None:
        # the oracle's C port of cNNGP on one fold at 4 grid points, all host threads
        keep = np.ones(n, bool)
        keep[folds[0]] = False  # fold indices are positions in the x order
        cm_, ym, Xm = co[keep], y[o][keep], X[o][keep]
        nbm = orc.mkNNIndxCB(np.ascontiguousarray(cm_.T).reshape(-1), M, threads=os.cpu_count() or 1)
        thr = os.cpu_count() or 1
        t0 = time.perf_counter()
        orc.cNNGP(ym, np.ascontiguousarray(Xm.T).reshape(-1), np.ascontiguousarray(cm_.T).reshape(-1),
                  ta[:4].reshape(-1), nbm[0], nbm[2], None, None, None, M, [2.0, 1.0], 0, threads=thr)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(ym) * 4 / dt, "unit": "solves/s", "cores": thr, "kind": "port",
                               "sample": f"oracle cNNGP (port of src/cNNGP.cpp:73-358) on one fold "
                                         f"(n={len(ym)}) at 4 grid points, no prediction"}
    return out


def section_serving(sp, ctx, warm_rates=(10, 50, 100, 200, 500, 1000, 2000), cold_rates=(10, 50, 200), seed=55,
                    max_requests=200, pool=32):
    """Serving: Poisson streams of spConjNNGP fit + predict requests, n log-uniform in [1e3, 5e5],
    prediction sets of U[1e3, 1e5] uniform points, m = 15, exponential, (phi, alpha) from the
    50 x 20 grid, HBM budget 150 GB; the continuous-batching server against the plain
    per-request form on the same arrival times.  Warm streams draw their datasets from a pool
    of 32 that the server keeps resident (the neighbor.info reuse); in cold streams every
    request brings a dataset of its own, so its upload, ordering and neighbor search are inside
    its latency."""
    from spnngp_gb300 import serving as S

    rng = np.random.default_rng(seed)
    phis, alphas = np.linspace(3, 30, 50), np.linspace(0.05, 2, 20)

    def make_dataset():
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(5e5))))
        c = rng.uniform(size=(n, 2))
        X = np.column_stack([np.ones(n), rng.normal(size=n)])
        y = X @ np.array([1.0, -0.5]) + np.sin(5 * c[:, 0]) * np.cos(3 * c[:, 1]) + rng.normal(scale=0.3, size=n)
        return c, X, y

    def make_pred():
        n0 = int(rng.uniform(1e3, 1e5))
        return rng.uniform(size=(n0, 2)), np.column_stack([np.ones(n0), rng.normal(size=n0)])

    datasets = [make_dataset() for _ in range(pool)]
    preds = [make_pred() for _ in range(pool)]

    def stream(rate, count, cold=False):
        t = np.cumsum(rng.exponential(1.0 / rate, size=count))
        reqs = []
        for k in range(count):
            pi = int(rng.integers(pool))
            c0, X0 = preds[pi]
            if cold:
                c, X, y = make_dataset()
                key = None  # its own dataset: uploaded, ordered and searched inside the request
            else:
                di = int(rng.integers(pool))
                c, X, y = datasets[di]
                key = di
            reqs.append(S.ConjRequest(c, X, y, c0, X0, float(rng.choice(phis)), float(rng.choice(alphas)),
                                      dataset=key, rid=k, arrival=float(t[k])))
        return reqs

    # warm-up: every pooled dataset resident once, kernels loaded
    srv = S.ConjServer(m=M, precision="fp32r", hbm_budget=150e9, ctx=ctx)
    S.serve(srv, stream(1000.0, pool), realtime=False)
    for d in range(pool):
        c, X, y = datasets[d]
        c0, X0 = preds[d]
        srv.submit(S.ConjRequest(c, X, y, c0, X0, 10.0, 0.5, dataset=d, rid=-1 - d))
    srv.drain()
    S.serve(srv, stream(1000.0, 4, cold=True), realtime=False)
    # accuracy of the served (FP32R) results against FP64 on a sample
    errs = []
    for k, r in enumerate(stream(1000.0, 6)):
        srv.submit(r)
        got = srv.step()[0]
        ref = S.fit_predict_one(r, m=M, precision="fp64", ctx=ctx)
        errs.append(max(abs(got.ab[1] - ref.ab[1]) / abs(ref.ab[1]),
                        float(np.max(np.abs(got.y0_hat - ref.y0_hat)) / max(1.0, np.max(np.abs(ref.y0_hat))))))

    def run(rate, cold):
        count = int(min(max_requests if not cold else 100, max(40, rate * 2)))
        reqs = stream(rate, count, cold=cold)
        before = dict(srv.stats)
        a = S.serve(srv, reqs)
        b = S.serve_per_request(reqs, m=M, precision="fp32r", ctx=ctx)
        # the server (one fused launch per batch) and the per-request host form run different job
        # tables and tile splits, so their FP32R results agree within the stated tolerance, not bitwise
        diff, worst = 0.0, None
        for x, z in zip(sorted(a["results"], key=lambda r: r.rid), sorted(b["results"], key=lambda r: r.rid)):
            for f in ("ab", "beta_hat", "y0_hat", "y0_hat_var"):
                u, v = getattr(x, f), getattr(z, f)
                if u is not None and v is not None:
                    dv = float(np.max(np.abs(u - v)) / max(1.0, float(np.max(np.abs(v)))))
                    if dv > diff:
                        diff, worst = dv, {"field": f, "rid": x.rid, "rid_other": z.rid, "batch": x.batch}
        return {"rate_rps": rate, "requests": count,
                "mean_n": float(np.mean([len(r.y) for r in reqs])),
                "server": {k: a[k] for k in ("throughput_rps", "p50_s", "p99_s", "mean_batch", "failed")},
                "per_request": {k: b[k] for k in ("throughput_rps", "p50_s", "p99_s", "failed")},
                "dataset_builds": srv.stats["misses"] - before["misses"],
                "max_rel_diff_server_vs_per_request": diff, "within_1e-6": diff <= 1e-6, "worst": worst}

    warm = [run(rate, False) for rate in warm_rates]
    cold = [run(rate, True) for rate in cold_rates]
    return {"workload": f"Poisson streams of conjugate fit+predict requests, n log-U[1e3,5e5], prediction sets "
                        f"n0 U[1e3,1e5], m={M}, exponential, FP32R, HBM budget 150 GB; warm: {pool} pooled "
                        f"datasets kept resident; cold: a new dataset per request (upload, ordering and neighbor "
                        f"search inside each request's latency)",
            "warm": warm, "cold": cold, "max_rel_err_fp32r_vs_fp64": float(max(errs)),
            "server_cache": dict(srv.stats)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import Oracle

    impl, kind, what = cpu_reference_impl()
    threads = os.cpu_count() or 1
    c, X, y = workload()
    ccm = np.ascontiguousarray(c.T).reshape(-1)
    Xcm = np.ascontiguousarray(X.T).reshape(-1)
    nn, _, lu = Oracle().mkNNIndxCB(ccm, M, threads=threads)  # neighbor search outside the timed step
    for _ in range(args.warmup):
        cpu_step_oracle(impl, ccm, nn, lu, Xcm, y, threads, N)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_step_oracle(impl, ccm, nn, lu, Xcm, y, threads, N)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = N / dt
    sample = f"full workload: updateBF + Q over all n={N} locations per step, {threads} OpenMP threads; {what}"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    import spnngp_gb300 as sp
    from spnngp_gb300._lib import Context, _dp, _i64

    ctx = Context(dev.index)
    if args.launch_shape:
        parts = [int(v) for v in args.launch_shape.split(",")]
        ctx.set_launch_shape(parts[0], parts[1], bool(parts[2]) if len(parts) > 2 else False)
    # one stream for torch's work (uploads, L2 flush, timing events) and the library's kernels
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    import ctypes as C

    c, X, y = workload()
    t0 = time.perf_counter()
    nbr = sp.mkNNIndxCB(c, M, ctx=ctx)
    knn_s = time.perf_counter() - t0
    nn, lu = nbr["nnIndx"], nbr["nnIndxLU"]
    ccm = np.ascontiguousarray(c.T).reshape(-1)
    V = np.column_stack([X, y])
    nv = V.shape[1]
    Vcm = np.ascontiguousarray(V.T).reshape(-1)
    d_c = torch.from_numpy(ccm).to(dev)
    d_nn = torch.from_numpy(nn).to(dev)
    d_lu = torch.from_numpy(lu).to(dev)
    d_V = torch.from_numpy(Vcm).to(dev)
    d_ld = torch.zeros(1, dtype=torch.float64, device=dev)
    d_G = torch.zeros(nv * nv, dtype=torch.float64, device=dev)
    th = np.array(list(THETA) + [0.0])
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(prec):
        ctx.call("nngp_loglik_gram_dev", N, M, nv, d_c.data_ptr(), d_nn.data_ptr(), d_lu.data_ptr(), d_V.data_ptr(),
                 0, th.ctypes.data_as(_dp), prec, d_ld.data_ptr(), d_G.data_ptr())

    def loglik():
        G = d_G.cpu().numpy().reshape(nv, nv)
        b = np.array([1.0, -0.5])
        q = b @ G[:2, :2] @ b - 2 * b @ G[:2, 2] + G[2, 2]
        return -0.5 * (d_ld.item() + q)

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            flush.zero_()
            step(prec)
        ctx.call("nngp_kernel_time", None, None)  # clear
        ctx.call("nngp_set_kernel_timing", 1)
        ctx.reset_launches()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for e0, e1 in ev:
            flush.zero_()  # L2 flush between timed steps (outside the events)
            e0.record(stream)
            step(prec)
            e1.record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        launches = ctx.launches
        kms = C.c_double()
        kn = _i64()
        ctx.call("nngp_kernel_time", C.byref(kms), C.byref(kn))
        ctx.call("nngp_set_kernel_timing", 0)
        ms = float(sum(e0.elapsed_time(e1) for e0, e1 in ev))
        return ms / steps, kms.value / max(kn.value, 1), launches

    # the clock sampler spans every timed region (FP64 form, FP32R headline, e2e)
    clk = ClockSampler(dev.index).__enter__()
    # FP64 form (for the >= 3x comparison and the error reference)
    ms64, kms64, _ = timed(0, max(3, args.steps // 4), 2)
    ll64 = loglik()
    # FP32R headline
    ms32, kms32, launches = timed(1, args.steps, args.warmup)
    ll32 = loglik()
    max_ms = max_over_ranks(ms32, dev)
    value = whole_job_rate(N, max_ms, ws)

    # e2e: the C-ABI host entry point with pinned host buffers, copies inside the timed region
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    h_c, h_nn, h_lu, h_V = pin(ccm), pin(nn), pin(lu), pin(Vcm)
    h_ld = np.zeros(1)
    h_G = np.zeros(nv * nv)
    from spnngp_gb300._lib import dptr, iptr

    def e2e_step():
        ctx.call("nngp_loglik_gram", N, M, nv, dptr(h_c), iptr(h_nn), iptr(h_lu), dptr(h_V), 0,
                 th.ctypes.data_as(_dp), 1, dptr(h_ld), dptr(h_G))

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_dt = (time.perf_counter() - t0) / e2e_steps
    clk.__exit__(None, None, None)
    h2d = h_c.nbytes + h_nn.nbytes + h_lu.nbytes + h_V.nbytes
    d2h = h_ld.nbytes + h_G.nbytes

    # roofline of the dominant kernel (the FP32R register kernel): its work is CUDA-core FP32
    # arithmetic (build, Cholesky, solves, the Dot2 refinement), so its algorithmic flops are set
    # against the measured FP32 FMA peak; its HBM bytes against the measured copy bandwidth
    pk64, pk32 = C.c_double(), C.c_double()
    ctx.call("nngp_measure_peak", 1, C.byref(pk64))
    ctx.call("nngp_measure_peak", 0, C.byref(pk32))
    base, f32 = algorithmic_flops(M)
    ach32 = N * f32 / (kms32 * 1e-3)
    traffic = None
    tpath = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("bfr_kernel_m15_fused_n1e6_bytes_per_launch")
        except Exception:
            traffic = None
    hbm_peak = None
    ppath = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(ppath):
        try:
            hbm_peak = float(json.load(open(ppath))["hbm_gbs"])
        except Exception:
            hbm_peak = None
    alg_bytes = N * algorithmic_bytes(M, nv)
    hbm_ach = alg_bytes / (kms32 * 1e-3) / 1e9
    tune = ctx.autotune_report()

    cpu = None
    parity = None
    if rank == 0 and not args.skip_cpu:
        try:
            impl, kind, what = cpu_reference_impl()
            threads = os.cpu_count() or 1
            Xcm = np.ascontiguousarray(X.T).reshape(-1)
            ll_cpu, B_cpu, F_cpu = cpu_step_oracle(impl, ccm, nn, lu, Xcm, y, threads, N, keep=True)
            t0 = time.perf_counter()
            reps = 2
            for _ in range(reps):
                cpu_step_oracle(impl, ccm, nn, lu, Xcm, y, threads, N)
            cdt = (time.perf_counter() - t0) / reps
            cpu = {"value": N / cdt, "unit": UNIT, "cores": threads, "kind": kind,
                   "sample": f"updateBF + Q over all n={N} locations ({what}), mean of {reps} runs"}
            parity = section_parity(sp, ctx, c, nbr, ll_cpu, B_cpu, F_cpu, ll64, ll32, threads, kind)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}

    sections = {}
    if rank == 0 and args.sections:
        clk2 = ClockSampler(dev.index).__enter__()
        if "config0" in args.sections:
            sections["config0_mcmc"] = section_config0(sp, ctx, args.skip_cpu)
        if "rep" in args.sections:
            sections["replicate"] = section_replicate(sp, ctx, skip_cpu=args.skip_cpu)
        if "accuracy" in args.sections:
            sections["accuracy"] = section_accuracy(sp, ctx, dev)
        if "mcmc" in args.sections:
            sections["mcmc_batch"] = section_mcmc_batch(sp, ctx, dev, args.mcmc_iters)
        if "conj" in args.sections:
            orc = None
            if not args.skip_cpu:
                from oracle.oracle import Oracle, build as build_oracle

                build_oracle()
                orc = Oracle()
            sections["conj_sweep"] = section_conj_sweep(sp, ctx, orc)
        if "serve" in args.sections:
            sections["serving"] = section_serving(sp, ctx)
        clk2.__exit__(None, None, None)
        sections["sections_clocks"] = clk2.summary()

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": max_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": bench_config(),
            "form": "FP32 covariance build and Cholesky, one double-float (Dot2) residual refinement; "
                    "locations the error estimate flags re-solved in double-float (FP64 where that "
                    "cannot certify them)",
            "fp64_form": {"value": N / (ms64 * 1e-3), "ms_per_step": ms64, "kernel_ms": kms64},
            "fp32r_over_fp64": ms64 / ms32,
            "loglik_rel_err_fp32r_vs_fp64": abs(ll32 - ll64) / abs(ll64),
            "loglik": {"fp64": ll64, "fp32r": ll32},
            "kernel_ms": kms32,
            "knn_seconds_n1e6": knn_s,
            "e2e": {"value": ws * N / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "fp32", "achieved": ach32 / 1e12, "peak": pk32.value / 1e12, "unit": "TFLOP/s",
                         "frac": ach32 / pk32.value, "traffic": traffic,
                         "algorithmic_flops_per_solve": f32, "kernel": "bfr_kernel<15, fused, exponential>",
                         "peak_source": "measured live: FP32 FMA-chain kernel (nngp_measure_peak)",
                         "hbm": {"achieved_gbs": hbm_ach, "peak_gbs": hbm_peak,
                                 "frac": (hbm_ach / hbm_peak) if hbm_peak else None,
                                 "algorithmic_bytes_per_solve": algorithmic_bytes(M, nv),
                                 "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
                         "fp64_pipe_peak_tflops": pk64.value / 1e12},
            "autotune": {k: {"wpb": v["wpb"], "grid_mode": v["grid_mode"], "tmem": v["tmem"], "ms": v["ms"]}
                         for k, v in tune.items()},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
            "parity": parity,
        }
        out.update(sections)
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_profile_pass(args):
    """One (m, model, precision, n) fused pass on resident inputs, --steps times after one untimed
    call (plan, tuning): a short program for ncu captures of one B/F kernel."""
    import torch

    import spnngp_gb300 as sp
    from spnngp_gb300._lib import Context, _dp

    m_s, model, prec, n_s = args.profile_pass.split(",")
    m, n = int(m_s), int(float(n_s))
    theta = dict((r[0], r[2]) for r in ACCURACY_CASES if r[1] == 0.05)[model]
    dev = torch.device("cuda", 0)
    ctx = Context(0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    c, X, y = workload(n)
    nb = sp.mkNNIndxCB(c, m, ctx=ctx)
    V = np.column_stack([X, y])
    nv = V.shape[1]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_c, d_V = t(np.ascontiguousarray(c.T).reshape(-1)), t(np.ascontiguousarray(V.T).reshape(-1))
    d_nn, d_lu = t(nb["nnIndx"]), t(nb["nnIndxLU"])
    d_ld = torch.zeros(1, dtype=torch.float64, device=dev)
    d_G = torch.zeros(nv * nv, dtype=torch.float64, device=dev)
    th = np.array(list(theta) + [0.0] * (4 - len(theta)))
    from spnngp_gb300.core import precision_code

    code, pc = sp.cov_model_index(model), precision_code(prec)

    def run():
        ctx.call("nngp_loglik_gram_dev", n, m, nv, d_c.data_ptr(), d_nn.data_ptr(), d_lu.data_ptr(), d_V.data_ptr(),
                 code, th.ctypes.data_as(_dp), pc, d_ld.data_ptr(), d_G.data_ptr())

    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        run()
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"profile_pass": args.profile_pass, "ms_per_pass": e0.elapsed_time(e1) / args.steps,
                      "log_det": d_ld.item()}), flush=True)
    ctx.close()


def run_profile_rep(args):
    """rNNGPReplicated at N locations and S samples (exponential, m = 15, FP32R), once after one
    untimed call: a short program for ncu captures of the replicate solve's kernels."""
    import torch

    import spnngp_gb300 as sp
    from spnngp_gb300._lib import Context

    n_s, ns_s = args.profile_rep.split(",")
    n, ns = int(float(n_s)), int(ns_s)
    ctx = Context(0)
    c, X, _ = workload(n)
    nb = sp.mkNNIndxCB(c, M, ctx=ctx)
    rng = np.random.default_rng(5)
    th = np.array(THETA)[:, None] * rng.uniform(0.8, 1.25, size=(3, ns))
    beta = rng.normal(size=(ns, 2))
    z = rng.standard_normal(size=n * ns)
    run = lambda: sp.rNNGPReplicated(X, M, c, COV, nb["nnIndx"], nb["nnIndxLU"], beta, th, z,  # noqa: E731
                                     precision="fp32r", ctx=ctx)
    run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    y = run()["y.rep.samples"]
    print(json.dumps({"profile_rep": args.profile_rep, "seconds": time.perf_counter() - t0,
                      "checksum": float(np.sum(y[:, 0]))}), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--sections", default="config0,rep,accuracy,mcmc,conj,serve",
                    help="comma-separated extra workloads reported beside the headline (config0, rep, accuracy, "
                         "mcmc, conj, serve), or ''")
    ap.add_argument("--mcmc-iters", type=int, default=5000)
    ap.add_argument("--launch-shape", default="",
                    help="W,G[,T]: run the FP32R register kernel with W warps per block, grid mode G and "
                         "(T = 1) the tensor-memory layout instead of the autotuned shape (results are "
                         "identical for every shape)")
    ap.add_argument("--profile-pass", default="",
                    help="M,MODEL,PRECISION,N: only run the fused pass at that configuration --steps times (after "
                         "one untimed call) and print its mean time -- the program for ncu captures of one kernel")
    ap.add_argument("--profile-rep", default="",
                    help="N,S: only run rNNGPReplicated at N locations and S samples (after one untimed call) -- "
                         "the program for ncu captures of the replicate kernels")
    args = ap.parse_args()
    if args.profile_pass:
        run_profile_pass(args)
        return
    if args.profile_rep:
        run_profile_rep(args)
        return
    args.warmup = max(args.warmup, 3)
    args.sections = [x for x in args.sections.split(",") if x]
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
