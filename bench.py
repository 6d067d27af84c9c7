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
fraction against the measured FP64 pipe peak, and the CPU baseline (the
oracle's C port of the reference loop, OpenMP on all host cores).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

Under torchrun (N > 1) every rank runs the same workload on its own GPU
(replicas: the pass does not exchange data) and value is the sum of solves
over all ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
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
    """Per-solve flop counts of the minimal algorithm (covariance build, Cholesky, two
    triangular solves, F), split into the FP32 part and the FP64 refinement part."""
    P = m * (m + 1) / 2
    base = 8 * P + m ** 3 / 3 + m ** 2 / 2 + m / 6 + 2 * m ** 2 + 2 * m
    fp32 = 8 * P + m ** 3 / 3 + m ** 2 / 2 + m / 6 + 2 * m ** 2 + 2 * m ** 2  # build, factor, solves, correction
    fp64 = 2 * m ** 2 + m + 2 * m + m  # residual c - C b, F, B update
    return base, fp32, fp64


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


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_step_oracle(orc, ccm, nn, lu, Xcm, y, threads, n):
    """One reference-path step on the host: updateBF (potrf/potri/symv per location) plus the
    log-likelihood quadratic form Q(X beta - y), as src/rNNGP.cpp:306-317 computes them."""
    B, F, ld, st = orc.updateBF(ccm, nn, lu, M, 0, *THETA, 0.0, threads=threads)
    r = Xcm[:n] * 1.0 + Xcm[n:] * -0.5 - y
    q = orc.Q(B, F, r, r, nn, lu, threads=threads)
    return -0.5 * (ld + q)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import Oracle, build

    build()
    orc = Oracle()
    threads = os.cpu_count() or 1
    c, X, y = workload()
    ccm = np.ascontiguousarray(c.T).reshape(-1)
    Xcm = np.ascontiguousarray(X.T).reshape(-1)
    nn, _, lu = orc.mkNNIndxCB(ccm, M, threads=threads)
    for _ in range(args.warmup):
        cpu_step_oracle(orc, ccm, nn, lu, Xcm, y, threads, N)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_step_oracle(orc, ccm, nn, lu, Xcm, y, threads, N)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = N / dt
    sample = f"full workload: updateBF + Q over all n={N} locations per step, {threads} OpenMP threads"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"n={N} uniform, m={M}, {COV} theta={THETA}, updateBF+loglik",
                   "l2": "host path"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
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
    stream = torch.cuda.current_stream(dev)
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

    # FP64 form (for the >= 3x comparison and the error reference)
    ms64, kms64, _ = timed(0, max(3, args.steps // 4), 2)
    ll64 = loglik()
    # FP32R headline, timed region under the clock sampler
    with ClockSampler(dev.index) as clk:
        ms32, kms32, launches = timed(1, args.steps, args.warmup)
    ll32 = loglik()
    max_ms = ms32
    if ws > 1:
        t = torch.tensor([ms32], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        max_ms = float(t.item())
    value = ws * N / (max_ms * 1e-3)

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
    h2d = h_c.nbytes + h_nn.nbytes + h_lu.nbytes + h_V.nbytes
    d2h = h_ld.nbytes + h_G.nbytes

    # roofline of the dominant kernel: the FP32R B/F kernel is bound by the FP64 pipe
    # (the refinement residual), so its FP64 algorithmic flops are set against the
    # measured FP64 FMA peak; the FP32 share is reported alongside.
    pk64, pk32 = C.c_double(), C.c_double()
    ctx.call("nngp_measure_peak", 1, C.byref(pk64))
    ctx.call("nngp_measure_peak", 0, C.byref(pk32))
    base, f32, f64 = algorithmic_flops(M)
    ach64 = N * f64 / (kms32 * 1e-3)
    ach32 = N * f32 / (kms32 * 1e-3)
    traffic = None
    tpath = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("bf_kernel_fp32r_n1e6_m15_bytes_per_launch")
        except Exception:
            traffic = None

    cpu = None
    if rank == 0 and not args.skip_cpu:
        try:
            from oracle.oracle import Oracle, build

            build()
            orc = Oracle()
            threads = os.cpu_count() or 1
            Xcm = np.ascontiguousarray(X.T).reshape(-1)
            cpu_step_oracle(orc, ccm, nn, lu, Xcm, y, threads, N)
            t0 = time.perf_counter()
            reps = 2
            for _ in range(reps):
                cpu_step_oracle(orc, ccm, nn, lu, Xcm, y, threads, N)
            cdt = (time.perf_counter() - t0) / reps
            cpu = {"value": N / cdt, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"updateBF + Q over all n={N} locations (the oracle's C port of src/rNNGP.cpp:46-101 "
                             f"and src/util.cpp:261-280), mean of {reps} runs"}
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": max_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"n={N} uniform [0,1]^2 x-ordered, m={M} code-book neighbors, {COV} "
                                   f"sigma2={THETA[0]} tau2={THETA[1]} phi={THETA[2]}, fused updateBF+loglik, "
                                   f"X=[1,N(0,1)], FP32 build/Cholesky + one FP64-residual refinement",
                       "l2": "flushed between timed steps (512 MB write); inputs ~100 MB"},
            "fp64_form": {"value": N / (ms64 * 1e-3), "ms_per_step": ms64, "kernel_ms": kms64},
            "fp32r_over_fp64": ms64 / ms32,
            "loglik_rel_err_fp32r_vs_fp64": abs(ll32 - ll64) / abs(ll64),
            "loglik": {"fp64": ll64, "fp32r": ll32},
            "kernel_ms": kms32,
            "knn_seconds_n1e6": knn_s,
            "e2e": {"value": ws * N / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "fp64", "achieved": ach64 / 1e12, "peak": pk64.value / 1e12, "unit": "TFLOP/s",
                         "frac": ach64 / pk64.value, "traffic": traffic,
                         "peak_source": "measured live (FMA-chain kernel, nngp_measure_peak)",
                         "fp32_share": {"achieved": ach32 / 1e12, "peak": pk32.value / 1e12,
                                        "frac": ach32 / pk32.value}},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
