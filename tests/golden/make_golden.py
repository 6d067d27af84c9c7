"""Generates the golden fixtures in this folder from the reference package's own
C++ (src/*.cpp of spNNGP 1.0.1, compiled unmodified against the R-API stand-in
by oracle/Makefile -> oracle/_ref/libspnngp_ref.so).

Run where the reference sources are available (the spNNGP source tree, given
as the argument or in the SPNNGP_REFERENCE environment variable):
    python tests/golden/make_golden.py /path/to/spNNGP
It writes reference_golden.npz (small cases of every routine) and
config0_golden.npz (the n = 2000, m = 15 response model with a 2000-sample
chain).
The inputs are seeded synthetic data (uniform coordinates, a regular lattice
with exact distance ties, coordinates with repeated x values); the random
streams fed to the MCMC are stored with the outputs so a run can be replayed.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
from oracle.oracle import Reference  # noqa: E402


def xorder(coords):
    """R's default NNGP ordering: order(coords[,1]), stable for ties."""
    return coords[np.argsort(coords[:, 0], kind="stable")]


def cm(coords):
    return np.ascontiguousarray(coords.T).reshape(-1)


def lattice(k):
    g = np.arange(k) / (k - 1)
    xx, yy = np.meshgrid(g, g)
    return np.column_stack([xx.ravel(), yy.ravel()])


def main(ref_root):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref_root}"], check=True)
    R = Reference()
    rng = np.random.default_rng(20241203)
    out = {}

    # ---- neighbor search
    knn_cases = {
        "uniform": xorder(rng.uniform(size=(2000, 2))),
        "lattice": xorder(lattice(25)),
        "dupx": xorder(np.column_stack([np.round(rng.uniform(size=900) * 20) / 20, rng.uniform(size=900)])),
        "small": xorder(rng.uniform(size=(17, 2))),
    }
    for name, c in knn_cases.items():
        out[f"knn_{name}_coords"] = c
        for m in (4, 10, 15):
            if m > len(c):
                continue
            a = R.mkNNIndxCB(cm(c), m)
            b = R.mkNNIndx(cm(c), m)
            assert a[3] == 0 and b[3] == 0, R.error()
            out[f"knn_{name}_m{m}_cb_nnIndx"], out[f"knn_{name}_m{m}_cb_nnDist"], out[f"knn_{name}_m{m}_lu"] = a[:3]
            out[f"knn_{name}_m{m}_brute_nnIndx"], out[f"knn_{name}_m{m}_brute_nnDist"] = b[:2]
    # reverse index of the uniform m = 10 graph
    nn, lu = out["knn_uniform_m10_cb_nnIndx"], out["knn_uniform_m10_lu"]
    for st in (0, 1, 2):
        u, ulu, ui, s = R.mkUIndx(2000, 10, nn, lu, st)
        assert s == 0
        out[f"uindx_t{st}_u"], out[f"uindx_t{st}_ulu"], out[f"uindx_t{st}_ui"] = u, ulu, ui

    # ---- B / F and Q at fixed theta on the uniform graph (m = 10 on the first 800 points)
    c = knn_cases["uniform"][:800]
    a = R.mkNNIndxCB(cm(c), 10)
    out["bf_coords"], out["bf_nnIndx"], out["bf_lu"] = c, a[0], a[2]
    bf_cases = [(0, [1.0, 0.1, 6.0, 0.0]), (1, [2.0, 0.2, 3.0, 0.0]), (2, [1.0, 0.1, 9.0, 1.5]),
                (2, [1.5, 0.3, 12.0, 0.8]), (3, [1.0, 0.05, 4.0, 0.0])]
    u = rng.normal(size=800)
    v = rng.normal(size=800)
    out["bf_u"], out["bf_v"] = u, v
    for k, (model, th) in enumerate(bf_cases):
        B, F, ld, s = R.updateBF(cm(c), a[0], a[2], 10, model, th, nu_unif_b=3.0)
        assert s == 0
        out[f"bf{k}_model"], out[f"bf{k}_theta"] = np.array(model), np.array(th)
        out[f"bf{k}_B"], out[f"bf{k}_F"], out[f"bf{k}_logdet"] = B, F, np.array(ld)
        out[f"bf{k}_Q"] = np.array(R.Q(B, F, u, v, a[0], a[2]))

    # ---- response MCMC (config-0 style, shortened)
    n, m, p = 300, 10, 2
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    D = np.sqrt(((c[:, None, :] - c[None, :, :]) ** 2).sum(-1))
    w = np.linalg.cholesky(np.exp(-6.0 * D) + 1e-10 * np.eye(n)) @ rng.normal(size=n)
    y = X @ np.array([1.0, -0.5]) + w + rng.normal(scale=np.sqrt(0.1), size=n)
    a = R.mkNNIndxCB(cm(c), m)
    out.update(mc_coords=c, mc_X=X, mc_y=y, mc_nnIndx=a[0], mc_lu=a[2])
    nS = 150
    for model, ts, tu in ((0, [1.0, 0.1, 6.0], [0.1, 0.1, 0.5]), (2, [1.0, 0.1, 6.0, 1.2], [0.1, 0.1, 0.5, 0.1])):
        nr = 5
        ri = np.zeros(nS, np.int32)
        ri[-nr:] = 1
        normals = rng.normal(size=nS * (p + len(ts)) + nr * n + 16)
        unifs = rng.uniform(size=nS + 4)
        r = R.rNNGP(y, cm(X), m, cm(c), model, a[0], a[2], [2, 1], [2, 0.1], [3, 30], [0.5, 2.5], [1.0, -0.5], ts, tu,
                    nS, normals, unifs, n_rep=nr, rep_indx=ri)
        assert r["status"] == 0, R.error()
        tag = f"mc{model}"
        out.update({f"{tag}_theta_start": np.array(ts), f"{tag}_tuning": np.array(tu), f"{tag}_normals": normals,
                    f"{tag}_unifs": unifs, f"{tag}_repindx": ri, f"{tag}_beta": r["beta"], f"{tag}_theta": r["theta"],
                    f"{tag}_rep": r["rep"], f"{tag}_used": np.array(r["used"][:2])})

    # ---- conjugate fit + prediction
    n0 = 40
    c0 = rng.uniform(size=(n0, 2))
    X0 = np.column_stack([np.ones(n0), rng.normal(size=n0)])
    D0 = np.sqrt(((c0[:, None, :] - c[None, :, :]) ** 2).sum(-1))
    nn0 = np.argsort(D0, axis=1, kind="stable")[:, :m].astype(np.int32)
    out.update(cj_coords0=c0, cj_X0=X0, cj_nnIndx0=nn0)
    for model, ta in ((0, np.array([[3.0, 0.1], [10.0, 0.5], [20.0, 1.0]])),
                      (2, np.array([[3.0, 0.1, 0.7], [10.0, 0.5, 1.5]]))):
        r = R.cNNGP(y, cm(X), cm(c), ta.reshape(-1), a[0], a[2], cm(X0), cm(c0), cm(nn0), m, [2.0, 1.0], model)
        assert r["status"] == 0, R.error()
        tag = f"cj{model}"
        out[f"{tag}_theta_alpha"] = ta
        for k in ("beta", "ab", "bBInv", "bb", "y0", "y0var"):
            out[f"{tag}_{k}"] = r[k]

    # ---- response prediction and replicates
    nS = 12
    beta = rng.normal(size=(p, nS))
    theta = np.vstack([rng.uniform(0.5, 2, nS), rng.uniform(0.05, 0.3, nS), rng.uniform(3, 20, nS)])
    z = rng.normal(size=n0 * nS)
    y0, s = R.rNNGPPredict(cm(X), y, cm(c), m, cm(X0), cm(c0), cm(nn0), cm(beta), cm(theta), 0, z)
    assert s == 0
    out.update(pr_beta=beta, pr_theta=theta, pr_z=z, pr_y0=y0)
    bsp = rng.normal(size=(nS, p))
    normals = rng.normal(size=nS * n)
    yr, s = R.rNNGPReplicated(cm(X), m, cm(c), 0, a[0], a[2], bsp, cm(theta), normals)
    assert s == 0
    out.update(rp_beta=bsp, rp_normals=normals, rp_yrep=yr)

    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes,", len(out), "arrays")
    config0(R)


def config0(R):
    """The plain response model at its CPU-sized configuration: n = 2000 locations iid
    U[0,1]^2 in x order, X = [1, N(0,1)], beta = (1, -0.5), w from the full exponential GP
    (sigma^2 = 1, phi = 6) by a dense Cholesky factor, y = X beta + w + N(0, 0.1); m = 15
    code-book neighbors; priors sigma.sq IG(2, 1), tau.sq IG(2, 0.1), phi U(3, 30); 2000
    samples from theta = (1, 0.1, 6) with tuning (0.1, 0.1, 0.5).  Stores the inputs, the
    host-fed streams and the reference's chain."""
    rng = np.random.default_rng(20250601)
    n, m, p, nS = 2000, 15, 2, 2000
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    D = np.sqrt(((c[:, None, :] - c[None, :, :]) ** 2).sum(-1))
    w = np.linalg.cholesky(np.exp(-6.0 * D) + 1e-10 * np.eye(n)) @ rng.normal(size=n)
    y = X @ np.array([1.0, -0.5]) + w + rng.normal(scale=np.sqrt(0.1), size=n)
    a = R.mkNNIndxCB(cm(c), m)
    assert a[3] == 0, R.error()
    ts, tu = [1.0, 0.1, 6.0], [0.1, 0.1, 0.5]
    normals = rng.normal(size=nS * (p + len(ts)) + 16)
    unifs = rng.uniform(size=nS + 4)
    r = R.rNNGP(y, cm(X), m, cm(c), 0, a[0], a[2], [2, 1], [2, 0.1], [3, 30], [0.5, 2.5], [1.0, -0.5], ts, tu, nS,
                normals, unifs)
    assert r["status"] == 0, R.error()
    out = dict(coords=c, X=X, y=y, nnIndx=a[0], nnDist=a[1], lu=a[2], theta_start=np.array(ts), tuning=np.array(tu),
               normals=normals, unifs=unifs, beta=r["beta"], theta=r["theta"], used=np.array(r["used"][:2]))
    path = os.path.join(HERE, "config0_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPNNGP_REFERENCE")
    if not src:
        sys.exit("usage: make_golden.py /path/to/spNNGP (or set SPNNGP_REFERENCE)")
    main(src)
