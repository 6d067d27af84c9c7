"""The oracle restatement (oracle/nngp_oracle.c) against fixtures produced by the
reference's own C++ (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest
from scipy.special import kv

from conftest import cm


@pytest.mark.parametrize("case", ["uniform", "lattice", "dupx", "small"])
@pytest.mark.parametrize("m", [4, 10, 15])
def test_knn_cb_and_brute(orc, golden, case, m):
    key = f"knn_{case}_m{m}"
    if key + "_lu" not in golden:
        pytest.skip("m larger than n")
    c = golden[f"knn_{case}_coords"]
    nn, dist, lu = orc.mkNNIndxCB(cm(c), m)
    assert np.array_equal(nn, golden[key + "_cb_nnIndx"])
    assert np.array_equal(dist, golden[key + "_cb_nnDist"])
    assert np.array_equal(lu, golden[key + "_lu"])
    nb, db, lub = orc.mkNNIndx(cm(c), m)
    assert np.array_equal(nb, golden[key + "_brute_nnIndx"])
    assert np.array_equal(db, golden[key + "_brute_nnDist"])
    assert np.array_equal(lub, golden[key + "_lu"])


@pytest.mark.parametrize("st", [0, 1, 2])
def test_uindx(orc, golden, st):
    u, ulu, ui = orc.mkUIndx(2000, 10, golden["knn_uniform_m10_cb_nnIndx"], golden["knn_uniform_m10_lu"], st)
    assert np.array_equal(u, golden[f"uindx_t{st}_u"])
    assert np.array_equal(ulu, golden[f"uindx_t{st}_ulu"])
    assert np.array_equal(ui, golden[f"uindx_t{st}_ui"])


@pytest.mark.parametrize("k", range(5))
def test_updateBF_and_Q(orc, golden, k):
    model = int(golden[f"bf{k}_model"])
    th = golden[f"bf{k}_theta"]
    B, F, ld, st = orc.updateBF(cm(golden["bf_coords"]), golden["bf_nnIndx"], golden["bf_lu"], 10, model,
                                th[0], th[1], th[2], th[3])
    assert st == 0
    gB, gF = golden[f"bf{k}_B"], golden[f"bf{k}_F"]
    assert np.max(np.abs(B - gB)) <= 1e-12 * np.max(np.abs(gB))
    assert np.max(np.abs(F - gF) / gF) <= 1e-12
    assert abs(ld - float(golden[f"bf{k}_logdet"])) <= 1e-12 * abs(float(golden[f"bf{k}_logdet"]))
    q = orc.Q(B, F, golden["bf_u"], golden["bf_v"], golden["bf_nnIndx"], golden["bf_lu"])
    assert abs(q - float(golden[f"bf{k}_Q"])) <= 1e-10 * abs(float(golden[f"bf{k}_Q"]))


@pytest.mark.parametrize("model", [0, 2])
def test_mcmc_replay(orc, golden, model):
    t = f"mc{model}"
    g = golden
    r = orc.rNNGP(g["mc_y"], cm(g["mc_X"]), 10, cm(g["mc_coords"]), model, g["mc_nnIndx"], g["mc_lu"], [2, 1],
                  [2, 0.1], [3, 30], [0.5, 2.5], [1.0, -0.5], g[f"{t}_theta_start"], g[f"{t}_tuning"], 150,
                  g[f"{t}_normals"], g[f"{t}_unifs"], n_rep=5, rep_indx=g[f"{t}_repindx"])
    assert r["status"] == 0
    assert np.array_equal(r["theta"], g[f"{t}_theta"])  # identical accept/reject sequence and values
    assert np.max(np.abs(r["beta"] - g[f"{t}_beta"])) <= 1e-10
    assert np.max(np.abs(r["rep"] - g[f"{t}_rep"])) <= 1e-9
    assert tuple(r["used"][:2]) == tuple(g[f"{t}_used"])


@pytest.mark.parametrize("model", [0, 2])
def test_conjugate(orc, golden, model):
    g = golden
    t = f"cj{model}"
    ta = g[f"{t}_theta_alpha"]
    r = orc.cNNGP(g["mc_y"], cm(g["mc_X"]), cm(g["mc_coords"]), ta.reshape(-1), g["mc_nnIndx"], g["mc_lu"],
                  cm(g["cj_X0"]), cm(g["cj_coords0"]), cm(g["cj_nnIndx0"]), 10, [2.0, 1.0], model)
    assert r["status"] == 0
    for k in ("beta", "ab", "bb", "y0", "y0var"):
        ref = g[f"{t}_{k}"]
        assert np.max(np.abs(r[k] - ref)) <= 1e-10 * max(1.0, np.max(np.abs(ref))), k
    p = 2
    for j in range(r["bBInv"].shape[1]):
        low = np.tril(r["bBInv"][:, j].reshape(p, p).T)
        refl = np.tril(g[f"{t}_bBInv"][:, j].reshape(p, p).T)
        assert np.max(np.abs(low - refl)) <= 1e-12


def test_predict_and_replicates(orc, golden):
    g = golden
    y0, st = orc.rNNGPPredict(cm(g["mc_X"]), g["mc_y"], cm(g["mc_coords"]), 10, cm(g["cj_X0"]), cm(g["cj_coords0"]),
                              cm(g["cj_nnIndx0"]), cm(g["pr_beta"]), cm(g["pr_theta"]), 0, g["pr_z"])
    assert st == 0 and np.max(np.abs(y0 - g["pr_y0"])) <= 1e-10
    yr, st = orc.rNNGPReplicated(cm(g["mc_X"]), 10, cm(g["mc_coords"]), 0, g["mc_nnIndx"], g["mc_lu"], g["rp_beta"],
                                 cm(g["pr_theta"]), g["rp_normals"])
    assert st == 0 and np.max(np.abs(yr - g["rp_yrep"])) <= 1e-9


def test_bessel_against_scipy(orc):
    worst = 0.0
    for nu in (0.1, 0.5, 0.8, 1.0, 1.5, 2.3, 2.5, 3.7, 7.2):
        for x in np.concatenate([np.logspace(-6, 0.3, 25), np.linspace(2.001, 80, 40)]):
            worst = max(worst, abs(orc.bessel_k(x, nu) - kv(nu, x)) / kv(nu, x))
    assert worst < 1e-13


@pytest.mark.parametrize("nu,closed", [(0.5, lambda x: np.exp(-x)), (1.5, lambda x: (1 + x) * np.exp(-x)),
                                       (2.5, lambda x: (1 + x + x * x / 3) * np.exp(-x))])
def test_matern_half_integer_closed_forms(orc, nu, closed):
    for d in (1e-4, 0.01, 0.1, 0.5, 1.3):
        phi = 7.0
        assert abs(orc.spcor(d, phi, nu, 2) - closed(phi * d)) <= 1e-13


def test_spherical_boundaries(orc):
    phi = 4.0
    assert orc.spcor(0.0, phi, 0, 1) == 1.0
    assert orc.spcor(1.0 / phi, phi, 0, 1) == pytest.approx(0.0, abs=1e-15)
    assert orc.spcor(2.0 / phi, phi, 0, 1) == 0.0


def test_shell_sort_tie_order(orc):
    # equal keys move only past strictly greater ones; pinned against the lattice fixture above
    x, idx = orc.rsort_with_index([3.0, 1.0, 2.0, 1.0, 3.0, 0.5, 1.0, 2.0, 1.0, 0.5, 3.0],
                                  list(range(11)))
    assert list(x) == sorted(x)


def test_config0_chain_replay(orc):
    """The n = 2000, m = 15 response model with a 2000-sample chain (tests/golden/config0_golden.npz,
    made by the reference's own C++): the oracle finds the same neighbor lists and replays the
    chain with identical accept/reject decisions."""
    import os

    from conftest import ROOT

    g = np.load(os.path.join(ROOT, "tests", "golden", "config0_golden.npz"))
    nn, dist, lu = orc.mkNNIndxCB(cm(g["coords"]), 15, threads=os.cpu_count() or 1)
    assert np.array_equal(nn, g["nnIndx"]) and np.array_equal(lu, g["lu"]) and np.array_equal(dist, g["nnDist"])
    r = orc.rNNGP(g["y"], cm(g["X"]), 15, cm(g["coords"]), 0, g["nnIndx"], g["lu"], [2, 1], [2, 0.1], [3, 30],
                  [0.5, 2.5], [1.0, -0.5], g["theta_start"], g["tuning"], 2000, g["normals"], g["unifs"],
                  threads=os.cpu_count() or 1)
    assert r["status"] == 0
    assert np.array_equal(r["theta"], g["theta"])
    assert np.max(np.abs(r["beta"] - g["beta"])) <= 1e-10
    assert tuple(r["used"][:2]) == tuple(g["used"])
