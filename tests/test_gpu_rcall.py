"""The R package's .Call layer (src/nngp_call.cpp, src/init.cpp) on a GB300: the stand-in's
drivers wrap the golden inputs into SEXPs and call rNNGP, cNNGP, rNNGPPredict,
rNNGPReplicated, mkNNIndx, mkNNIndxCB and mkUIndx by name, exactly as they call the
reference's own routines to make tests/golden; the named outputs must match the reference's.
The layer draws R's random numbers itself (norm_rand / unif_rand, here the stand-in's
host-fed streams), so the chain replays only if it consumes them in the reference's order."""
import numpy as np
import pytest

from conftest import cm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def layer():
    from spnngp_gb300.build import build

    build()
    from oracle.oracle import RCALL_SO, Reference, build as build_oracle

    build_oracle(rcall=True)
    return Reference(RCALL_SO)


@pytest.mark.parametrize("case", ["uniform", "lattice", "dupx", "small"])
@pytest.mark.parametrize("m", [4, 10, 15])
def test_neighbor_routines(layer, golden, case, m):
    key = f"knn_{case}_m{m}"
    if key + "_lu" not in golden:
        pytest.skip("m larger than n")
    c = cm(golden[f"knn_{case}_coords"])
    nn, dist, lu, st = layer.mkNNIndxCB(c, m)
    assert st == 0, layer.error()
    assert np.array_equal(nn, golden[key + "_cb_nnIndx"]) and np.array_equal(lu, golden[key + "_lu"])
    assert np.array_equal(dist, golden[key + "_cb_nnDist"])
    nb, db, lub, st = layer.mkNNIndx(c, m)
    assert st == 0, layer.error()
    assert np.array_equal(nb, golden[key + "_brute_nnIndx"]) and np.array_equal(db, golden[key + "_brute_nnDist"])


@pytest.mark.parametrize("st", [0, 1, 2])
def test_mkUIndx(layer, golden, st):
    u, ulu, ui, s = layer.mkUIndx(2000, 10, golden["knn_uniform_m10_cb_nnIndx"], golden["knn_uniform_m10_lu"], st)
    assert s == 0, layer.error()
    assert np.array_equal(u, golden[f"uindx_t{st}_u"]) and np.array_equal(ulu, golden[f"uindx_t{st}_ulu"])
    assert np.array_equal(ui, golden[f"uindx_t{st}_ui"])


@pytest.mark.parametrize("model", [0, 2])
def test_rNNGP(layer, golden, model):
    g = golden
    t = f"mc{model}"
    r = layer.rNNGP(g["mc_y"], cm(g["mc_X"]), 10, cm(g["mc_coords"]), model, g["mc_nnIndx"], g["mc_lu"], [2, 1],
                    [2, 0.1], [3, 30], [0.5, 2.5], [1.0, -0.5], g[f"{t}_theta_start"], g[f"{t}_tuning"], 150,
                    g[f"{t}_normals"], g[f"{t}_unifs"], n_rep=5, rep_indx=g[f"{t}_repindx"])
    assert r["status"] == 0, layer.error()
    th, gth = r["theta"], g[f"{t}_theta"]
    assert np.array_equal(np.any(np.diff(th, axis=1) != 0, axis=0), np.any(np.diff(gth, axis=1) != 0, axis=0))
    assert np.max(np.abs(th - gth) / np.abs(gth)) <= 1e-9
    assert np.max(np.abs(r["beta"] - g[f"{t}_beta"])) <= 1e-8
    assert np.max(np.abs(r["rep"] - g[f"{t}_rep"])) <= 1e-8
    # the layer drew exactly as many normals and uniforms as the reference consumed
    assert tuple(r["used"][:2]) == tuple(g[f"{t}_used"])


@pytest.mark.parametrize("model", [0, 2])
def test_cNNGP(layer, golden, model):
    g = golden
    t = f"cj{model}"
    r = layer.cNNGP(g["mc_y"], cm(g["mc_X"]), cm(g["mc_coords"]), g[f"{t}_theta_alpha"].reshape(-1), g["mc_nnIndx"],
                    g["mc_lu"], cm(g["cj_X0"]), cm(g["cj_coords0"]), cm(g["cj_nnIndx0"]), 10, [2.0, 1.0], model)
    assert r["status"] == 0, layer.error()
    for k in ("beta", "ab", "bb", "y0", "y0var"):
        ref = g[f"{t}_{k}"]
        assert np.max(np.abs(r[k] - ref)) <= 1e-9 * max(1.0, np.max(np.abs(ref))), k
    for j in range(r["bBInv"].shape[1]):
        low = np.tril(r["bBInv"][:, j].reshape(2, 2).T)
        assert np.max(np.abs(low - np.tril(g[f"{t}_bBInv"][:, j].reshape(2, 2).T))) <= 1e-9


def test_rNNGPPredict_and_replicates(layer, golden):
    g = golden
    y0, st = layer.rNNGPPredict(cm(g["mc_X"]), g["mc_y"], cm(g["mc_coords"]), 10, cm(g["cj_X0"]), cm(g["cj_coords0"]),
                                cm(g["cj_nnIndx0"]), cm(g["pr_beta"]), cm(g["pr_theta"]), 0, g["pr_z"])
    assert st == 0, layer.error()
    assert np.max(np.abs(y0 - g["pr_y0"])) <= 1e-9 * max(1.0, np.max(np.abs(g["pr_y0"])))
    yr, st = layer.rNNGPReplicated(cm(g["mc_X"]), 10, cm(g["mc_coords"]), 0, g["mc_nnIndx"], g["mc_lu"], g["rp_beta"],
                                   cm(g["pr_theta"]), g["rp_normals"])
    assert st == 0, layer.error()
    assert np.max(np.abs(yr - g["rp_yrep"])) <= 1e-9 * max(1.0, np.max(np.abs(g["rp_yrep"])))


def test_not_spd_becomes_an_R_error(layer, golden):
    g = golden
    # a negative nugget larger than sigma^2: the first pivot fails
    c = cm(g["bf_coords"])
    ta = np.array([6.0, -2.0])
    layer.lib.ref_clear_error()
    r = layer.cNNGP(g["mc_y"][:800] if len(g["mc_y"]) >= 800 else np.resize(g["mc_y"], 800), np.ones(800), c, ta,
                    g["bf_nnIndx"], g["bf_lu"], None, None, None, 10, [2.0, 1.0], 0)
    assert r["status"] != 0 and "cNNGP" in layer.error()
