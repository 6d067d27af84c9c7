"""CUDA kernels against the oracle (and the reference fixtures): neighbor search
bit-exact, B/F / Q / fused Gram within the stated tolerances."""
import numpy as np
import pytest

from conftest import cm, xorder

pytestmark = pytest.mark.gpu

# Tolerances (relative): FP64 mode vs the reference's potrf->potri->symv path.
TOL_FP64 = 1e-10
# FP32R mode (float build + Cholesky, one FP64-residual refinement) vs FP64:
TOL_FP32R_LOGLIK = 1e-6


def lattice(k):
    g = np.arange(k) / (k - 1)
    xx, yy = np.meshgrid(g, g)
    return np.column_stack([xx.ravel(), yy.ravel()])


# ------------------------------------------------------------------ neighbors

@pytest.mark.parametrize("case", ["uniform", "lattice", "dupx", "small"])
@pytest.mark.parametrize("m", [4, 10, 15])
def test_knn_matches_reference_fixtures(sp, golden, case, m):
    key = f"knn_{case}_m{m}"
    if key + "_lu" not in golden:
        pytest.skip("m larger than n")
    c = golden[f"knn_{case}_coords"]
    g = sp.mkNNIndxCB(c, m)
    assert np.array_equal(g["nnIndx"], golden[key + "_cb_nnIndx"])
    assert np.array_equal(g["nnDist"], golden[key + "_cb_nnDist"])
    assert np.array_equal(g["nnIndxLU"], golden[key + "_lu"])
    b = sp.mkNNIndx(c, m)
    assert np.array_equal(b["nnIndx"], golden[key + "_brute_nnIndx"])
    assert np.array_equal(b["nnDist"], golden[key + "_brute_nnDist"])


@pytest.mark.parametrize("n,m,seed", [(5000, 15, 1), (3000, 32, 2), (2500, 64, 3), (40, 40, 4), (41, 40, 5),
                                      (1, 1, 6), (2, 1, 7), (300, 1, 8)])
def test_knn_cb_random(sp, orc, n, m, seed):
    rng = np.random.default_rng(seed)
    c = xorder(rng.uniform(size=(n, 2)) * [1000.0, 300.0] + [5e5, 4e6])  # UTM-like magnitudes
    g = sp.mkNNIndxCB(c, m)
    o = orc.mkNNIndxCB(cm(c), m)
    assert np.array_equal(g["nnIndx"], o[0])
    assert np.array_equal(g["nnDist"], o[1])
    assert np.array_equal(g["nnIndxLU"], o[2])


def _knn_case(kind, n, rng):
    if kind == "uniform":
        return xorder(rng.uniform(size=(n, 2)))
    if kind == "clustered":
        centers = rng.uniform(0.1, 0.9, size=(20, 2))
        lab = rng.integers(0, 20, size=n)
        c = np.clip(centers[lab] + rng.normal(scale=0.03, size=(n, 2)), 0, 1)
        c[: n // 5] = rng.uniform(size=(n // 5, 2))
        return xorder(c)
    if kind == "line":  # collinear, y constant
        return xorder(np.column_stack([rng.uniform(size=n), np.full(n, 0.25)]))
    if kind == "duplicates":  # every location three times
        base = rng.uniform(size=(n // 3, 2))
        return xorder(np.vstack([base, base, base]))
    if kind == "utm":
        return xorder(rng.uniform(size=(n, 2)) * [2.0e4, 1.5e4] + [4.2e5, 4.6e6])
    raise ValueError(kind)


@pytest.mark.parametrize("kind,n,m", [("uniform", 60_000, 15), ("uniform", 20_000, 32), ("clustered", 30_000, 15),
                                      ("line", 12_000, 10), ("duplicates", 9_000, 12), ("utm", 25_000, 20),
                                      ("uniform", 2_049, 15), ("uniform", 4_000, 64)])
def test_knn_cb_grid_matches_oracle(sp, orc, kind, n, m):
    """Past 2048 locations the search runs on the grid (locations whose result could depend on
    the walk's order go back to the walk): indices and distances bit-exact with the oracle's
    port of the reference's code-book search."""
    c = _knn_case(kind, n, np.random.default_rng(n + m))
    g = sp.mkNNIndxCB(c, m)
    o = orc.mkNNIndxCB(cm(c), m)
    assert np.array_equal(g["nnIndx"], o[0])
    assert np.array_equal(g["nnDist"], o[1])
    assert np.array_equal(g["nnIndxLU"], o[2])


@pytest.mark.parametrize("k", [12, 30, 70])
def test_knn_cb_ties(sp, orc, k):
    # regular lattice in a non-x order (ties in x, in u = x + y and in distance)
    c = lattice(k)
    rng = np.random.default_rng(k)
    c = c[rng.permutation(len(c))]
    for m in (5, 12):
        g = sp.mkNNIndxCB(c, m)
        o = orc.mkNNIndxCB(cm(c), m)
        assert np.array_equal(g["nnIndx"], o[0])
        assert np.array_equal(g["nnDist"], o[1])
        b = sp.mkNNIndx(c, m)
        ob = orc.mkNNIndx(cm(c), m)
        assert np.array_equal(b["nnIndx"], ob[0])
        assert np.array_equal(b["nnDist"], ob[1])


@pytest.mark.parametrize("st", [0, 1, 2])
def test_uindx_matches_reference(sp, golden, st):
    u = sp.mkUIndx(2000, 10, golden["knn_uniform_m10_cb_nnIndx"], golden["knn_uniform_m10_lu"], st)
    assert np.array_equal(u["u.indx"], golden[f"uindx_t{st}_u"])
    assert np.array_equal(u["u.indx.lu"], golden[f"uindx_t{st}_ulu"])
    assert np.array_equal(u["ui.indx"], golden[f"uindx_t{st}_ui"])


def test_uindx_larger(sp, orc):
    rng = np.random.default_rng(11)
    c = xorder(rng.uniform(size=(20000, 2)))
    o = orc.mkNNIndxCB(cm(c), 15)
    for st in (1, 2):
        g = sp.mkUIndx(20000, 15, o[0], o[2], st)
        r = orc.mkUIndx(20000, 15, o[0], o[2], st)
        assert np.array_equal(g["u.indx"], r[0]) and np.array_equal(g["u.indx.lu"], r[1])
        assert np.array_equal(g["ui.indx"], r[2])


@pytest.mark.parametrize("n,n0,k", [(3000, 500, 15), (500, 200, 32), (50, 10, 50)])
def test_nn2_exact(sp, orc, n, n0, k):
    rng = np.random.default_rng(n + k)
    c = rng.uniform(size=(n, 2))
    c0 = rng.uniform(size=(n0, 2))
    gi, gd = sp.nn2(c, c0, k)
    oi, od = orc.nn2(c, c0, k)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)


@pytest.mark.parametrize("kind,n,n0,k", [("uniform", 40_000, 5_000, 15), ("clustered", 30_000, 4_000, 25),
                                         ("lattice", 4_900, 3_000, 12), ("outside", 20_000, 3_000, 10)])
def test_nn2_grid_cases(sp, orc, kind, n, n0, k):
    """The grid search of nn2: prediction points inside and outside the training extent,
    clustered training sets, and a lattice with exact distance ties (ordered by index)."""
    rng = np.random.default_rng(n0 + k)
    if kind == "lattice":
        g = np.arange(70) / 69.0
        c = np.array([(x, y) for x in g for y in g])
        c0 = np.round(rng.uniform(size=(n0, 2)) * 138) / 138.0  # on the half-lattice: many ties
    elif kind == "clustered":
        c = _knn_case("clustered", n, rng)
        c0 = rng.uniform(size=(n0, 2))
    else:
        c = rng.uniform(size=(n, 2))
        c0 = rng.uniform(-0.5, 1.5, size=(n0, 2)) if kind == "outside" else rng.uniform(size=(n0, 2))
    gi, gd = sp.nn2(c, c0, k)
    oi, od = orc.nn2(c, c0, k)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)


# ---------------------------------------------------------------- B, F and Q

@pytest.mark.parametrize("k", range(5))
def test_updateBF_fp64_matches_reference(sp, golden, k):
    model = int(golden[f"bf{k}_model"])
    th = golden[f"bf{k}_theta"]
    B, F, ld = sp.updateBF(golden["bf_coords"], golden["bf_nnIndx"], golden["bf_lu"], 10, model, th, "fp64")
    gB, gF, gld = golden[f"bf{k}_B"], golden[f"bf{k}_F"], float(golden[f"bf{k}_logdet"])
    assert np.max(np.abs(B - gB)) <= TOL_FP64 * np.max(np.abs(gB))
    assert np.max(np.abs(F - gF) / gF) <= TOL_FP64
    assert abs(ld - gld) <= TOL_FP64 * abs(gld)
    q = sp.Q(B, F, golden["bf_u"], golden["bf_v"], golden["bf_nnIndx"], golden["bf_lu"])
    assert abs(q - float(golden[f"bf{k}_Q"])) <= TOL_FP64 * abs(float(golden[f"bf{k}_Q"]))


CASES = [("exponential", (1.0, 0.1, 6.0)), ("exponential", (1.0, 0.1, 59.91)), ("spherical", (2.0, 0.2, 3.0)),
         ("matern", (1.0, 0.1, 9.488, 1.5)), ("matern", (1.0, 0.2, 12.0, 0.8)), ("gaussian", (1.0, 0.05, 4.0))]


@pytest.mark.parametrize("model,theta", CASES)
@pytest.mark.parametrize("m", [10, 15, 20, 32])
def test_updateBF_fp64_random(sp, orc, model, theta, m):
    rng = np.random.default_rng(m)
    n = 4000
    c = xorder(rng.uniform(size=(n, 2)))
    o = orc.mkNNIndxCB(cm(c), m)
    B, F, ld = sp.updateBF(c, o[0], o[2], m, model, theta, "fp64")
    Bo, Fo, ldo, st = orc.updateBF(cm(c), o[0], o[2], m, model, *theta[:3], theta[3] if len(theta) > 3 else 0.0)
    assert st == 0
    assert np.max(np.abs(B - Bo)) <= TOL_FP64 * max(1.0, np.max(np.abs(Bo)))
    assert np.max(np.abs(F - Fo) / Fo) <= TOL_FP64
    assert abs(ld - ldo) <= TOL_FP64 * abs(ldo)


@pytest.mark.parametrize("model,theta", CASES)
@pytest.mark.parametrize("m", [15, 32])
def test_updateBF_fp32r_loglik_error(sp, orc, model, theta, m):
    rng = np.random.default_rng(100 + m)
    n = 6000
    c = xorder(rng.uniform(size=(n, 2)))
    o = orc.mkNNIndxCB(cm(c), m)
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = X @ [1.0, -0.5] + rng.normal(size=n)
    V = np.column_stack([X, y])
    ld64, G64 = sp.loglik_gram(c, o[0], o[2], m, V, model, theta, "fp64")
    ld32, G32 = sp.loglik_gram(c, o[0], o[2], m, V, model, theta, "fp32r")
    beta = np.array([1.0, -0.5])
    q64 = beta @ G64[:2, :2] @ beta - 2 * beta @ G64[:2, 2] + G64[2, 2]
    q32 = beta @ G32[:2, :2] @ beta - 2 * beta @ G32[:2, 2] + G32[2, 2]
    ll64, ll32 = -0.5 * (ld64 + q64), -0.5 * (ld32 + q32)
    assert abs(ll32 - ll64) <= TOL_FP32R_LOGLIK * abs(ll64)


@pytest.mark.parametrize("model,theta", CASES[:4])
def test_loglik_gram_matches_Q_composition(sp, orc, model, theta):
    rng = np.random.default_rng(5)
    n, m = 3000, 15
    c = xorder(rng.uniform(size=(n, 2)))
    o = orc.mkNNIndxCB(cm(c), m)
    X = np.column_stack([np.ones(n), rng.normal(size=n), rng.normal(size=n)])
    y = rng.normal(size=n)
    V = np.column_stack([X, y])
    ld, G = sp.loglik_gram(c, o[0], o[2], m, V, model, theta, "fp64")
    Bo, Fo, ldo, st = orc.updateBF(cm(c), o[0], o[2], m, model, *theta[:3], theta[3] if len(theta) > 3 else 0.0)
    assert abs(ld - ldo) <= TOL_FP64 * abs(ldo)
    for a in range(4):
        for b in range(4):
            ref = orc.Q(Bo, Fo, V[:, a], V[:, b], o[0], o[2])
            assert abs(G[a, b] - ref) <= TOL_FP64 * max(1.0, abs(ref))


@pytest.mark.parametrize("m", [10, 32])
def test_not_spd_reports_location(sp, orc, m):
    # a negative nugget larger than sigma^2 makes the first pivot negative at location 1
    rng = np.random.default_rng(3)
    c = xorder(rng.uniform(size=(200, 2)))
    o = orc.mkNNIndxCB(cm(c), m)
    for prec in ("fp64", "fp32r"):
        with pytest.raises(sp.NNGPError) as e:
            sp.updateBF(c, o[0], o[2], m, "exponential", (1.0, -2.0, 6.0), prec)
        assert e.value.status == 3 and e.value.location == 1


def test_duplicate_coordinates_like_oracle(sp, orc):
    # duplicated coordinates with no nugget: singular neighborhoods; the status must agree with the oracle
    rng = np.random.default_rng(4)
    c = xorder(rng.uniform(size=(300, 2)))
    c[151] = c[150]
    o = orc.mkNNIndxCB(cm(c), 10)
    _, _, _, st = orc.updateBF(cm(c), o[0], o[2], 10, 0, 1.0, 0.0, 6.0, 0.0)
    if st != 0:
        with pytest.raises(sp.NNGPError) as e:
            sp.updateBF(c, o[0], o[2], 10, "exponential", (1.0, 0.0, 6.0), "fp64")
        assert e.value.status == 3 and e.value.location >= 151


def test_bad_arguments_raise(sp):
    with pytest.raises(sp.NNGPError):
        sp.updateBF(np.zeros((10, 2)), np.zeros(45, np.int32), np.zeros(20, np.int32), 40, "exponential",
                    (1, 0.1, 1), "fp64")
    with pytest.raises(ValueError):
        sp.cov_model_index("cubic")


def test_fp64_pass_on_two_devices_in_one_process(sp, orc):
    """The FP64 kernels' shared-memory attribute is set per device: a pass on a second device of
    the same process must launch (skipped when only one GPU is visible)."""
    import torch

    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU visible")
    rng = np.random.default_rng(9)
    c = xorder(rng.uniform(size=(3000, 2)))
    o = orc.mkNNIndxCB(cm(c), 15)
    out = []
    for dev in (0, 1):
        ctx = sp.Context(dev)
        out.append(sp.updateBF(c, o[0], o[2], 15, "exponential", (1.0, 0.1, 6.0), "fp64", ctx=ctx))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
