"""The FP32R kernels -- thread per location for m <= 16, warp per location for 16 < m <= 32:
B, F and the fused likelihood sums against the FP64 form and the oracle, for every
correlation model and every compiled neighbor bound; results independent of the launch shape
the autotuner picks."""
import numpy as np
import pytest

from conftest import cm, xorder

pytestmark = pytest.mark.gpu

# FP32R against FP64 (the stated bounds): log-likelihood, per-location F (relative) and B
# (relative to the largest |B|).  The refinement residual uses the covariance in
# double-float, and a location whose estimated F error exceeds 1e-8 F is re-solved in FP64.
TOL_LOGLIK = 1e-6
TOL_F = 1e-6
TOL_B = 1e-6

MODELS = [("exponential", (1.0, 0.1, 6.0)), ("exponential", (1.0, 0.0, 59.91)),
          ("spherical", (2.0, 0.2, 3.0)), ("matern", (1.0, 0.1, 9.488, 1.5)),
          ("matern", (1.0, 0.1, 30.0, 2.5)), ("matern", (1.0, 0.2, 12.0, 0.8)),
          ("gaussian", (1.0, 1e-6, 34.62)), ("gaussian", (1.0, 1e-6, 3.462)), ("gaussian", (1.0, 0.05, 4.0))]


def dataset(n, seed, nv=3):
    rng = np.random.default_rng(seed)
    c = xorder(rng.uniform(size=(n, 2)))
    X = np.column_stack([np.ones(n)] + [rng.normal(size=n) for _ in range(nv - 2)])
    y = X @ np.linspace(1.0, -0.5, nv - 1) + rng.normal(size=n)
    return c, X, y


def loglik(ld, G, beta):
    p = len(beta)
    return -0.5 * (ld + beta @ G[:p, :p] @ beta - 2 * beta @ G[:p, p] + G[p, p])


@pytest.mark.parametrize("model,theta", MODELS)
@pytest.mark.parametrize("m", [5, 10, 12, 15, 16, 17, 20, 24, 25, 32])
def test_fp32r_B_F_against_fp64(sp, orc, model, theta, m):
    c, X, y = dataset(3000, 10 + m)
    o = orc.mkNNIndxCB(cm(c), m)
    B64, F64, ld64 = sp.updateBF(c, o[0], o[2], m, model, theta, "fp64")
    B32, F32, ld32 = sp.updateBF(c, o[0], o[2], m, model, theta, "fp32r")
    assert np.all(np.isfinite(B32)) and np.all(F32 > 0)
    assert np.max(np.abs(F32 - F64) / F64) <= TOL_F
    assert abs(ld32 - ld64) <= TOL_LOGLIK * max(1.0, abs(ld64))
    assert np.max(np.abs(B32 - B64)) <= TOL_B * max(1.0, np.max(np.abs(B64)))


@pytest.mark.parametrize("model,theta", MODELS)
@pytest.mark.parametrize("m,nv", [(10, 2), (15, 3), (16, 5), (20, 3), (32, 4), (32, 8)])
def test_fp32r_fused_loglik_against_fp64(sp, orc, model, theta, m, nv):
    c, X, y = dataset(5000, 20 + m, nv)
    o = orc.mkNNIndxCB(cm(c), m)
    V = np.column_stack([X, y])
    ld64, G64 = sp.loglik_gram(c, o[0], o[2], m, V, model, theta, "fp64")
    ld32, G32 = sp.loglik_gram(c, o[0], o[2], m, V, model, theta, "fp32r")
    beta = np.linspace(1.0, -0.5, nv - 1)
    ll64, ll32 = loglik(ld64, G64, beta), loglik(ld32, G32, beta)
    assert abs(ll32 - ll64) <= TOL_LOGLIK * abs(ll64)
    assert np.max(np.abs(G32 - G64)) <= 1e-6 * np.max(np.abs(G64))


def test_fp32r_matches_oracle_loglik(sp, orc):
    """The fused FP32R pass against the oracle's port of updateBF + Q (src/rNNGP.cpp:306-317)."""
    c, X, y = dataset(4000, 33)
    m = 15
    o = orc.mkNNIndxCB(cm(c), m)
    theta = (1.3, 0.2, 11.0)
    Bo, Fo, ldo, st = orc.updateBF(cm(c), o[0], o[2], m, 0, *theta, 0.0)
    assert st == 0
    beta = np.array([1.0, 0.25])
    r = X @ beta - y
    llo = -0.5 * (ldo + orc.Q(Bo, Fo, r, r, o[0], o[2]))
    ld, G = sp.loglik_gram(c, o[0], o[2], m, np.column_stack([X, y]), "exponential", theta, "fp32r")
    assert abs(loglik(ld, G, beta) - llo) <= TOL_LOGLIK * abs(llo)


SHAPES = [(1, 0, 0), (2, 0, 0), (4, 0, 0), (8, 0, 0), (1, 1, 0), (4, 1, 0), (8, 2, 0), (2, 2, 0),
          (4, 0, 1), (8, 0, 1), (4, 1, 1), (8, 2, 1)]


@pytest.mark.parametrize("m", [10, 15, 16])
def test_launch_shape_does_not_change_results(sp, orc, m):
    """Every launch shape the autotuner may pick gives bitwise-identical results."""
    c, X, y = dataset(7001, 40 + m)
    o = orc.mkNNIndxCB(cm(c), m)
    V = np.column_stack([X, y])
    ctx = sp.default_context()
    ref = None
    try:
        for wpb, gm, tm in SHAPES:
            ctx.set_launch_shape(wpb, gm, tm)
            B, F, ld = sp.updateBF(c, o[0], o[2], m, "exponential", (1.0, 0.1, 8.0), "fp32r")
            ldg, G = sp.loglik_gram(c, o[0], o[2], m, V, "exponential", (1.0, 0.1, 8.0), "fp32r")
            got = (B, F, np.array([ld]), np.array([ldg]), G)
            if ref is None:
                ref = got
            else:
                for a, b in zip(ref, got):
                    assert np.array_equal(a, b), (wpb, gm, tm)
    finally:
        ctx.set_launch_shape(0, 0, 0)
    ldt, Gt = sp.loglik_gram(c, o[0], o[2], m, V, "exponential", (1.0, 0.1, 8.0), "fp32r")
    assert ldt == ref[3][0] and np.array_equal(Gt, ref[4])


def test_autotune_reports_choice(sp):
    """A pass of at least 2048 tiles (64 K locations) is tuned once per class; smaller ones run
    the default shape untuned."""
    ctx = sp.Context(0)
    small = dataset(20000, 76)
    nbs = sp.mkNNIndxCB(small[0], 15, ctx=ctx)
    sp.loglik_gram(small[0], nbs["nnIndx"], nbs["nnIndxLU"], 15, np.column_stack(small[1:]), "gaussian",
                   (1.0, 0.1, 5.0), "fp32r", ctx=ctx)
    assert ctx.autotune_report() == {}
    c, X, y = dataset(100_000, 77)
    nb = sp.mkNNIndxCB(c, 15, ctx=ctx)
    o = (nb["nnIndx"], None, nb["nnIndxLU"])
    V = np.column_stack([X, y])
    sp.loglik_gram(c, o[0], o[2], 15, V, "gaussian", (1.0, 0.1, 5.0), "fp32r", ctx=ctx)
    rep = ctx.autotune_report()
    key = [k for k in rep if k.startswith("M=15 mode=1 cov=3")]
    assert len(key) == 1
    e = rep[key[0]]
    assert 1 <= e["wpb"] <= 8 and len(e["candidates"]) >= 4
    assert e["ms"] == pytest.approx(min(e["candidates"].values()), rel=1e-3, abs=1e-4)
    # a second pass of the same class reuses the choice
    sp.loglik_gram(c, o[0], o[2], 15, V, "gaussian", (1.0, 0.1, 5.0), "fp32r", ctx=ctx)
    assert ctx.autotune_report() == rep
    ctx.close()


@pytest.mark.parametrize("m", [15, 32])
@pytest.mark.parametrize("precision", ["fp32r", "fp64"])
def test_streamed_host_form_matches_resident_form(sp, precision, m):
    """The host-pointer entry points stream their inputs in location chunks (n = 300k: 2 chunks)
    and launch the pass tile range by tile range; results are bitwise those of the
    device-pointer form, which runs the pass in one launch."""
    import ctypes as C

    import torch

    from spnngp_gb300._lib import _dp

    n, nv = 300_000, 3
    c, X, y = dataset(n, 91, nv)
    nb = sp.mkNNIndxCB(c, m)
    nn, lu = nb["nnIndx"], nb["nnIndxLU"]
    V = np.column_stack([X, y])
    theta = (1.0, 0.1, 30.0)
    ld_h, G_h = sp.loglik_gram(c, nn, lu, m, V, "exponential", theta, precision)
    B_h, F_h, ldb_h = sp.updateBF(c, nn, lu, m, "exponential", theta, precision)
    ctx = sp.default_context()
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_c, d_nn, d_lu, d_V = t(cm(c)), t(nn), t(lu), t(cm(V))
    d_ld = torch.zeros(1, dtype=torch.float64, device=dev)
    d_G = torch.zeros(nv * nv, dtype=torch.float64, device=dev)
    th = np.array(list(theta) + [0.0])
    prec = 1 if precision == "fp32r" else 0
    torch.cuda.synchronize()  # the library runs on its own stream
    ctx.call("nngp_loglik_gram_dev", n, m, nv, d_c.data_ptr(), d_nn.data_ptr(), d_lu.data_ptr(), d_V.data_ptr(), 0,
             th.ctypes.data_as(_dp), prec, d_ld.data_ptr(), d_G.data_ptr())
    assert d_ld.item() == ld_h
    assert np.array_equal(d_G.cpu().numpy().reshape(nv, nv), G_h)
    d_B = torch.zeros(len(nn), dtype=torch.float64, device=dev)
    d_F = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    ctx.call("nngp_updateBF_dev", n, m, d_c.data_ptr(), d_nn.data_ptr(), d_lu.data_ptr(), 0, th.ctypes.data_as(_dp),
             prec, d_B.data_ptr(), d_F.data_ptr(), d_ld.data_ptr())
    assert np.array_equal(d_B.cpu().numpy(), B_h) and np.array_equal(d_F.cpu().numpy(), F_h)
    assert d_ld.item() == ldb_h


@pytest.mark.parametrize("m", [20, 32])
def test_fp32r_wide_matches_oracle_and_flags_ill_conditioned(sp, orc, m):
    """16 < m <= 32 (the warp-per-location kernel): B, F and the fused pass against the oracle's
    port of updateBF + Q on a well-conditioned case; and a gaussian case with a 1e-6 nugget at
    range 0.5, whose float pivots fail or whose error estimate exceeds the bound almost
    everywhere, against the FP64 form (F there is a 1e-6 remainder of a cancellation, so even
    two FP64 evaluations agree only to about 1e-5: the oracle is no reference for it)."""
    c, X, y = dataset(2500, 60 + m)
    o = orc.mkNNIndxCB(cm(c), m)
    V = np.column_stack([X, y])
    beta = np.array([1.0, 0.25])
    theta = (1.3, 0.2, 11.0)
    Bo, Fo, ldo, st = orc.updateBF(cm(c), o[0], o[2], m, 0, *theta, 0.0)
    assert st == 0
    r = X @ beta - y
    llo = -0.5 * (ldo + orc.Q(Bo, Fo, r, r, o[0], o[2]))
    ld, G = sp.loglik_gram(c, o[0], o[2], m, V, "exponential", theta, "fp32r")
    assert abs(loglik(ld, G, beta) - llo) <= TOL_LOGLIK * abs(llo)
    B, F, _ = sp.updateBF(c, o[0], o[2], m, "exponential", theta, "fp32r")
    assert np.max(np.abs(F - Fo) / Fo) <= TOL_F
    assert np.max(np.abs(B - Bo)) <= TOL_B * max(1.0, np.max(np.abs(Bo)))
    gau = (1.0, 1e-6, 3.462)
    ld64, G64 = sp.loglik_gram(c, o[0], o[2], m, V, "gaussian", gau, "fp64")
    ld32, G32 = sp.loglik_gram(c, o[0], o[2], m, V, "gaussian", gau, "fp32r")
    assert abs(loglik(ld32, G32, beta) - loglik(ld64, G64, beta)) <= TOL_LOGLIK * abs(loglik(ld64, G64, beta))
    B64, F64, _ = sp.updateBF(c, o[0], o[2], m, "gaussian", gau, "fp64")
    B32, F32, _ = sp.updateBF(c, o[0], o[2], m, "gaussian", gau, "fp32r")
    assert np.max(np.abs(F32 - F64) / F64) <= TOL_F
    assert np.max(np.abs(B32 - B64)) <= TOL_B * max(1.0, np.max(np.abs(B64)))


@pytest.mark.parametrize("m", [15, 32])
def test_resolved_count_reports_fp64_handoffs(sp, orc, m):
    """nngp_fp32r_resolved: a well-conditioned case re-solves (almost) nothing in FP64; the
    gaussian with a 1e-6 nugget at range 0.5 re-solves most locations; an FP64 pass reports 0."""
    c, X, y = dataset(4000, 80 + m)
    o = orc.mkNNIndxCB(cm(c), m)
    ctx = sp.default_context()
    sp.updateBF(c, o[0], o[2], m, "exponential", (1.0, 0.1, 6.0), "fp32r")
    r_easy, n_easy = ctx.fp32r_resolved()
    assert n_easy == 4000 and r_easy <= 40
    sp.updateBF(c, o[0], o[2], m, "gaussian", (1.0, 1e-6, 3.462), "fp32r")
    r_hard, n_hard = ctx.fp32r_resolved()
    assert n_hard == 4000 and r_hard >= 2000
    sp.updateBF(c, o[0], o[2], m, "gaussian", (1.0, 1e-6, 3.462), "fp64")
    assert ctx.fp32r_resolved() == (0, 0)


@pytest.mark.parametrize("m", [10, 15, 16, 20, 32])
@pytest.mark.parametrize("phi", [34.62, 3.462])
def test_double_float_tier_on_ill_conditioned_gaussian(sp, orc, m, phi):
    """Gaussian covariance with a 1e-6 nugget (condition numbers ~1e7): nearly every location is
    flagged by the float solve; the double-float re-solve takes them (thread per location for
    m <= 16, warp per location beyond; FP64 only for tiles it cannot certify), and F stays
    within 1e-6 of its exact value (extended precision) and the log-likelihood within 1e-6 of
    the FP64 form."""
    from test_gpu_parity_scale import _exact_F

    c, X, y = dataset(4000, 300 + m)
    o = orc.mkNNIndxCB(cm(c), m)
    theta = (1.0, 1e-6, phi)
    ctx = sp.default_context()
    _, F32, _ = sp.updateBF(c, o[0], o[2], m, "gaussian", theta, "fp32r")
    n_df, n_64 = ctx.fp32r_tiers()
    resolved, _ = ctx.fp32r_resolved()
    assert n_df + n_64 == resolved and resolved > 0.5 * len(c)
    assert n_df > 0.5 * resolved  # the double-float tier takes most of them
    Ft = _exact_F(c, o[0], o[2], m, theta)
    assert float(np.max(np.abs(F32 - Ft) / Ft)) <= 1e-6
    V = np.column_stack([X, y])
    beta = np.array([1.0, -0.5])
    ll = {}
    for prec in ("fp64", "fp32r"):
        ld, G = sp.loglik_gram(c, o[0], o[2], m, V, "gaussian", theta, prec)
        ll[prec] = -0.5 * (ld + beta @ G[:2, :2] @ beta - 2 * beta @ G[:2, 2] + G[2, 2])
    assert abs(ll["fp32r"] - ll["fp64"]) <= 1e-6 * abs(ll["fp64"])


@pytest.mark.parametrize("m", [15, 20, 32])
@pytest.mark.parametrize("model,theta", [("spherical", (1.0, 1e-7, 0.8)), ("matern", (1.0, 1e-5, 2.0, 2.3))])
def test_double_float_tier_scalar_covariance_paths(sp, m, model, theta):
    """The double-float re-solve on the covariance paths without a packed form: spherical and
    Matern with a general nu (K_nu evaluated in FP64), long ranges and small nuggets, so the
    float factor cannot be certified (F stays above 1e-6 (sigma^2 + tau^2), the double-float
    tier's floor); F, B and the log-likelihood against the FP64 form."""
    c, X, y = dataset(6000, 900 + m)
    ctx = sp.default_context()
    nb = sp.mkNNIndxCB(c, m)
    nn, lu = nb["nnIndx"], nb["nnIndxLU"]
    B64, F64, _ = sp.updateBF(c, nn, lu, m, model, theta, "fp64")
    B32, F32, _ = sp.updateBF(c, nn, lu, m, model, theta, "fp32r")
    n_df, n_64 = ctx.fp32r_tiers()
    assert n_df > 0.25 * len(c), (n_df, n_64)  # the tier under test took a good share
    assert float(np.max(np.abs(F32 - F64) / F64)) <= TOL_F
    assert float(np.max(np.abs(B32 - B64))) <= TOL_B * max(1.0, float(np.max(np.abs(B64))))
    V = np.column_stack([X, y])
    beta = np.array([1.0, -0.5])
    ll = {}
    for prec in ("fp64", "fp32r"):
        ld, G = sp.loglik_gram(c, nn, lu, m, V, model, theta, prec)
        ll[prec] = loglik(ld, G, beta)
    assert abs(ll["fp32r"] - ll["fp64"]) <= TOL_LOGLIK * abs(ll["fp64"])


@pytest.mark.parametrize("m,precision", [(20, "fp32r"), (32, "fp32r")])
def test_warp_kernel_tuning_keeps_results(sp, m, precision):
    """The warp-per-location FP32R kernel (16 < m <= 32) is tuned on its first large pass (1, 2
    or 4 warps per block, one tile per warp or a persistent grid); the tuned shape gives
    bitwise the results of the default shape."""
    c, X, y = dataset(80_000, 500 + m)
    V = np.column_stack([X, y])
    ctx = sp.Context(0)
    nb = sp.mkNNIndxCB(c, m, ctx=ctx)
    theta = (1.0, 0.1, 8.0)
    ctx.call("nngp_set_autotune", 0)
    B0, F0, _ = sp.updateBF(c, nb["nnIndx"], nb["nnIndxLU"], m, "exponential", theta, precision, ctx=ctx)
    ld0, G0 = sp.loglik_gram(c, nb["nnIndx"], nb["nnIndxLU"], m, V, "exponential", theta, precision, ctx=ctx)
    ctx.call("nngp_set_autotune", 1)
    B1, F1, _ = sp.updateBF(c, nb["nnIndx"], nb["nnIndxLU"], m, "exponential", theta, precision, ctx=ctx)
    ld1, G1 = sp.loglik_gram(c, nb["nnIndx"], nb["nnIndxLU"], m, V, "exponential", theta, precision, ctx=ctx)
    rep = ctx.autotune_report()
    bound = 20 if m <= 20 else 24 if m <= 24 else 32  # the warp kernels' instantiated bounds
    prefix = f"warp M={bound} "
    keys = [k for k in rep if k.startswith(prefix)]
    assert len(keys) == 2  # the standalone and the fused mode
    for k in keys:
        assert rep[k]["wpb"] in (1, 2, 4) and len(rep[k]["candidates"]) >= 3
    assert np.array_equal(B0, B1) and np.array_equal(F0, F1)
    assert ld0 == ld1 and np.array_equal(G0, G1)
    ctx.close()
