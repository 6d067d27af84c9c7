"""The grid-bucketed neighbor search's exactness argument, checked on the CPU.

A model of the device search (spnngp_gb300/csrc/nngp_knn.cu: build_grid, grid_knn_kernel,
grid_nn2_kernel -- the same grid geometry, ring order, termination bound with its slop, and
tie / near-tie flags, in Python's IEEE double arithmetic with the kernels' expressions) is
compared with brute force (the ring search never stops before it has the exact list) and with
the oracle's code-book search, the reference's fastNN (src/nn.cpp:128-258): every list the grid
search does not hand back to the walk equals the reference's.  The device kernels themselves are
checked against the oracle by the GPU tests; this pins the argument they rest on."""
import math

import numpy as np
import pytest

from conftest import cm

INF = math.inf
CELL_POINTS = 3  # kGridCellPoints


def build_grid(c):
    n = len(c)
    mn, mx = c.min(0), c.max(0)
    W, H = float(mx[0] - mn[0]), float(mx[1] - mn[1])
    span = max(W, H)
    area = max(W, 1e-3 * span) * max(H, 1e-3 * span)
    h = math.sqrt(area * CELL_POINTS / n)
    while True:
        nx, ny = int(min(W / h, 1e9)) + 1, int(min(H / h, 1e9)) + 1
        if nx * ny <= 4 * n + 64:
            break
        h *= 1.25
    M = float(np.abs(np.concatenate([mn, mx])).max())
    g = {"x0": float(mn[0]), "y0": float(mn[1]), "h": h, "inv": 1.0 / h, "nx": nx, "ny": ny,
         "slop": 1e-7 * h + 1e-13 * M}
    cx = np.clip(np.floor((c[:, 0] - g["x0"]) * g["inv"]).astype(np.int64), 0, nx - 1)
    cy = np.clip(np.floor((c[:, 1] - g["y0"]) * g["inv"]).astype(np.int64), 0, ny - 1)
    key = cy * nx + cx
    order = np.argsort(key, kind="stable")  # a cell lists its locations by increasing index
    g["cells"] = np.split(order, np.searchsorted(key[order], np.arange(1, nx * ny)))
    return g


def coord(v, v0, inv, nc):
    return min(max(int(math.floor((v - v0) * inv)), 0), nc - 1)


def ring_search(c, g, qx, qy, visit, full, worst):
    """Visits the cells ring by ring around (qx, qy) until every unvisited cell is farther than
    the current worst key (full() true) or the grid is covered."""
    nx, ny, h = g["nx"], g["ny"], g["h"]
    cx, cy = coord(qx, g["x0"], g["inv"], nx), coord(qy, g["y0"], g["inv"], ny)
    k = 0
    while True:
        for yy in range(max(cy - k, 0), min(cy + k, ny - 1) + 1):
            if yy in (cy - k, cy + k):
                xs = range(max(cx - k, 0), min(cx + k, nx - 1) + 1)
            else:
                xs = [x for x in ((cx - k,) if cx - k >= 0 else ()) + ((cx + k,) if k > 0 and cx + k < nx else ())]
            for xx in xs:
                visit(g["cells"][yy * nx + xx])
        lb = INF
        if cx - k > 0:
            lb = min(lb, qx - (g["x0"] + (cx - k) * h))
        if cx + k < nx - 1:
            lb = min(lb, (g["x0"] + (cx + k + 1) * h) - qx)
        if cy - k > 0:
            lb = min(lb, qy - (g["y0"] + (cy - k) * h))
        if cy + k < ny - 1:
            lb = min(lb, (g["y0"] + (cy + k + 1) * h) - qy)
        if lb == INF:
            return
        if full():
            l = lb - g["slop"]
            if l > 0.0 and l * l > worst() * (1.0 + 1e-12):
                return
        k += 1


def key(qx, qy, xj, yj):
    dx, dy = qx - xj, qy - yj  # __dadd_rn(q, -x), then __dadd_rn(__dmul_rn, __dmul_rn)
    return dx * dx + dy * dy


def grid_cb(c, g, q, cnt):
    """grid_knn_kernel's list for location q (predecessors j < q) and its hand-back flag."""
    qx, qy = float(c[q, 0]), float(c[q, 1])
    kd, il = [], []
    st = {"next": INF, "tie": False}

    def consider(j):
        de = key(qx, qy, float(c[j, 0]), float(c[j, 1]))
        if len(kd) == cnt and not de < kd[-1]:
            st["tie"] |= de == kd[-1]
            st["next"] = min(st["next"], de)
            return
        if len(kd) == cnt:
            st["next"] = min(st["next"], kd[-1])
            kd.pop()
            il.pop()
        t = len(kd)
        while t > 0 and kd[t - 1] > de:
            t -= 1
        st["tie"] |= t > 0 and kd[t - 1] == de
        kd.insert(t, de)
        il.insert(t, j)

    def visit(cell):
        for j in cell:
            if j >= q:
                break
            consider(int(j))

    ring_search(c, g, qx, qy, visit, lambda: len(kd) == cnt, lambda: kd[-1])
    flagged = st["tie"] or (len(kd) == cnt and st["next"] <= kd[-1] * (1.0 + 1e-13))
    return il, kd, flagged


def grid_nn2(c, g, qx, qy, k):
    """grid_nn2_kernel's list: the k nearest training locations ordered by (key, index)."""
    kd, il = [], []

    def visit(cell):
        for j in cell:
            de = key(qx, qy, float(c[j, 0]), float(c[j, 1]))
            if len(kd) == k and not (de < kd[-1] or (de == kd[-1] and j < il[-1])):
                continue
            if len(kd) == k:
                kd.pop()
                il.pop()
            t = len(kd)
            while t > 0 and (kd[t - 1] > de or (kd[t - 1] == de and il[t - 1] > j)):
                t -= 1
            kd.insert(t, de)
            il.insert(t, int(j))

    ring_search(c, g, qx, qy, visit, lambda: len(kd) == k, lambda: kd[-1])
    return il, kd


def cases(kind, n, rng):
    if kind == "uniform":
        c = rng.uniform(size=(n, 2))
    elif kind == "clustered":
        centers = rng.uniform(0.1, 0.9, size=(8, 2))
        c = np.clip(centers[rng.integers(0, 8, size=n)] + rng.normal(scale=0.03, size=(n, 2)), 0, 1)
        c[: n // 5] = rng.uniform(size=(n // 5, 2))
    elif kind == "utm":
        c = rng.uniform(size=(n, 2)) * [2.0e4, 1.5e4] + [4.2e5, 4.6e6]
    elif kind == "lattice":  # exact distance ties
        s = int(math.isqrt(n))
        grid = np.arange(s) / (s - 1.0)
        c = np.array([(x, y) for x in grid for y in grid])
    else:
        raise ValueError(kind)
    return c[np.argsort(c[:, 0], kind="stable")]


@pytest.mark.parametrize("kind,n,m", [("uniform", 2500, 15), ("clustered", 2500, 10), ("utm", 2000, 20),
                                      ("lattice", 1600, 12)])
def test_grid_model_matches_brute_force_and_reference(orc, kind, n, m):
    c = cases(kind, n, np.random.default_rng(n + m))
    n = len(c)
    g = build_grid(c)
    nn, dist, lu = orc.mkNNIndxCB(cm(c), m)
    flagged = 0
    for q in range(150, n, 3):  # q >= 150: the model runs the rings (the kernel scans q < 2048 directly)
        cnt = min(q, m)
        il, kd, fl = grid_cb(c, g, q, cnt)
        # the ring search never stops early: its keys are the cnt smallest of all predecessors
        allk = np.array([key(float(c[q, 0]), float(c[q, 1]), float(c[j, 0]), float(c[j, 1])) for j in range(q)])
        assert np.array_equal(np.sort(allk)[:cnt], np.array(kd)), (kind, q)
        if fl:
            flagged += 1
            continue
        off = lu[q]
        assert list(nn[off:off + cnt]) == il, (kind, q)
        assert np.array_equal(dist[off:off + cnt], np.sqrt(np.array(kd))), (kind, q)
    if kind == "lattice":
        assert flagged > 0  # equal keys go back to the walk
    else:
        assert flagged == 0  # continuous coordinates: no key equalities


@pytest.mark.parametrize("inside", [True, False])
def test_grid_nn2_model_matches_brute_force(inside):
    rng = np.random.default_rng(5 + inside)
    c = rng.uniform(size=(3000, 2))
    c[:40] = c[40:80]  # duplicated training locations: ties ordered by index
    g = build_grid(c)
    k = 12
    pts = rng.uniform(size=(300, 2)) if inside else rng.uniform(-0.6, 1.6, size=(300, 2))
    for qx, qy in pts:
        il, kd = grid_nn2(c, g, float(qx), float(qy), k)
        allk = [key(float(qx), float(qy), float(x), float(y)) for x, y in c]
        ref = sorted(range(len(c)), key=lambda j: (allk[j], j))[:k]
        assert il == ref
