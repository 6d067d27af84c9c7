"""Host-side logic of the conjugate server (admission, eviction, HBM accounting), on the CPU: no
device work runs here."""
import collections

import numpy as np

from spnngp_gb300 import serving as S


def bare_server(budget, cache=True):
    srv = object.__new__(S.ConjServer)
    srv.m, srv.budget, srv.max_batch, srv.cache = 15, int(budget), 512, cache
    srv.queue = collections.deque()
    srv.datasets = collections.OrderedDict()
    srv.resident = 0
    srv.iterations = 0
    srv.stats = {"hits": 0, "misses": 0, "evictions": 0, "rejected": 0}
    return srv


def req(n, n0, rid, dataset=None):
    return S.ConjRequest(np.zeros((n, 2)), np.zeros((n, 2)), np.zeros(n), np.zeros((n0, 2)), np.zeros((n0, 2)),
                         5.0, 0.5, dataset=dataset, rid=rid)


def test_byte_formulas_grow_with_sizes():
    assert S.dataset_bytes(2000, 2, 15) < S.dataset_bytes(4000, 2, 15)
    assert S.request_bytes(1000, 10, 2, 15) < S.request_bytes(1000, 20, 2, 15)
    # nnIndx dominates a resident dataset: 4 bytes per neighbor pair
    n, m = 100000, 15
    assert S.dataset_bytes(n, 2, m) >= 4 * S.n_indx(n, m)


def test_admission_is_fifo_and_within_budget():
    per = S.dataset_bytes(1000, 2, 15) + S.request_bytes(1000, 100, 2, 15)
    # the search scratch is transient (one search at a time): room for two requests exactly
    srv = bare_server(2 * per + S.search_bytes(1000, 15) + 1)
    for k in range(5):
        srv.submit(req(1000, 100, k))
    b = srv._admit()
    assert [r.rid for r, key, err in b] == [0, 1]
    assert srv.resident <= srv.budget
    assert [r.rid for r in srv.queue] == [2, 3, 4]


def test_oversized_request_rejected_and_queue_moves_on():
    one = S.dataset_bytes(1000, 2, 15) + S.request_bytes(1000, 100, 2, 15) + S.search_bytes(1000, 15)
    srv = bare_server(one)
    srv.submit(req(50000, 100, 0))
    srv.submit(req(1000, 100, 1))
    b = srv._admit()
    assert b[0][2] is not None and b[0][1] is None
    assert b[1][0].rid == 1 and b[1][2] is None
    assert srv.stats["rejected"] == 1


def test_shared_dataset_counted_once_and_idle_datasets_evicted():
    ds = S.dataset_bytes(1000, 2, 15)
    rq = S.request_bytes(1000, 100, 2, 15)
    assert ds > rq
    srv = bare_server(ds + 2 * rq + S.search_bytes(1000, 15))
    srv.submit(req(1000, 100, 0, dataset="A"))
    srv.submit(req(1000, 100, 1, dataset="A"))
    b = srv._admit()
    assert len(b) == 2 and srv.resident == ds + 2 * rq
    # retire the batch by hand: dataset A stays resident and idle
    srv.resident -= 2 * rq
    srv.datasets["A"] = S._Dataset(n=1000, nbytes=ds)
    srv.submit(req(1000, 100, 2, dataset="B"))
    b = srv._admit()
    assert len(b) == 1 and srv.stats["evictions"] == 1 and "A" not in srv.datasets


def test_busy_dataset_is_never_evicted():
    ds = S.dataset_bytes(1000, 2, 15)
    rq = S.request_bytes(1000, 100, 2, 15)
    srv = bare_server(ds + rq + S.search_bytes(1000, 15))
    srv.datasets["A"] = S._Dataset(n=1000, nbytes=ds, busy=1)
    srv.resident = ds
    srv.submit(req(1000, 100, 0, dataset="B"))
    assert srv._admit() == [] and "A" in srv.datasets


def test_summarize_percentiles():
    rs = [S.ConjResult(rid=k, arrival=0.0, done=0.01 * (k + 1), batch=k // 2) for k in range(10)]
    s = S.summarize(rs)
    assert s["completed"] == 10 and abs(s["p50_s"] - 0.055) < 1e-12
    assert s["iterations"] == 5 and s["mean_batch"] == 2.0
