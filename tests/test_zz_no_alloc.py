"""nngp_loglik_gram_noalloc: the FP64 fused likelihood pass for callers that cannot
allocate device memory (its scratch is a static device array in the library).  It
is called through the C ABI and must give the same log-determinant and Gram as
the allocating entry point nngp_loglik_gram_dev, on two calls in a row (the
shared array keeps the previous call's contents).  This file is collected last."""
import ctypes as C

import numpy as np
import pytest

from conftest import cm, xorder

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same FP64 kernel and reduction order: the results agree to rounding


def _setup(n, m, seed):
    import torch

    from oracle.oracle import Oracle, build

    build()
    orc = Oracle()
    rng = np.random.default_rng(seed)
    c = xorder(rng.uniform(size=(n, 2)))
    nn, _, lu = orc.mkNNIndxCB(cm(c), m)
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = X @ [1.0, -0.5] + rng.normal(size=n)
    V = np.column_stack([X, y])
    dev = torch.device("cuda", 0)
    t = dict(c=torch.from_numpy(cm(c)).to(dev), nn=torch.from_numpy(nn).to(dev), lu=torch.from_numpy(lu).to(dev),
             V=torch.from_numpy(cm(V)).to(dev))
    return t, V.shape[1]


def _lib():
    from spnngp_gb300.build import build

    return C.CDLL(build())


def _fn(lib):
    f = lib.nngp_loglik_gram_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                  C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    return f


def _noalloc(lib, t, n, m, nv, model, theta):
    import torch

    f = _fn(lib)
    ld = torch.zeros(1, dtype=torch.float64, device="cuda")
    G = torch.zeros(nv * nv, dtype=torch.float64, device="cuda")
    th = np.array(list(theta) + [0.0] * (4 - len(theta)))
    err = C.create_string_buffer(256)
    st = f(None, n, m, nv, t["c"].data_ptr(), t["nn"].data_ptr(), t["lu"].data_ptr(), t["V"].data_ptr(), model,
           th.ctypes.data_as(C.POINTER(C.c_double)), ld.data_ptr(), G.data_ptr(), err, 256)
    return st, ld.item(), G.cpu().numpy().reshape(nv, nv), err.value.decode()


def _alloc(t, n, m, nv, model, theta):
    import torch

    from spnngp_gb300._lib import Context, _dp

    ctx = Context(0)
    ld = torch.zeros(1, dtype=torch.float64, device="cuda")
    G = torch.zeros(nv * nv, dtype=torch.float64, device="cuda")
    th = np.array(list(theta) + [0.0] * (4 - len(theta)))
    torch.cuda.synchronize()  # the context runs on its own stream, not torch's
    ctx.call("nngp_loglik_gram_dev", n, m, nv, t["c"].data_ptr(), t["nn"].data_ptr(), t["lu"].data_ptr(),
             t["V"].data_ptr(), model, th.ctypes.data_as(_dp), 0, ld.data_ptr(), G.data_ptr())
    out = (ld.item(), G.cpu().numpy().reshape(nv, nv))
    ctx.close()
    return out


@pytest.mark.parametrize("n,m,model,theta", [(3000, 15, 0, (1.0, 0.1, 6.0)), (5000, 32, 2, (1.0, 0.2, 9.0, 1.5)),
                                             # 1875 tiles of 32 locations: two reduction chunks of 1024 tiles
                                             (60000, 32, 0, (1.0, 0.1, 6.0))])
def test_noalloc_matches_allocating_pass_twice(n, m, model, theta):
    lib = _lib()
    t, nv = _setup(n, m, n + m)
    ld_ref, G_ref = _alloc(t, n, m, nv, model, theta)
    for _ in range(2):  # the second call must not see stale contents of the shared array
        st, ld, G, err = _noalloc(lib, t, n, m, nv, model, theta)
        assert st == 0, err
        assert abs(ld - ld_ref) <= TOL * abs(ld_ref)
        assert np.max(np.abs(G - G_ref)) <= TOL * np.max(np.abs(G_ref))


def test_noalloc_rejects_oversized_requests():
    lib = _lib()
    t, nv = _setup(3000, 15, 1)
    f = _fn(lib)
    err = C.create_string_buffer(256)
    th = np.array([1.0, 0.1, 6.0, 0.0])
    st = f(None, 70000, 15, nv, t["c"].data_ptr(), t["nn"].data_ptr(), t["lu"].data_ptr(), t["V"].data_ptr(), 0,
           th.ctypes.data_as(C.POINTER(C.c_double)), None, None, err, 256)
    assert st == 1 and b"65536" in err.value


def test_noalloc_allocates_no_device_memory():
    """Once warm, calls leave the device's free memory and torch's pool unchanged."""
    import torch

    lib = _lib()
    n, m, model, theta = 20000, 15, 0, (1.0, 0.1, 6.0)
    t, nv = _setup(n, m, 5)
    ld = torch.zeros(1, dtype=torch.float64, device="cuda")
    G = torch.zeros(nv * nv, dtype=torch.float64, device="cuda")
    th = np.array(list(theta) + [0.0])
    err = C.create_string_buffer(256)
    f = _fn(lib)
    args = (None, n, m, nv, t["c"].data_ptr(), t["nn"].data_ptr(), t["lu"].data_ptr(), t["V"].data_ptr(), model,
            th.ctypes.data_as(C.POINTER(C.c_double)), ld.data_ptr(), G.data_ptr(), err, 256)
    assert f(*args) == 0, err.value  # warm: the array's address is looked up, the kernels are loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        assert f(*args) == 0, err.value
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_refuses_stream_capture():
    """A call on a stream that is being captured returns NNGP_ERR_ARG and enqueues nothing."""
    import torch

    lib = _lib()
    n, m = 3000, 15
    t, nv = _setup(n, m, 9)
    ld = torch.zeros(1, dtype=torch.float64, device="cuda")
    G = torch.zeros(nv * nv, dtype=torch.float64, device="cuda")
    th = np.array([1.0, 0.1, 6.0, 0.0])
    err = C.create_string_buffer(256)
    f = _fn(lib)
    assert f(None, n, m, nv, t["c"].data_ptr(), t["nn"].data_ptr(), t["lu"].data_ptr(), t["V"].data_ptr(), 0,
             th.ctypes.data_as(C.POINTER(C.c_double)), ld.data_ptr(), G.data_ptr(), err, 256) == 0
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
            ld.add_(0.0)
            st = f(C.c_void_p(side.cuda_stream), n, m, nv, t["c"].data_ptr(), t["nn"].data_ptr(), t["lu"].data_ptr(),
                   t["V"].data_ptr(), 0, th.ctypes.data_as(C.POINTER(C.c_double)), ld.data_ptr(), G.data_ptr(), err,
                   256)
    assert st == 1 and b"captured" in err.value
