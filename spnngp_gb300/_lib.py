"""ctypes binding of libspnngp_gb300.so (the C ABI declared in include/spnngp_gb300.h).

There is no CPU implementation behind this module: if the library is missing or
no GB300 is usable, calls raise.  Arrays are passed as numpy buffers
(host entry points) or as raw device pointers (``*_dev`` entry points).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libspnngp_gb300.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_i64 = C.c_int64

# status codes (include/spnngp_gb300.h)
NNGP_OK, NNGP_ERR_ARG, NNGP_ERR_CUDA, NNGP_ERR_NOT_SPD, NNGP_ERR_NO_MEMORY, NNGP_ERR_STREAM = range(6)
FP64, FP32R = 0, 1

_SIGNATURES = {
    "nngp_create": (_i, [_i, C.POINTER(_vp)]),
    "nngp_destroy": (None, [_vp]),
    "nngp_error_message": (C.c_char_p, [_vp]),
    "nngp_error_location": (_i64, [_vp]),
    "nngp_set_stream": (_i, [_vp, _vp]),
    "nngp_get_stream": (_vp, [_vp]),
    "nngp_synchronize": (_i, [_vp]),
    "nngp_launch_count": (_i64, [_vp]),
    "nngp_reset_launch_count": (None, [_vp]),
    "nngp_max_neighbors": (_i, []),
    "nngp_n_indx": (_i64, [_i, _i]),
    "nngp_mkNNIndxCB": (_i, [_vp, _i, _i, _dp, _ip, _dp, _ip]),
    "nngp_mkNNIndx": (_i, [_vp, _i, _i, _dp, _ip, _dp, _ip]),
    "nngp_mkUIndx": (_i, [_vp, _i, _i, _ip, _ip, _ip, _ip, _ip, _i]),
    "nngp_nn2": (_i, [_vp, _i, _dp, _i, _dp, _i, _ip, _dp]),
    "nngp_updateBF": (_i, [_vp, _i, _i, _dp, _ip, _ip, _i, _dp, _i, _dp, _dp, _dp]),
    "nngp_updateConjBF": (_i, [_vp, _i, _i, _dp, _ip, _ip, _i, _d, _d, _d, _i, _dp, _dp]),
    "nngp_Q": (_i, [_vp, _dp, _dp, _dp, _dp, _i, _ip, _ip, _dp]),
    "nngp_loglik_gram": (_i, [_vp, _i, _i, _i, _dp, _ip, _ip, _dp, _i, _dp, _i, _dp, _dp]),
    "nngp_rNNGP": (_i, [_vp, _dp, _dp, _i, _i, _i, _dp, _i, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                        _i, _i, _ip, _dp, _i64, _dp, _i64, _i, _dp, _dp, _dp, _ip]),
    "nngp_cNNGP": (_i, [_vp, _dp, _dp, _i, _i, _dp, _dp, _ip, _ip, _dp, _dp, _i, _ip, _i, _i, _dp, _i, _i,
                        _dp, _dp, _dp, _dp, _dp, _dp]),
    "nngp_rNNGPPredict": (_i, [_vp, _dp, _dp, _dp, _i, _i, _i, _dp, _dp, _i, _ip, _dp, _dp, _i, _i, _dp, _i,
                               _dp]),
    "nngp_rNNGPReplicated": (_i, [_vp, _dp, _i, _i, _i, _dp, _i, _ip, _ip, _dp, _dp, _i, _dp, _i, _dp]),
    "nngp_conj_posterior_samples": (_i, [_vp, _i, _dp, _dp, _d, _d, _d, _i, _dp, _dp, _dp]),
    # device-resident variants: every array argument is a device pointer (theta stays on the host)
    "nngp_updateBF_dev": (_i, [_vp, _i, _i, _vp, _vp, _vp, _i, _dp, _i, _vp, _vp, _vp]),
    "nngp_loglik_gram_dev": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _i, _dp, _i, _vp, _vp]),
    "nngp_mkNNIndxCB_dev": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp]),
    "nngp_nn2_dev": (_i, [_vp, _i, _vp, _i, _vp, _i, _vp, _vp]),
    "nngp_measure_peak": (_i, [_vp, _i, _dp]),
    "nngp_cNNGP_multi": (_i, [_vp, _i, _vp, _i, _i, _dp, _i, _i, _i]),
    "nngp_rNNGP_batch": (_i, [_vp, _i, _vp, _i, _i, _i]),
    "nngp_set_kernel_timing": (_i, [_vp, _i]),
    "nngp_kernel_time": (_i, [_vp, _dp, C.POINTER(_i64)]),
    "nngp_fp32r_resolved": (_i, [_vp, C.POINTER(_i64), C.POINTER(_i64)]),
    "nngp_fp32r_tiers": (_i, [_vp, C.POINTER(_i64), C.POINTER(_i64)]),
    "nngp_set_autotune": (_i, [_vp, _i]),
    "nngp_set_launch_shape": (_i, [_vp, _i, _i, _i]),
    "nngp_autotune_report": (_i, [_vp, C.c_char_p, _i]),
}


class ConjProblem(C.Structure):
    """nngp_conj_problem (include/spnngp_gb300.h): one dataset of a batched conjugate run."""

    _fields_ = [("n", C.c_int), ("n0", C.c_int), ("g", C.c_int)] + [
        (name, C.c_void_p) for name in ("y", "X", "coords", "nnIndx", "nnIndxLU", "X0", "coords0", "nnIndx0",
                                        "thetaAlpha", "y0True", "betaHat", "ab", "bBInv", "bb", "y0Hat",
                                        "y0HatVar", "crps", "rmspe")]


class MCMCProblem(C.Structure):
    """nngp_mcmc_problem (include/spnngp_gb300.h): one chain of a batched response-model run."""

    _fields_ = [("n", C.c_int), ("m", C.c_int), ("covModel", C.c_int), ("nSamples", C.c_int)] + [
        (name, C.c_void_p) for name in ("y", "X", "coords", "nnIndx", "nnIndxLU", "sigmaSqIG", "tauSqIG", "phiUnif",
                                        "nuUnif", "betaStarting", "thetaStarting", "tuning", "normals")] + [
        ("nNormals", C.c_int64), ("unifs", C.c_void_p), ("nUnifs", C.c_int64), ("betaSamples", C.c_void_p),
        ("thetaSamples", C.c_void_p), ("nAccept", C.c_int)]


class NNGPError(RuntimeError):
    """A non-zero status from the library; ``location`` is the failing location or -1."""

    def __init__(self, status: int, message: str, location: int = -1):
        super().__init__(f"[status {status}] {message}")
        self.status = status
        self.location = location


class _Lib:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            raise ImportError(
                f"{path} is not built; build it with `python -m spnngp_gb300.build` (requires nvcc)")
        self.path = path
        self.cdll = C.CDLL(path)
        self._fns = {}

    def fn(self, name: str):
        f = self._fns.get(name)
        if f is None:
            f = getattr(self.cdll, name)
            res, args = _SIGNATURES[name]
            f.restype = res
            f.argtypes = args
            self._fns[name] = f
        return f


_LIB = None
_LIB_LOCK = threading.Lock()


def lib() -> _Lib:
    global _LIB
    with _LIB_LOCK:
        if _LIB is None:
            _LIB = _Lib()
        return _LIB


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One library context (device, stream, scratch).  Not thread-safe; use one per thread."""

    def __init__(self, device: int = 0):
        self._lib = lib()
        h = _vp()
        st = self._lib.fn("nngp_create")(device, C.byref(h))
        if st != NNGP_OK:
            raise NNGPError(st, f"could not create a context on CUDA device {device} (no usable GB300?)")
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self._lib.fn("nngp_destroy")(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name: str, *args) -> int:
        st = self._lib.fn(name)(self.handle, *args)
        if st != NNGP_OK:
            msg = self._lib.fn("nngp_error_message")(self.handle)
            loc = self._lib.fn("nngp_error_location")(self.handle)
            raise NNGPError(st, (msg or b"").decode(), int(loc))
        return st

    def set_stream(self, stream_handle: int | None):
        """Launch on this cudaStream_t handle; None = the context's own (non-blocking) stream.

        Handle 0 is CUDA's legacy default stream (torch's default stream), which the C ABI cannot
        name (NULL selects the context's own stream): work on it would not be ordered with this
        library's.  Share a torch.cuda.Stream() instead."""
        if stream_handle is not None and int(stream_handle) == 0:
            raise ValueError("stream handle 0 (the legacy default stream) cannot be shared with the library; "
                             "use a torch.cuda.Stream() (and make it current) or None for the context's own stream")
        self._lib.fn("nngp_set_stream")(self.handle, stream_handle)

    def synchronize(self):
        self.call("nngp_synchronize")

    @property
    def launches(self) -> int:
        return int(self._lib.fn("nngp_launch_count")(self.handle))

    def reset_launches(self):
        self._lib.fn("nngp_reset_launch_count")(self.handle)

    def set_autotune(self, on: bool):
        self.call("nngp_set_autotune", 1 if on else 0)

    def set_launch_shape(self, warps_per_block: int, grid_mode: int = 0, tmem: bool = False):
        """Forces the FP32R register kernel's launch shape (warps_per_block 0: autotune again);
        tmem selects the variant keeping the covariance's low-order parts in tensor memory."""
        self.call("nngp_set_launch_shape", int(warps_per_block), int(grid_mode), 1 if tmem else 0)

    def fp32r_tiers(self) -> tuple[int, int]:
        """(re-solved in double-float, re-solved in FP64) of the last single-dataset FP32R pass."""
        a, b = _i64(), _i64()
        self.call("nngp_fp32r_tiers", C.byref(a), C.byref(b))
        return int(a.value), int(b.value)

    def fp32r_resolved(self) -> tuple[int, int]:
        """(locations re-solved in higher precision -- double-float or FP64 --, locations covered)
        of the last single-dataset FP32R pass."""
        r, n = _i64(), _i64()
        self.call("nngp_fp32r_resolved", C.byref(r), C.byref(n))
        return int(r.value), int(n.value)

    def autotune_report(self) -> dict:
        """Tuned launch shapes: {class: {"wpb", "grid_mode", "tmem", "ms", "candidates": {"WxBLOCKS[t]": ms}}}."""
        buf = C.create_string_buffer(1 << 16)
        self._lib.fn("nngp_autotune_report")(self.handle, buf, len(buf))
        out = {}
        for line in buf.value.decode().splitlines():
            head, _, cands = line.partition(" | ")
            key, _, rest = head.partition(": ")
            kv = dict(t.split("=") for t in rest.split())
            out[key] = {"wpb": int(kv["wpb"]), "grid_mode": int(kv["grid_mode"]), "tmem": int(kv["tmem"]),
                        "ms": float(kv["ms"]),
                        "candidates": {c.split(":")[0]: float(c.split(":")[1]) for c in cands.split()}}
        return out


_DEFAULT = None


def default_context() -> Context:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


def n_indx(n: int, m: int) -> int:
    return int((1 + m) / 2 * m + (n - m - 1) * m)
