"""The R package's .Call layer (src/): compiled against the project's R-API stand-in and
linked to the GB300 library, it registers the reference's routine table and refuses work
without a device.  CPU only; tests/test_gpu_rcall.py runs the routines on a GB300."""
import ctypes as C

import pytest

# The reference's .Call table (src/init.cpp:11-22) and the neighbor routines R/nn.R calls
# (src/nn.h:18,25,38): name -> number of arguments.
REFERENCE_TABLE = {"rNNGP": 28, "sNNGP": 29, "sNNGPLogit": 27, "cNNGP": 18, "cSLGP": 21, "rNNGPPredict": 17,
                   "sNNGPPredict": 19, "PGLogit": 9, "rNNGPReplicated": 14, "mkNNIndx": 7, "mkNNIndxCB": 7,
                   "mkUIndx": 8}


class CallMethodDef(C.Structure):
    _fields_ = [("name", C.c_char_p), ("fun", C.c_void_p), ("numArgs", C.c_int)]


@pytest.fixture(scope="module")
def rcall():
    from spnngp_gb300.build import build

    build()
    from oracle.oracle import RCALL_SO, build as build_oracle

    build_oracle(rcall=True)
    return C.CDLL(RCALL_SO)


def test_registration_table_matches_reference(rcall):
    rcall.R_init_spNNGP(None)
    rcall.shim_call_routines.restype = C.POINTER(CallMethodDef)
    tab = rcall.shim_call_routines()
    got = {}
    k = 0
    while tab[k].name:
        got[tab[k].name.decode()] = tab[k].numArgs
        assert tab[k].fun == C.cast(getattr(rcall, tab[k].name.decode()), C.c_void_p).value
        k += 1
    assert got == REFERENCE_TABLE


def test_out_of_scope_routine_raises(rcall):
    rcall.ref_last_error.restype = C.c_char_p
    rcall.ref_clear_error()
    rcall.PGLogit.restype = C.c_void_p
    rcall.PGLogit(*([None] * 9))
    assert b"not part of the GB300 build" in rcall.ref_last_error()


def test_no_device_is_an_error_not_a_fallback(rcall):
    import numpy as np
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible: the routine would run")
    from oracle.oracle import Reference, RCALL_SO

    lib = Reference(RCALL_SO)
    c = np.random.default_rng(0).uniform(size=(50, 2))
    nn, dist, lu, st = lib.mkNNIndxCB(np.ascontiguousarray(c.T).reshape(-1), 5)
    assert st != 0 and "device" in lib.error()
