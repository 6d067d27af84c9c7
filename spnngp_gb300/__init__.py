"""spnngp_gb300: the response / conjugate NNGP hot path of the R package spNNGP,
rebuilt for one NVIDIA GB300 (sm_103a).

The compute runs in libspnngp_gb300.so (CUDA, built in-tree by
``spnngp_gb300.build``); this package is the host side that mirrors the
reference's R entry points.  Importing it does not touch the GPU; the first
call that needs the library loads it and raises if it is missing.
"""
from ._lib import FP32R, FP64, Context, NNGPError, default_context, lib  # noqa: F401
from .core import (COV_MODELS, Q, cNNGP, cNNGP_multi, rNNGP_batch, cov_model_index, loglik_gram, mkNNIndx, mkNNIndxCB,  # noqa: F401
                   mkUIndx, nn2, rNNGP, rNNGPPredict, rNNGPReplicated, updateBF, updateConjBF)

__version__ = "0.1.0"
