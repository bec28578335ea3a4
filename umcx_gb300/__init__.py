"""umcx_gb300 - GB300 (sm_103a) photon-transport hot path of umcx behind the reference's JSON / C interfaces.

The compute path is libumcx_gb300.so (hand-written CUDA kernels + C ABI, include/umcx_gpu.h); this package holds
its Python binding and build script.
"""
from ._lib import LIB_PATH, Result, Sim, Tuning, load
from .api import Batch, Context, Forward, Job, autotune_batch, detp_columns, measure_peaks, seeds_from_rngseed

__all__ = ["LIB_PATH", "Result", "Sim", "Tuning", "load", "Batch", "Context", "Forward", "Job", "autotune_batch",
           "detp_columns", "measure_peaks", "seeds_from_rngseed"]
