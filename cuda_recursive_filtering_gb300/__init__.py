"""GB300 (sm_103a) cascaded-biquad IIR filtering.

Drop-in for the filtering path of Haotian-RA/cuda_recursive_filtering: the four
realizations PH, STCR (loop / unrolled), DTCR (loop / unrolled) and PLR, selectable with
their BLOCK_SIZE x N_BLOCKS geometry, each a single persistent launch with a
launch-versioned decoupled lookback. The compute path is libiir_gb300.so (C ABI in
include/iir_gb300.h); this package is its Python host mirror.
"""
from ._lib import KERNELS, IirError, load as load_library
from .api import Batch, Plan, PlrPlan, sosfilt

__all__ = ["Plan", "PlrPlan", "Batch", "sosfilt", "KERNELS", "IirError", "load_library"]
__version__ = "1.0.0"
