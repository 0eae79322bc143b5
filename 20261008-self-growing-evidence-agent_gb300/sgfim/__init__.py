"""sgfim -- GB300-native exact maximal-frequent-itemset mining.

The compute lives in libsgfim.so (hand-written CUDA for sm_103a behind a C
ABI, include/sgfim.h); this package binds it with ctypes and mirrors the
reference's engine adapter (code/pipeline/engine_adapter.py).
"""
__version__ = "0.1.0"
