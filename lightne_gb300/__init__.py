"""lightne_gb300 — GB300-native (sm_103a) LightNE embedding pipeline.

The compute path is the CUDA library liblightne_gb300.so behind the C ABI in
include/lightne_gb300.h; this package is its Python host mirror.
"""
from ._lib import LneError, load  # noqa: F401

__version__ = "0.1.0"
