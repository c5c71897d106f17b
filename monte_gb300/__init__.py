"""GB300-native Monte hot paths: FDK reconstruction and photon Monte Carlo.

The compute lives in libmonte.so (CUDA for sm_103a behind the C ABI in
include/monte.h); this package loads it and gives Python callers the same
entry points.
"""
from .abi import *  # noqa: F401,F403
