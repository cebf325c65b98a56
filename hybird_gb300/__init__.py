"""GB300-native (sm_103a) implementation of hybird's time-step hot path.

The product is the CUDA shared library ``_lib/libhybird_gpu.so`` behind the C-ABI in
``include/hybird_gpu.h``; :mod:`hybird_gb300.abi` mirrors its structs and
:mod:`hybird_gb300.gpu` wraps the calls for Python callers.
"""
from . import abi  # noqa: F401
