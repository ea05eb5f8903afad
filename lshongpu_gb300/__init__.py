"""lshongpu_gb300: GB300-native k-NN / LSH engine (C++ host + sm_103a CUDA kernels).

The compute lives in liblshg.so (C ABI: include/lshg.h); this package is the Python
binding of that ABI, mirroring the reference's launch surface
(LinearScan/kernel.cu:27 linearScans, :91 LSH) plus the resident index and serving
loop.  Build the library with `python -m lshongpu_gb300.build`.
"""
from .api import *  # noqa: F401,F403
from .api import __all__  # noqa: F401
from ._lib import LshgError, SYMBOLS, lib, lib_path  # noqa: F401
