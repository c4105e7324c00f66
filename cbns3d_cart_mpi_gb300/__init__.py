"""GB300-native (sm_103a) right-hand side of the cbns3d compressible
Navier-Stokes solver, reached through the C ABI in ``include/cbns_gpu.h``."""
from ._abi import CbnsParams, tgv_params  # noqa: F401

__version__ = "0.1.0"
