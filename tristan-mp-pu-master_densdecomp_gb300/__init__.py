"""GB300-native TRISTAN-MP hot path: host side.

The compute path lives in ``csrc/`` (CUDA for sm_103a behind the C-ABI
declared in ``include/tristan_gpu.h``). This package holds the host-side
mirror of the reference's per-step subroutines (``gpu.py``), the run
configuration the reference derives from its ``input`` file
(``config.py``), seeded synthetic loaders (``setups.py``) and the build
recipe (``build.py``).
"""
from .config import SimConfig  # noqa: F401
from . import setups  # noqa: F401
