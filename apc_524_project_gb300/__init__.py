"""GB300-native EMOOPIC per-timestep PIC loop (C ABI in include/emoo.h).

`abi` loads the native library libemoo.so (CUDA kernels for sm_103a plus the
host-side ABI); `configs` builds run configurations; `sim` is the Python view
of the reference's class API on top of the ABI.
"""
from . import abi, configs  # noqa: F401

__all__ = ["abi", "configs"]
