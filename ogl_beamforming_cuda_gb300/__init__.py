"""GB300-native beamforming pipeline behind the ogl_beamformer_lib C ABI.

The product is the in-tree shared library lib/libogl_beamformer_lib.so (C++ host
code + sm_103a CUDA kernels, sources in csrc/). `abi` is its ctypes binding.
"""
from . import abi  # noqa: F401
