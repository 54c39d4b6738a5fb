"""GB300 renderer core for the anari-visionaray raycast / pathtracer hot path.

libvsr.so (built by build.py) holds the CUDA kernels and the C ABI of
include/vsr.h; vsr.py binds it; scenes.py generates the benchmark scenes.
"""
from . import vsr, scenes  # noqa: F401
