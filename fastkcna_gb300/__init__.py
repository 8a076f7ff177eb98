"""GB300-native (sm_103a) FastKCNA graph construction.

The CUDA library libkcna.so (C ABI: include/kcna.h) does the work; this
package holds its Python binding (kcna.py), the in-tree build recipe
(build.py) and the seeded dataset generator (synth.py).
"""
from . import synth  # noqa: F401

__all__ = ["synth", "kcna", "build"]
