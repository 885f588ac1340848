"""costal_gb300 — a GB300-native (sm_103a) exact cosine kNN graph for CosTaL 2.1.0.

`costal_gb300._costal` is a drop-in for the reference's `costal._costal` extension; the kernels live
in libcostal_gb300.so (costal_gb300/csrc/, C ABI in include/costal_gb300.h).
"""

from . import _costal
from ._costal import __version__

__all__ = ["_costal", "__version__"]
