"""Import path of the reference's compiled module: ``spring_core.phase_retrieval``,
``spring_core.pattern`` and ``spring_core.GPUtils`` (reference
``src/wrapper.cpp:24-27, 318, 459-484``).  ``phase_retrieval`` is the
package's own Solver / Reconstruction module, registered under this path."""
import sys

from .. import phase_retrieval
from . import GPUtils, pattern

sys.modules[__name__ + ".phase_retrieval"] = phase_retrieval

__all__ = ["GPUtils", "pattern", "phase_retrieval"]
