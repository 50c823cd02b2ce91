"""Import path of the reference's compiled module: ``spring_core.phase_retrieval``,
``spring_core.pattern`` and ``spring_core.GPUtils`` (reference
``src/wrapper.cpp:24-27, 318, 459-484``)."""
from . import GPUtils, pattern, phase_retrieval

__all__ = ["GPUtils", "pattern", "phase_retrieval"]
