"""Import path of the reference's compiled module: ``spring_core.phase_retrieval``
and ``spring_core.pattern`` (reference ``src/wrapper.cpp:24-27, 318``)."""
from . import pattern, phase_retrieval

__all__ = ["pattern", "phase_retrieval"]
