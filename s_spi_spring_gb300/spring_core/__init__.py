"""Import path of the reference's compiled module: ``spring_core.phase_retrieval``
(reference ``src/wrapper.cpp:24-27``)."""
from . import phase_retrieval

__all__ = ["phase_retrieval"]
