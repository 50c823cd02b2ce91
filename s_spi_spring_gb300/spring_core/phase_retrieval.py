"""``spring_core.phase_retrieval``: Solver and Reconstruction (reference
``src/wrapper.cpp:28-312``)."""
from ..phase_retrieval import Reconstruction, Solver, parse_algorithm

__all__ = ["Reconstruction", "Solver", "parse_algorithm"]
