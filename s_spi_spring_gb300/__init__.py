"""GB300-native phase-retrieval engine for SPRING (memetic phase retrieval for
single-shot coherent diffraction imaging).

The hot path -- HIO / RAAR / ER iterations with the masked modulus projection,
shrink-wrap, error metrics -- runs as fused sm_103a kernels behind the C ABI
of ``include/spe_engine.h``.  ``phase_retrieval`` mirrors the reference's
``spring_core.phase_retrieval`` Python API on top of it.
"""
from . import _lib
from .phase_retrieval import Reconstruction, Solver

__all__ = ["Reconstruction", "Solver", "_lib"]
