"""Plain per-individual cuFFT path used as the GPU baseline of bench.py
(measurement infrastructure; not part of the engine)."""
