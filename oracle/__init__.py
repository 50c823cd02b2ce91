"""CPU oracle of the phase-retrieval path: test infrastructure only."""
