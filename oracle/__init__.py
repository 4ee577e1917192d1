"""CPU FP64 oracle of the IMEX-DG hot path (test infrastructure only)."""
