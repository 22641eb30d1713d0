"""FP64 CPU oracle of the MPM substep (test infrastructure only)."""
