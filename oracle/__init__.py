"""CPU oracle for the coarsening hot path (test infrastructure only)."""
