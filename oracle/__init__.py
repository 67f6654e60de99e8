"""CPU oracle for the finite-difference hot path (test infrastructure only)."""
