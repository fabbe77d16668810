"""CPU oracle for the pressure-Poisson path (test infrastructure only)."""
