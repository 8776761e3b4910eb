"""CPU oracle for crowddynamics_gb300 (test infrastructure only)."""
