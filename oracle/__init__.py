"""CPU oracle for parity tests (test infrastructure only)."""
