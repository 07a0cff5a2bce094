"""CPU oracle and parity reference (test infrastructure only)."""
