"""CPU oracle (test infrastructure)."""
