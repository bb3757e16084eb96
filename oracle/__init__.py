"""CPU oracle of the reference algorithm (test infrastructure only)."""
