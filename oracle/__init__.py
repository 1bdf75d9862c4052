"""CPU oracle of the per-thread ensemble solver (test infrastructure only)."""
