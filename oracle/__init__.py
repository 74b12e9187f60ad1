"""CPU oracle of the preconditioned-Krylov path (test infrastructure only)."""
