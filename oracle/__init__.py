"""CPU oracle of the reference algorithm: test infrastructure only (see oracle.h)."""
