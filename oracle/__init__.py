"""CPU oracle for the tall-skinny products: test infrastructure only (see oracle.h)."""
