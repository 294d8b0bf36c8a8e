"""CPU oracle for the symmetry-reduced H*x path (test infrastructure only; never imported by the product)."""
