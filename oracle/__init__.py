"""CPU oracle package (test infrastructure only; never on the product path)."""
