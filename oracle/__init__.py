"""CPU oracle of the ELBM level step (test infrastructure, never the product)."""
