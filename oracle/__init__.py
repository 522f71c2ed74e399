"""CPU oracle of the batched simulation step (test infrastructure: the checker, never the product)."""
