"""CPU oracle of the radiance-cascade path (test infrastructure only)."""
