"""CPU oracle of the GFM combustion-space iteration (test infrastructure only)."""
