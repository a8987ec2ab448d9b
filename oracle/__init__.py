"""CPU oracle of the reference's single-rank step (test infrastructure only)."""
