"""CPU oracle of the surface Green's-function path: test infrastructure only."""
