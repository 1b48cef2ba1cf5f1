"""Linear algebra of the GPU dense path (solver, preconditioners)."""
