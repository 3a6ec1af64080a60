"""CPU oracle of the path-tracing integrator (test infrastructure only)."""
