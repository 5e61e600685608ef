"""CPU oracle for the upwind advection hot path (test infrastructure only)."""
from .oracle import Port, Reference, build, cfl_dt, reference_dt  # noqa: F401
