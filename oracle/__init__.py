"""CPU oracle of the level-set hot path (test infrastructure only; see oracle.py)."""
from .oracle import Oracle, Problem, SampleOracle, build_port, build_ref, ref_available  # noqa: F401
