"""GB300-native Krylov linear-solver core for T-FlowS (CG / BiCG / CGS + Prec1)."""
from . import mesh  # noqa: F401
