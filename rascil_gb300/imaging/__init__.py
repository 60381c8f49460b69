"""RASCIL-facing imaging functions backed by the GB300 gridder."""
from .ng import invert_ng, predict_ng, invert_gb, predict_gb  # noqa: F401
from .imaging import invert_blockvisibility, predict_blockvisibility  # noqa: F401
from .weighting import weight_visibility, weight_blockvisibility  # noqa: F401
