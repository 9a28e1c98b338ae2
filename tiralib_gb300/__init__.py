"""tiralib_gb300: tiralib's tensor-voting path (structure tensor, 2D/3D
stick / plate / ball voting, batched symmetric eigendecomposition) as
hand-written sm_103a CUDA behind a C ABI (include/tvgb.h, libtvgb.so)."""
from .api import *  # noqa: F401,F403
from ._lib import TvgbError, lib  # noqa: F401

__version__ = "0.1.0"
