"""GB300-native engine for GRANIITTI's event-weight path.

phase-space map -> Regge |M|^2 -> eikonal kt-loop screening -> VEGAS -> unweighting,
as hand-written sm_103a CUDA kernels behind a C ABI (include/graniitti_gb300.h).
"""
from . import _abi, card, modeldata  # noqa: F401
from .engine import FP64, MIXED, Batch, Engine, Flow, Graniitti  # noqa: F401

__all__ = ["Batch", "Engine", "Flow", "Graniitti", "FP64", "MIXED", "card", "modeldata"]
