"""GB300-native panoptic / semantic / instance segmentation evaluation.

Public API of AndyBarcia/panoptic-evaluator (``panoptic_evaluator/__init__.py``)
backed by the sm_103a kernels of ``libpe_gb300.so`` through its C ABI.
"""

from .evaluator import PanopticBatch, PanopticEvaluator, panoptic_quality

__all__ = [
    "PanopticBatch",
    "PanopticEvaluator",
    "panoptic_quality",
]
