"""GB300-native panoptic / semantic / instance segmentation evaluation.

Public API of AndyBarcia/panoptic-evaluator (``panoptic_evaluator/__init__.py``)
backed by the sm_103a kernels of ``libpe_gb300.so`` through its C ABI.
"""

from .evaluator import PanopticBatch, PanopticEvaluator, panoptic_quality
from .instance import InstanceBatch, InstanceEvaluator
from .combined import SegmentationEvaluator
from .prefix import segmentation_prefixes

__all__ = [
    "PanopticBatch",
    "PanopticEvaluator",
    "panoptic_quality",
    "InstanceBatch",
    "InstanceEvaluator",
    "SegmentationEvaluator",
    "segmentation_prefixes",
]
