"""ffsrl: GB300-native multi-environment soft-tissue step, BVH refit and ray-cast.

Public classes keep the reference's names (``FF_SRL/FF_SRL/__init__.py:1-6``):
``SimModelDO``, ``SimIntegratorDO``, ``SimBVH``, ``WarpRaycastRendererDO``; ``SimCutting``
holds the cutting and heating state the reference keeps per simMesh.
"""

from . import meshgen
from ._lib import FFSRLError
from .model import SimModelDO
from .integrator import SimIntegratorDO, BatchPlan
from .bvh import SimBVH
from .render import RenderMode, WarpRaycastRendererDO, quat_rpy, look_at_rotation
from .cutting import SimCutting

__all__ = ["SimModelDO", "SimIntegratorDO", "BatchPlan", "SimBVH", "WarpRaycastRendererDO", "RenderMode", "meshgen",
           "FFSRLError", "quat_rpy", "look_at_rotation", "SimCutting"]
