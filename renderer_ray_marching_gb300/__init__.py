"""GB300-native renderer hot path: exact nearest-neighbour radii, culling and
the sphere-tracing marcher of Auratons/renderer_ray_marching, as hand-written
CUDA for sm_103a behind the C ABI in ``include/rm.h``.

``Renderer`` (``renderer.py``) is the Python front end of that ABI,
``synthetic`` generates seeded scenes and views, ``autograd`` wraps the
forward and backward kernels in a ``torch.autograd.Function``.
"""
from .renderer import Renderer, View, views_from_specs  # noqa: F401

__all__ = ["Renderer", "View", "views_from_specs"]
