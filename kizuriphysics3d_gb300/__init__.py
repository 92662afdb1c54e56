"""GB300-native per-step contact pipeline of KizuriPhysics (PhysicsWorld::StepFixed).

Public surface:
  * ``scenes``  - seeded scene builders and the binary scene format
  * ``World``   - device-resident world over the C-ABI in include/kzg.h (libkzg.so)
  * ``resolve`` - host-side hull construction and mass properties
  * ``build``   - in-tree nvcc build of libkzg.so for sm_103a
"""
from . import build, capi, scenes  # noqa: F401
from .world import Resolved, World, build_hull, make_edit, resolve  # noqa: F401

__all__ = ["World", "Resolved", "resolve", "build_hull", "make_edit", "scenes", "build", "capi"]
