"""GB300-native kinetic 2D Delaunay engine (move -> untangle -> Lawson flips ->
one-ring / fixed-radius neighbour queries) behind the reference's
HostTriangulation / DeviceTriangulation / GridCount2d call surface.

The compute lives in libmcl_gb300.so (hand-written CUDA for sm_103a, C ABI in
include/mcl_gb300.h); this package is its Python binding.
"""
from ._lib import McleapError, lib  # noqa: F401
from .batch import MeshBatch  # noqa: F401
from .periodic import PeriodicTriangulation  # noqa: F401
from .triangulation import DeviceTriangulation, GridCount2d, HostTriangulation  # noqa: F401

__all__ = ["HostTriangulation", "DeviceTriangulation", "GridCount2d", "MeshBatch", "McleapError", "lib"]
