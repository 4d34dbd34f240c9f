"""freud_gb300: GB300-native (sm_103a) neighbour-query -> pair-reduction path with
the freud API: freud.box, freud.locality (AABBQuery, LinkCell, CellQuery,
NeighborList), freud.density.RDF / CorrelationFunction, freud.order.Steinhardt
and freud.pmft, plus batched frames (FrameBatch), a GSD trajectory reader (gsd)
and multi-process RDF states (replicas). Importing this package loads the CUDA
library; there is no CPU fallback.
"""

from . import box, data, density, gsd, locality, order, parallel, pmft, replicas
from .box import Box
from .locality import AABBQuery, CellQuery, FrameBatch, LinkCell, NeighborList

__version__ = "0.1.0"

__all__ = ["__version__", "box", "data", "density", "gsd", "locality", "order", "parallel", "pmft", "replicas", "Box",
           "AABBQuery", "CellQuery", "FrameBatch", "LinkCell", "NeighborList"]
