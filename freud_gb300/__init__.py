"""freud_gb300: GB300-native (sm_103a) neighbour-query -> pair-reduction path with
the freud API: freud.box, freud.locality (AABBQuery, LinkCell, NeighborList),
freud.density.RDF and freud.order.Steinhardt. Importing this package loads the
CUDA library; there is no CPU fallback.
"""

from . import box, data, density, locality, order, parallel, replicas
from .box import Box
from .locality import AABBQuery, CellQuery, FrameBatch, LinkCell, NeighborList

__version__ = "0.1.0"

__all__ = ["__version__", "box", "data", "density", "locality", "order", "parallel", "Box", "AABBQuery", "LinkCell",
           "NeighborList"]
