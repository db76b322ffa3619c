"""Load objects of the drop-in API (finite_elements/loads.py).

ElementsLoad keeps the total value; its area split (loads.py:32-34) and the element
to node factors are computed on the device during assembly."""
from __future__ import annotations


class ElementsLoad:
    """A total ``value`` spread over ``elements`` in proportion to their areas,
    applied in 1-based ``dimension`` (loads.py:13-35)."""

    def __init__(self, elements, value: float, dimension: int):
        self.elements = list(elements)
        self.value = value
        self.dimension = dimension


class ElementLoad:
    """One element's load (loads.py:38-56); not used by the analysis."""

    def __init__(self, element, value: float, dimension: int):
        self.element = element
        self.value = value
        self.dimension = dimension


class EdgeLoad:
    """Half of ``value`` to each end node of ``edge`` (loads.py:59-69,
    analysis.py:431-447)."""

    def __init__(self, edge, value, dimension):
        self.edge = edge
        self.value = value
        self.dimension = dimension


class NodeLoad:
    """``value`` on node ``node`` in 1-based ``dimension`` (loads.py:72-102)."""

    def __init__(self, node, value: float, dimension):
        self.node = node
        self.value = value
        self.dimension = dimension

    def c_matrix(self):
        return ()

    def source_c_matrix(self):
        return self.value


class MagnetLoad:
    """Magnetisation load (loads.py:105-147).  Not part of the GPU path: an analysis
    given one raises NotImplementedError."""

    def __init__(self, elements, non_contour_nodes, magnetization_vector):
        self.elements = elements
        self.non_contour_nodes = non_contour_nodes
        self.magnetization_vector = magnetization_vector
