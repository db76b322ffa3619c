"""Boundary conditions of the drop-in API (finite_elements/conditions.py)."""
from __future__ import annotations


class BoundaryCondition:
    """Prescribed ``value`` of 1-based ``dimension`` on ``application``
    (conditions.py:11-58)."""

    def __init__(self, application, value: float, dimension, name: str = ''):
        self.application = application
        self.value = value
        self.dimension = dimension
        self.name = name

    def c_matrix(self):
        return (1, 1)

    def source_c_matrix(self):
        return self.value


class NodeBoundaryCondition(BoundaryCondition):
    """On a node (conditions.py:61-107)."""


class EdgeBoundaryCondition(BoundaryCondition):
    """On both end nodes of an edge, half the value each in the analysis
    (conditions.py:110-150, analysis.py:222-239)."""

    def to_node_boundary_condition(self):
        return [NodeBoundaryCondition(p, self.value, self.dimension)
                for p in (self.application.start, self.application.end)]


class ElementBoundaryCondition(BoundaryCondition):
    """On the three nodes of an element, weighted by element_to_node_factors in the
    analysis (conditions.py:153-193, analysis.py:201-220)."""

    def to_node_boundary_condition(self):
        return [NodeBoundaryCondition(p, self.value, self.dimension)
                for p in self.application.points]


class ContinuityCondition:
    """Periodic (value 1) or anti-periodic (value -1) link of two nodes,
    A(node1) = value * A(node2) (conditions.py:196-241); one multiplier row in the
    analysis (analysis.py:175-199)."""

    def __init__(self, node1, node2, value):
        self.node1 = node1
        self.node2 = node2
        self.value = value

    def c_matrix(self):
        return (1, 1, -self.value, -self.value)

    def source_c_matrix(self):
        return ()
