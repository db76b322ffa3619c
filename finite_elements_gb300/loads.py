"""Load objects of the drop-in API (finite_elements/loads.py).

ElementsLoad keeps the total value; its area split (loads.py:32-34) and the element
to node factors are computed on the device during assembly."""
from __future__ import annotations

import numpy as np


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
    """Magnetisation load (loads.py:105-147): the equivalent surface current of a magnet
    made of the triangles ``elements``, with magnetisation ``magnetization_vector``.
    Every edge of the magnet's contour (an edge of one of its triangles only, unless
    both its points are ``non_contour_nodes``) adds (M . t) L / 2 to the right-hand
    side at both its points, t the edge's interior normal turned by +90 degrees and L
    its length (analysis.py:556-577)."""

    def __init__(self, elements, non_contour_nodes, magnetization_vector):
        self.elements = elements
        self.non_contour_nodes = non_contour_nodes
        self.magnetization_vector = magnetization_vector
        self.element_magnetization_vector = (magnetization_vector[0] / len(elements),
                                             magnetization_vector[1] / len(elements))


def magnet_contributions(coords, conn, elements, non_contour_nodes, magnetization):
    """(node indices, values) one MagnetLoad adds to the right-hand side, in the
    reference's order: contour edges in order of first appearance over the triangles'
    edges (p1, p2), (p2, p3), (p3, p1), each giving its start point then its end point
    (loads.py:129-147, analysis.py:556-577).  Arrays only: the edge count is a sort,
    not a dict of edge objects."""
    coords = np.asarray(coords, np.float64)
    tri = np.asarray(conn, np.int64)[np.asarray(elements, np.int64)]
    if tri.size == 0:
        return np.zeros(0, np.int64), np.zeros(0)
    start = tri.reshape(-1)
    end = np.roll(tri, -1, axis=1).reshape(-1)
    opposite = np.roll(tri, -2, axis=1).reshape(-1)
    lo, hi = np.minimum(start, end), np.maximum(start, end)
    key = lo * (int(coords.shape[0]) + 1) + hi
    _, inverse, counts = np.unique(key, return_inverse=True, return_counts=True)
    single = counts[inverse] == 1
    nc = np.zeros(coords.shape[0] + 1, bool)
    nc[np.asarray(non_contour_nodes, np.int64)] = True
    keep = single & ~(nc[start] & nc[end])
    idx = np.flatnonzero(keep)          # each kept edge occurs once: list order is first-appearance order
    a, b, c = coords[start[idx], :2], coords[end[idx], :2], coords[opposite[idx], :2]
    tx, ty = b[:, 0] - a[:, 0], b[:, 1] - a[:, 1]
    length = np.sqrt(tx ** 2 + ty ** 2)
    nx, ny = -ty / length, tx / length
    flip = nx * (c[:, 0] - a[:, 0]) + ny * (c[:, 1] - a[:, 1]) < 0
    nx, ny = np.where(flip, -nx, nx), np.where(flip, -ny, ny)
    mx, my = float(magnetization[0]), float(magnetization[1])
    val = (mx * -ny + my * nx) * length / 2
    nodes = np.stack([start[idx], end[idx]], axis=1).reshape(-1)
    return nodes, np.repeat(val, 2)
