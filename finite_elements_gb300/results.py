"""Result container (finite_elements/results.py:23-54)."""
from __future__ import annotations


class Result:
    """``mesh`` and ``result_vector``: n_nodes*dim displacements (or potentials)
    followed by one Lagrange multiplier per Dirichlet condition."""

    def __init__(self, mesh, result_vector):
        self.mesh = mesh
        self.result_vector = result_vector

    @property
    def dimension(self):
        return self.mesh.elements_groups[0].elements[0].dimension
