"""Result containers (finite_elements/results.py:23-54) and the GPU-computed
per-element results of elasticity and magnetostatic solutions."""
from __future__ import annotations

import numpy as np


class Result:
    """``mesh`` and ``result_vector``: n_nodes*dim displacements (or potentials)
    followed by one Lagrange multiplier per Dirichlet condition."""

    def __init__(self, mesh, result_vector):
        self.mesh = mesh
        self.result_vector = result_vector

    @property
    def dimension(self):
        return self.mesh.elements_groups[0].elements[0].dimension


def _system_for(mesh, plane_strain=None, plane_stress=None):
    """A GPU system for a mesh of elasticity or magnetic elements (stiffness only:
    the post-processing reads element matrices and geometry)."""
    from .analysis import FiniteElementAnalysis
    fea = FiniteElementAnalysis(mesh, [], [], [], [], [], [], [], [], plane_strain, plane_stress)
    return fea.system()


class ElasticityResults2D(Result):
    """Per-element strain, stress and energy of a plane-elasticity solution
    (finite_elements/results.py:930, :700-830), computed by the GPU kernels.
    Arrays follow the mesh's element order (groups, then elements)."""

    def __init__(self, mesh, result_vector, plane_strain, plane_stress, system=None):
        Result.__init__(self, mesh, result_vector)
        self.plane_strain = plane_strain
        self.plane_stress = plane_stress
        self._system = system
        self._post = None

    def _compute(self):
        if self._post is None:
            if self._system is None:
                self._system = _system_for(self.mesh, self.plane_strain, self.plane_stress)
            self._post = self._system.post(np.asarray(self.result_vector, np.float64))
        return self._post

    @property
    def strain(self):
        return self._compute()["strain"]

    @property
    def stress(self):
        return self._compute()["stress"]

    @property
    def energy_per_element(self):
        return self._compute()["energy"]

    @property
    def energy(self):
        return float(np.sum(self.energy_per_element))

    @property
    def displacement_vectors_per_node(self):
        n = len(self.mesh.nodes)
        return np.asarray(self.result_vector[: 2 * n], np.float64).reshape(n, 2)


class MagneticResults(Result):
    """Per-element magnetic flux density B = curl A of a magnetostatic solution
    (finite_elements/results.py:57-152), computed by the GPU kernel."""

    def __init__(self, mesh, result_vector, system=None):
        Result.__init__(self, mesh, result_vector)
        self._system = system
        self._field = None

    @property
    def magnetic_field_per_element(self):
        if self._field is None:
            if self._system is None:
                self._system = _system_for(self.mesh)
            self._field = self._system.post(np.asarray(self.result_vector, np.float64))["field"]
        return self._field

    @property
    def magnetic_field_norm(self):
        return np.hypot(self.magnetic_field_per_element[:, 0], self.magnetic_field_per_element[:, 1])
