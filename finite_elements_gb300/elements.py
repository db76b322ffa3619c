"""Element objects of the drop-in API (finite_elements/elements.py:56-91, :194-464).

They carry the element's points and material only; every element matrix is
computed by the GPU element kernels when the analysis assembles (the per-element
numpy matrices of the reference are not recomputed here: use
``FiniteElementAnalysis.element_matrices()`` for them, batched on the device).
"""
from __future__ import annotations

from .mesh import TetrahedralElement, TriangularElement2D


class Element2D(TriangularElement2D):
    """A triangle of the analysis mesh."""


class MagneticElement2D(Element2D):
    """Magnetostatic triangle with absolute permeability ``mu_total``
    (elements.py:74-91); one DOF (A_z) per node."""

    def __init__(self, triangular_element, mu_total: float, name: str = ''):
        self.triangular_element = triangular_element
        Element2D.__init__(self, triangular_element.points, name=name)
        self.mu_total = mu_total

    @property
    def dimension(self):
        return 1


class ElasticityElement:
    """Elastic material attached to a mesh element (elements.py:229-249)."""

    def __init__(self, mesh_element, elasticity_modulus, poisson_ratio, mass_density,
                 displacements=None, stress=None, strain=None, name: str = ''):
        self.mesh_element = mesh_element
        self.elasticity_modulus = elasticity_modulus
        self.poisson_ratio = poisson_ratio
        self.mass_density = mass_density
        self.points = mesh_element.points
        self.displacements = displacements
        self.stress = stress
        self.strain = strain
        self.name = name

    @classmethod
    def with_material_object(cls, mesh_element, material, displacements=None, stress=None,
                             strain=None, name: str = ''):
        return cls(mesh_element=mesh_element, elasticity_modulus=material.elasticity_modulus,
                   poisson_ratio=material.poisson_ratio, mass_density=material.mass_density,
                   displacements=displacements, stress=stress, strain=strain, name=name)


class ElasticityTriangularElement2D(ElasticityElement, Element2D):
    """Plane-elasticity triangle (elements.py:333-391); two DOFs per node."""

    def __init__(self, mesh_element, elasticity_modulus, poisson_ratio, mass_density,
                 thickness: float = 1.0, displacements=None, stress=None, strain=None,
                 name: str = ''):
        self.thickness = thickness
        ElasticityElement.__init__(self, mesh_element, elasticity_modulus, poisson_ratio,
                                   mass_density, displacements, stress, strain, name)
        Element2D.__init__(self, mesh_element.points, name=name)

    @property
    def dimension(self):
        return 2


class ElasticityTetrahedralElement3D(ElasticityElement, TetrahedralElement):
    """Linear elasticity tetrahedron (elements.py:663-876); three DOFs per node, the
    isotropic 3D D whichever plane flag the analysis sets."""

    def __init__(self, mesh_element, elasticity_modulus, poisson_ratio, mass_density,
                 displacements=None, stress=None, strain=None, name: str = ''):
        ElasticityElement.__init__(self, mesh_element, elasticity_modulus, poisson_ratio,
                                   mass_density, displacements, stress, strain, name)
        TetrahedralElement.__init__(self, mesh_element.points, name=name)

    @property
    def dimension(self):
        return 3
