"""Material and constants (finite_elements/core.py:31, :139-171)."""
import math

MU = 4 * math.pi * 1e-7


class Material:
    """Elastic material: elasticity modulus, Poisson ratio, mass density."""

    def __init__(self, elasticity_modulus, poisson_ratio, mass_density, name: str = ''):
        self.elasticity_modulus = elasticity_modulus
        self.poisson_ratio = poisson_ratio
        self.mass_density = mass_density
        self.name = name


def global_matrix_positions(dimension, nodes_number):
    """{(node, d): node*dimension + d - 1} for d = 1..dimension (core.py:89-108)."""
    return {(i, j + 1): i * dimension + j for i in range(nodes_number) for j in range(dimension)}
