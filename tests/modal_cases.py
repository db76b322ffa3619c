"""A free 10 x 1 plane-stress beam (the reference's scripts/ModalAnalysis/beam2d_*.py
set-up: no loads, no conditions; E = 30e6, nu = 0.25, t = 1, rho = 2.7)."""
import numpy as np

from finite_elements_gb300 import meshgen
from finite_elements_gb300.problem import ELASTIC, Problem


def free_beam(nx, ny):
    c, conn = meshgen.rect_grid(nx, ny, 10.0, 1.0)
    ne = len(conn)
    return Problem(ELASTIC, c, conn, E=np.full(ne, 30e6), nu=np.full(ne, 0.25), thickness=np.full(ne, 1.0),
                   rho=np.full(ne, 2.7), plane_strain=False, plane_stress=True)


def free_beam_3d(nx, ny, nz):
    """The reference's scripts/ModalAnalysis/beam3d_1.py set-up on a Kuhn grid: a free
    10 x 2 x 2 solid of linear tetrahedra, E = 210e9, nu = 0.25, rho = 7860."""
    from finite_elements_gb300.problem import ELASTIC3D
    c, conn = meshgen.box_tets(nx, ny, nz, 10.0, 2.0, 2.0)
    ne = len(conn)
    return Problem(ELASTIC3D, c, conn, E=np.full(ne, 210e9), nu=np.full(ne, 0.25), rho=np.full(ne, 7860.0),
                   plane_strain=False, plane_stress=True)
