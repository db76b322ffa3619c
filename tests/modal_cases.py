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
