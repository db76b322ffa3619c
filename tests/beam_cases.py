"""The cantilever of the reference's scripts/Elasticity/beam2d_example_3.py: a 10 x 1
plane-stress beam (E = 30e6, nu = 0.25, t = 1), clamped at x = 0, a -1000 load in
dimension 2 at (10, 1); Euler-Bernoulli tip deflection P L^3 / (3 E I), I = t b^3 / 12."""
import numpy as np

from finite_elements_gb300.problem import ELASTIC, Problem

E, NU, T, LOAD = 30e6, 0.25, 1.0, -1000.0
ANALYTIC_TIP = LOAD * 10.0 ** 3 / (3 * E * (T * 1.0 ** 3 / 12))


def beam_problem(coords, conn):
    """(Problem, tip node) of the beam on a mesh of the 10 x 1 rectangle."""
    coords = np.asarray(coords, np.float64)[:, :2]
    tip = int(np.flatnonzero((np.abs(coords[:, 0] - 10) < 1e-9) & (np.abs(coords[:, 1] - 1) < 1e-9))[0])
    clamp = np.flatnonzero(np.abs(coords[:, 0]) < 1e-9)
    ne = len(conn)
    prob = Problem(ELASTIC, coords, conn, E=np.full(ne, E), nu=np.full(ne, NU), thickness=np.full(ne, T),
                   rho=np.full(ne, 2.7), plane_strain=False, plane_stress=True,
                   node_load_node=[tip], node_load_dim=[2], node_load_value=[LOAD],
                   node_bc_node=np.repeat(clamp, 2), node_bc_dim=np.tile([1, 2], clamp.size),
                   node_bc_value=np.zeros(2 * clamp.size))
    return prob, tip
