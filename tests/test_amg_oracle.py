"""The CPU model of a smoothed-aggregation preconditioner (oracle/amg_oracle.py) on the
benchmark's problem family: it solves the eliminated system to the oracle's direct
solution, and its PCG iteration count stays flat as the grid is refined while the
block-Jacobi Chebyshev preconditioner's grows."""
import numpy as np
import scipy.sparse.linalg as spla

from finite_elements_gb300 import meshgen
from oracle import amg_oracle as AMG
from oracle import fe_oracle as O


def test_smoothed_aggregation_is_mesh_independent():
    its, cheb = [], []
    for nx, ny in ((60, 30), (120, 60)):
        prob = meshgen.plane_strain_random(nx, ny, seed=0)
        A, b, free, *_ = O.reduced_system(prob)
        A = A.tocsr()
        xy = prob.coords[free[0::2] // 2]
        M = AMG.SmoothedAggregation(A, AMG.rigid_modes_2d(xy))
        x, it = AMG.pcg(A, b, M)
        xd = spla.spsolve(A.tocsc(), b)
        assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)
        its.append(it)
        Minv = AMG.block_diag_inv(A, 2)
        ch = AMG.chebyshev(A, Minv, AMG.lmax_power(A, Minv, 40), 1e5, 31)
        cheb.append(AMG.pcg(A, b, ch)[1])
    assert its[1] <= its[0] + 4 and its[1] <= 35, its
    assert cheb[1] > cheb[0], cheb
