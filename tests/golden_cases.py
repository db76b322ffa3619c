"""Load the golden cases of tests/golden/*.npz back into Problem objects."""
from __future__ import annotations

import glob
import os

import numpy as np

from finite_elements_gb300.problem import ElementLoadSet, MagnetLoadSet, Problem

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def solvable_names():
    """The cases whose reference solve returned a solution (the others raised scipy's
    dimension-mismatch ValueError, kept as ``solve_error``)."""
    out = []
    for n in names():
        with np.load(os.path.join(GOLDEN_DIR, n + ".npz")) as z:
            if "ref_x" in z.files:
                out.append(n)
    return out


def load(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    kind = str(z["kind"])
    plane = z["plane"].tolist()
    kw = {}
    for k in ("E", "nu", "thickness", "rho", "mu"):
        if k in z.files:
            kw[k] = z[k]
    loads = [ElementLoadSet(z[f"element_load_{k}_elements"], float(z[f"element_load_{k}_value"]),
                            int(z[f"element_load_{k}_dim"]))
             for k in range(int(z["n_element_loads"]))]
    magnets = [MagnetLoadSet(z[f"magnet_load_{k}_elements"], z[f"magnet_load_{k}_non_contour"],
                             tuple(z[f"magnet_load_{k}_m"].tolist()))
               for k in range(int(z["n_magnet_loads"]) if "n_magnet_loads" in z.files else 0)]
    cont = {k: z[k] for k in ("cont_node1", "cont_node2", "cont_value") if k in z.files}
    prob = Problem(kind, z["coords"], z["conn"], magnet_loads=magnets, **cont,
                   plane_strain=None if plane[0] < 0 else bool(plane[0]),
                   plane_stress=None if plane[1] < 0 else bool(plane[1]),
                   element_loads=loads,
                   **kw,
                   **{k: z[k] for k in ("node_load_node", "node_load_dim", "node_load_value",
                                        "edge_load_nodes", "edge_load_dim", "edge_load_value",
                                        "node_bc_node", "node_bc_dim", "node_bc_value",
                                        "element_bc_element", "element_bc_dim",
                                        "element_bc_value", "edge_bc_nodes", "edge_bc_dim",
                                        "edge_bc_value")})
    ref = {k[4:]: z[k] for k in z.files if k.startswith("ref_")}
    if "group_names" in z.files:
        ref["_group_names"] = z["group_names"]
    if "motor" in z.files:
        ref["_motor"] = z["motor"]
        ref["_motor_maxwell_elements"] = z["motor_maxwell_elements"]
    return prob, z["groups"], ref
