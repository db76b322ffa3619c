"""Batched solves of many independent elasticity problems in one set of launches.

``BatchedSystem(problems)`` concatenates the problems into one block-diagonal union
(node and element indices shifted, loads and conditions kept in instance order), so
the whole batch is assembled by one fe_assemble and solved by the batched PCG of
fe_batch_* with per-instance step sizes and convergence.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .engine import GpuSystem
from .problem import ELASTIC, ElementLoadSet, Problem


def shard_instances(n_dof, world):
    """Independent instances split across `world` ranks (one GPU each, no data exchange
    between them): largest first, each to the least-loaded rank (ties: the lower rank).
    Returns, per rank, its instance indices in increasing order.  Every rank's DOF total
    is then within the largest instance of every other rank's."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(n_dof)), key=lambda i: (-int(n_dof[i]), i))
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += int(n_dof[i])
    return [sorted(o) for o in out]


def union_problem(problems):
    """(union Problem, node_ptr, element_ptr) of a list of elasticity Problems that
    share the plane mode."""
    if not problems:
        raise ValueError("no problem to batch")
    modes = {(bool(p.plane_strain), bool(p.plane_stress)) for p in problems}
    if len(modes) != 1 or any(p.kind != ELASTIC for p in problems):
        raise ValueError("a batch holds elasticity problems of one plane mode")
    node_ptr = np.cumsum([0] + [p.n_nodes for p in problems]).astype(np.int64)
    elem_ptr = np.cumsum([0] + [p.n_elements for p in problems]).astype(np.int64)
    cat = np.concatenate

    def sh(a, k):
        return np.asarray(a) + node_ptr[k]

    loads = []
    for k, p in enumerate(problems):
        loads += [ElementLoadSet(s.elements + elem_ptr[k], s.value, s.dimension) for s in p.element_loads]
    rho = None
    if all(p.rho is not None for p in problems):
        rho = cat([p.rho for p in problems])
    u = Problem(
        ELASTIC, cat([p.coords for p in problems]),
        cat([p.conn.astype(np.int64) + node_ptr[k] for k, p in enumerate(problems)]),
        E=cat([p.E for p in problems]), nu=cat([p.nu for p in problems]),
        thickness=cat([p.thickness for p in problems]), rho=rho,
        plane_strain=problems[0].plane_strain, plane_stress=problems[0].plane_stress,
        node_load_node=cat([sh(p.node_load_node, k) for k, p in enumerate(problems)]),
        node_load_dim=cat([p.node_load_dim for p in problems]),
        node_load_value=cat([p.node_load_value for p in problems]),
        element_loads=loads,
        edge_load_nodes=cat([sh(p.edge_load_nodes, k).reshape(-1, 2) for k, p in enumerate(problems)]),
        edge_load_dim=cat([p.edge_load_dim for p in problems]),
        edge_load_value=cat([p.edge_load_value for p in problems]),
        node_bc_node=cat([sh(p.node_bc_node, k) for k, p in enumerate(problems)]),
        node_bc_dim=cat([p.node_bc_dim for p in problems]),
        node_bc_value=cat([p.node_bc_value for p in problems]),
        element_bc_element=cat([np.asarray(p.element_bc_element) + elem_ptr[k] for k, p in enumerate(problems)]),
        element_bc_dim=cat([p.element_bc_dim for p in problems]),
        element_bc_value=cat([p.element_bc_value for p in problems]),
        edge_bc_nodes=cat([sh(p.edge_bc_nodes, k).reshape(-1, 2) for k, p in enumerate(problems)]),
        edge_bc_dim=cat([p.edge_bc_dim for p in problems]),
        edge_bc_value=cat([p.edge_bc_value for p in problems]))
    return u, node_ptr, elem_ptr


class BatchedSystem:
    """All problems assembled as one union handle plus the batched solver."""

    def __init__(self, problems):
        self.problems = list(problems)
        self.union, self.node_ptr, self.elem_ptr = union_problem(self.problems)
        self.system = GpuSystem(self.union)
        lib = _lib.load()
        self._lib = lib
        b = ctypes.c_void_p()
        _lib.check(lib.fe_batch_create(self.system.handle.h, len(self.problems), _lib.ptr(self.node_ptr),
                                       ctypes.byref(b)), "fe_batch_create")
        self.b = b

    def autotune(self):
        lanes, rows, us = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_double()
        _lib.check(self._lib.fe_batch_autotune(self.b, ctypes.byref(lanes), ctypes.byref(rows), ctypes.byref(us)),
                   "fe_batch_autotune")
        return {"lanes": lanes.value, "rows_per_chunk": rows.value, "us_per_iteration": us.value}

    def set_tiles(self, lanes, rows_per_chunk):
        _lib.check(self._lib.fe_batch_set_tiles(self.b, lanes, rows_per_chunk), "fe_batch_set_tiles")

    def solve(self, tol=1e-8, max_iter=0, want_x=True):
        """Per-instance displacements (list of arrays, n_dof_i each) or None, and
        the stats: iterations, status, true relative residual per instance, device ms."""
        n = len(self.problems)
        it = np.zeros(n, np.int32)
        stv = np.zeros(n, np.int32)
        rel = np.zeros(n)
        x = np.empty(self.union.n_dof) if want_x else None
        ms = ctypes.c_double()
        _lib.check(self._lib.fe_batch_solve(self.b, tol, max_iter, _lib.ptr(it), _lib.ptr(stv), _lib.ptr(rel),
                                            _lib.ptr(x) if want_x else None, ctypes.byref(ms)), "fe_batch_solve")
        parts = None
        if want_x:
            parts = [x[2 * self.node_ptr[k]: 2 * self.node_ptr[k + 1]] for k in range(n)]
        return parts, {"iterations": it, "status": stv, "relres": rel, "solve_ms": ms.value}

    def close(self):
        if getattr(self, "b", None):
            self._lib.fe_batch_destroy(self.b)
            self.b = None
        if getattr(self, "system", None):
            self.system.close()
            self.system = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
