"""Seeded synthetic problems of the sizes the path is benchmarked and tested on.

Every generator returns a :class:`~finite_elements_gb300.problem.Problem` (arrays
only), so that meshes of millions of triangles never exist as Python objects.

Grids use the reference's own split of a rectangle cell into two triangles,
(i,j)(i+1,j)(i,j+1) and (i+1,j+1)(i+1,j)(i,j+1)
(scripts/Elasticity/beam2d_example_2.py:38-41), with node id = j*(nx+1) + i.
"""
from __future__ import annotations

import math

import numpy as np

from .problem import ELASTIC, MAGNETIC, ElementLoadSet, Problem

MU0 = 4 * math.pi * 1e-7   # finite_elements/core.py:31


def rect_grid(nx, ny, lx, ly, jitter=0.0, rng=None):
    """Structured nx-by-ny cell grid on [0,lx]x[0,ly] -> (coords (n,2), conn (2*nx*ny,3)).

    With ``jitter`` > 0 the interior nodes move by U(-jitter, jitter) cell sizes in x
    and y; boundary nodes stay put so the outer boundary stays straight."""
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(xs, ys)                       # (ny+1, nx+1), row j, column i
    if jitter > 0:
        hx, hy = lx / nx, ly / ny
        dx = rng.uniform(-jitter, jitter, size=X.shape) * hx
        dy = rng.uniform(-jitter, jitter, size=Y.shape) * hy
        dx[0, :] = dx[-1, :] = dx[:, 0] = dx[:, -1] = 0.0
        dy[0, :] = dy[-1, :] = dy[:, 0] = dy[:, -1] = 0.0
        X = X + dx
        Y = Y + dy
    coords = np.stack([X.reshape(-1), Y.reshape(-1)], axis=1)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny))
    i = i.reshape(-1)
    j = j.reshape(-1)
    w = nx + 1
    n00 = j * w + i
    n10 = n00 + 1
    n01 = n00 + w
    n11 = n01 + 1
    t1 = np.stack([n00, n10, n01], axis=1)
    t2 = np.stack([n11, n10, n01], axis=1)
    conn = np.stack([t1, t2], axis=1).reshape(-1, 3).astype(np.int32)
    return coords, conn


def edge_nodes(nx, ny, side):
    """Node ids of one side of the grid in increasing id order."""
    w = nx + 1
    if side == "left":
        return np.arange(ny + 1) * w
    if side == "right":
        return np.arange(ny + 1) * w + nx
    if side == "bottom":
        return np.arange(nx + 1)
    if side == "top":
        return ny * w + np.arange(nx + 1)
    raise ValueError(side)


def clamp(nodes, dims=(1, 2)):
    """Node conditions fixing ``dims`` of every node, ordered node then dimension."""
    nodes = np.asarray(nodes, dtype=np.int64)
    k = len(dims)
    return (np.repeat(nodes, k), np.tile(np.asarray(dims, np.int64), nodes.size),
            np.zeros(nodes.size * k))


def cantilever_c1():
    """Plane stress 40x20 rectangle 1.0 x 0.5 m, 1,600 triangles, 861 nodes:
    E=210e9 Pa, nu=0.3, t=1e-3 m, left edge clamped, -1e3 N in total spread as equal
    NodeLoads in dimension 2 over the 21 right-edge nodes."""
    nx, ny = 40, 20
    coords, conn = rect_grid(nx, ny, 1.0, 0.5)
    ne = conn.shape[0]
    bn, bd, bv = clamp(edge_nodes(nx, ny, "left"))
    right = edge_nodes(nx, ny, "right")
    return Problem(ELASTIC, coords, conn, E=np.full(ne, 210e9), nu=np.full(ne, 0.3),
                   thickness=np.full(ne, 1e-3), rho=np.full(ne, 7850.0),
                   plane_stress=True, plane_strain=False,
                   node_load_node=right, node_load_dim=np.full(right.size, 2),
                   node_load_value=np.full(right.size, -1e3 / right.size),
                   node_bc_node=bn, node_bc_dim=bd, node_bc_value=bv)


def magnetostatic(nx=1000, ny=500, seed=0, lx=0.2, ly=0.1):
    """Magnetostatic A_z problem on a jittered nx-by-ny grid over lx x ly: an iron core
    (mu_r=1000) and two coils (current densities +-1e6 A/m^2, sign drawn from the
    seed) in air (mu_r=1); A_z = 0 on every outer-boundary node.

    Each coil is one ElementsLoad whose total value is J times the coil's area, so
    that the reference's area split (finite_elements/loads.py:32-34) hands each
    element J times its own area."""
    rng = np.random.default_rng(seed)
    coords, conn = rect_grid(nx, ny, lx, ly, jitter=0.3, rng=rng)
    cen = coords[conn].mean(axis=1)
    cx, cy = cen[:, 0] / lx, cen[:, 1] / ly
    in_y = (cy > 0.3) & (cy < 0.7)
    core = in_y & (cx > 0.3) & (cx < 0.7)
    coil_a = in_y & (cx > 0.15) & (cx < 0.25)
    coil_b = in_y & (cx > 0.75) & (cx < 0.85)
    mu = np.where(core, 1000.0, 1.0) * MU0
    sign = 1.0 if rng.uniform() < 0.5 else -1.0
    p = coords[conn]
    area = np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                  - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])) / 2
    loads = []
    for mask, s in ((coil_a, sign), (coil_b, -sign)):
        ids = np.flatnonzero(mask)
        loads.append(ElementLoadSet(ids, s * 1e6 * float(area[ids].sum()), 1))
    w = nx + 1
    jj, ii = np.divmod(np.arange(coords.shape[0]), w)
    boundary = np.flatnonzero((ii == 0) | (ii == nx) | (jj == 0) | (jj == ny))
    return Problem(MAGNETIC, coords, conn, mu=mu, element_loads=loads,
                   node_bc_node=boundary, node_bc_dim=np.ones(boundary.size, np.int64),
                   node_bc_value=np.zeros(boundary.size))


def plane_strain_random(nx=2000, ny=1000, seed=0, lx=2.0, ly=1.0):
    """Plane strain nx-by-ny grid over lx x ly with per-element E = 10**U(9, 12) Pa and
    nu ~ U(0.2, 0.45), left edge clamped, seeded random traction as NodeLoads on
    every top-edge node (dimension 1 ~ U(-0.5, 0.5) kN, dimension 2 ~ U(-1, 0) kN)."""
    rng = np.random.default_rng(seed)
    coords, conn = rect_grid(nx, ny, lx, ly)
    ne = conn.shape[0]
    E = 10.0 ** rng.uniform(9.0, 12.0, ne)
    nu = rng.uniform(0.2, 0.45, ne)
    bn, bd, bv = clamp(edge_nodes(nx, ny, "left"))
    top = edge_nodes(nx, ny, "top")
    fx = rng.uniform(-0.5, 0.5, top.size) * 1e3
    fy = rng.uniform(-1.0, 0.0, top.size) * 1e3
    return Problem(ELASTIC, coords, conn, E=E, nu=nu, thickness=np.ones(ne),
                   rho=np.full(ne, 7800.0), plane_strain=True, plane_stress=False,
                   node_load_node=np.concatenate([top, top]),
                   node_load_dim=np.concatenate([np.ones(top.size, np.int64),
                                                 np.full(top.size, 2, np.int64)]),
                   node_load_value=np.concatenate([fx, fy]),
                   node_bc_node=bn, node_bc_dim=bd, node_bc_value=bv)


def batch_instance_sizes(n_instances=512, seed=0, tri_min=2e3, tri_max=2e5):
    """(nx, ny) of each instance: triangle counts log-uniform in [tri_min, tri_max],
    aspect ratio nx/ny ~ U(1, 8)."""
    rng = np.random.default_rng(seed)
    tri = np.exp(rng.uniform(math.log(tri_min), math.log(tri_max), n_instances))
    aspect = rng.uniform(1.0, 8.0, n_instances)
    ny = np.maximum(1, np.round(np.sqrt(tri / (2 * aspect)))).astype(int)
    nx = np.maximum(1, np.round(tri / (2 * ny))).astype(int)
    return list(zip(nx.tolist(), ny.tolist())), rng


def plane_stress_instance(nx, ny, rng):
    """One batched instance: plane stress cantilever nx-by-ny over (nx/ny) x 1 m,
    E ~ U(50e9, 300e9), nu ~ U(0.2, 0.4), left edge clamped, random NodeLoads on the
    right edge in both dimensions."""
    coords, conn = rect_grid(nx, ny, nx / ny, 1.0)
    ne = conn.shape[0]
    E = rng.uniform(50e9, 300e9)
    nu = rng.uniform(0.2, 0.4)
    bn, bd, bv = clamp(edge_nodes(nx, ny, "left"))
    right = edge_nodes(nx, ny, "right")
    f = rng.uniform(-1.0, 1.0, (2, right.size)) * 1e3
    return Problem(ELASTIC, coords, conn, E=np.full(ne, E), nu=np.full(ne, nu),
                   thickness=np.ones(ne), rho=np.full(ne, 7800.0),
                   plane_stress=True, plane_strain=False,
                   node_load_node=np.concatenate([right, right]),
                   node_load_dim=np.repeat(np.array([1, 2], np.int64), right.size),
                   node_load_value=f.reshape(-1),
                   node_bc_node=bn, node_bc_dim=bd, node_bc_value=bv)


def batch_c4(n_instances=512, seed=0, tri_min=2e3, tri_max=2e5):
    sizes, rng = batch_instance_sizes(n_instances, seed, tri_min, tri_max)
    return [plane_stress_instance(nx, ny, rng) for nx, ny in sizes]


def gaussian_random_field(shape, corr, rng):
    """Zero-mean, unit-variance smooth field on a (ny, nx) grid: white noise filtered
    by a Gaussian kernel of correlation length ``corr`` (in grid cells)."""
    ny, nx = shape
    noise = rng.standard_normal((ny, nx))
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    filt = np.exp(-0.5 * (2 * math.pi * corr) ** 2 * (kx ** 2 + ky ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    f -= f.mean()
    s = f.std()
    return f / s if s > 0 else f


def grf_elasticity(nx, ny, seed=0, lx=None, ly=1.0):
    """Plane strain problem with a smooth random stiffness field: log10 E = 10.5 +
    0.5 * GRF (correlation length 0.1 of the domain), nu ~ U(0.2, 0.45) per draw, one
    randomly chosen clamped side and random NodeLoads on the opposite side."""
    rng = np.random.default_rng(seed)
    if lx is None:
        lx = nx / ny * ly
    coords, conn = rect_grid(nx, ny, lx, ly)
    field = gaussian_random_field((ny, nx), 0.1 * max(nx, ny), rng)
    cell = np.repeat(field.reshape(-1), 2)
    E = 10.0 ** (10.5 + 0.5 * cell)
    ne = conn.shape[0]
    nu = np.full(ne, rng.uniform(0.2, 0.45))
    sides = ("left", "right", "bottom", "top")
    opposite = {"left": "right", "right": "left", "bottom": "top", "top": "bottom"}
    side = sides[int(rng.integers(0, 4))]
    bn, bd, bv = clamp(edge_nodes(nx, ny, side))
    ln = edge_nodes(nx, ny, opposite[side])
    f = rng.uniform(-1.0, 1.0, (2, ln.size)) * 1e3
    return Problem(ELASTIC, coords, conn, E=E, nu=nu, thickness=np.ones(ne),
                   rho=np.full(ne, 7800.0), plane_strain=True, plane_stress=False,
                   node_load_node=np.concatenate([ln, ln]),
                   node_load_dim=np.repeat(np.array([1, 2], np.int64), ln.size),
                   node_load_value=f.reshape(-1),
                   node_bc_node=bn, node_bc_dim=bd, node_bc_value=bv)


# ---------------------------------------------------------------- 3D: linear tetrahedra

# Kuhn split of a hexahedral cell into 6 tetrahedra: corner bits (x=1, y=2, z=4), one
# tetrahedron per axis order, 000 -> +axis1 -> +axis2 -> 111.  Every cell uses the same
# split, so faces match between neighbours.  The odd axis orders give negatively
# oriented tetrahedra (both orientations are exercised).
_KUHN = np.array([[0, 1, 3, 7], [0, 1, 5, 7], [0, 2, 3, 7],
                  [0, 2, 6, 7], [0, 4, 5, 7], [0, 4, 6, 7]], np.int64)


def box_tets(nx, ny, nz, lx, ly, lz, jitter=0.0, rng=None):
    """Structured nx-by-ny-by-nz cell grid on [0,lx]x[0,ly]x[0,lz] split into 6 tetrahedra
    per cell -> (coords (n,3), conn (6*nx*ny*nz,4)), node id = (k*(ny+1) + j)*(nx+1) + i.

    With ``jitter`` > 0 the interior nodes move by U(-jitter, jitter) cell sizes; boundary
    nodes stay put."""
    xs, ys, zs = np.linspace(0.0, lx, nx + 1), np.linspace(0.0, ly, ny + 1), np.linspace(0.0, lz, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")              # (nz+1, ny+1, nx+1)
    coords = np.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], axis=1)
    if jitter > 0:
        h = np.array([lx / nx, ly / ny, lz / nz])
        d = rng.uniform(-jitter, jitter, size=coords.shape) * h
        k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        inner = ((i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)).reshape(-1)
        coords = coords + d * inner[:, None]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    base = ((k * (ny + 1) + j) * (nx + 1) + i).reshape(-1)
    sx, sy, sz = 1, nx + 1, (nx + 1) * (ny + 1)
    corner = np.array([(b & 1) * sx + ((b >> 1) & 1) * sy + ((b >> 2) & 1) * sz for b in range(8)], np.int64)
    conn = (base[:, None, None] + corner[_KUHN][None, :, :]).reshape(-1, 4).astype(np.int32)
    return coords, conn


def cantilever_3d(nx, ny, nz, length=10.0, width=2.0, height=2.0, E=210e9, nu=0.25, rho=7860.0,
                  load=-1000.0, jitter=0.0, seed=0):
    """A solid cantilever of linear tetrahedra, as the reference's 3D beam scripts set it
    up (scripts/Elasticity/beam3d_example_2.py): every node of the face x = 0 clamped
    in dimensions 1, 2 and 3, a NodeLoad ``load`` in dimension 3 at every node of the
    free end's top edge (x = length, z = height)."""
    rng = np.random.default_rng(seed)
    coords, conn = box_tets(nx, ny, nz, length, width, height, jitter, rng)
    ne = conn.shape[0]
    x, z = coords[:, 0], coords[:, 2]
    clamped = np.flatnonzero(x == 0.0)
    tip = np.flatnonzero((x == length) & (z == height))
    from .problem import ELASTIC3D
    return Problem(ELASTIC3D, coords, conn, E=np.full(ne, E), nu=np.full(ne, nu), rho=np.full(ne, rho),
                   plane_strain=False, plane_stress=True,
                   node_load_node=tip, node_load_dim=np.full(tip.size, 3, np.int64),
                   node_load_value=np.full(tip.size, load),
                   node_bc_node=np.repeat(clamped, 3), node_bc_dim=np.tile([1, 2, 3], clamped.size),
                   node_bc_value=np.zeros(3 * clamped.size))


# ---------------------------------------------------------------- 2D: a motor-like annulus

def annulus(radii, nt):
    """Polar grid on the radii r_0 < r_1 < ... < r_m and nt sectors (periodic in the
    angle): node (i, j) at radius r_i and angle 2 pi j / nt has id i * nt + j; each cell
    is split into the two triangles (i,j)(i,j+1)(i+1,j) and (i+1,j+1)(i+1,j)(i,j+1).
    Returns (coords (n,2), conn (2 m nt, 3)); the triangles of radial layer i are
    conn[2 nt i : 2 nt (i+1)]."""
    radii = np.asarray(radii, np.float64)
    m = radii.size - 1
    th = 2 * math.pi * np.arange(nt) / nt
    R, T = np.meshgrid(radii, th, indexing="ij")
    coords = np.stack([(R * np.cos(T)).reshape(-1), (R * np.sin(T)).reshape(-1)], axis=1)
    i, j = np.meshgrid(np.arange(m), np.arange(nt), indexing="ij")
    i, j = i.reshape(-1), j.reshape(-1)
    jn = (j + 1) % nt
    a, b, c, d = i * nt + j, i * nt + jn, (i + 1) * nt + j, (i + 1) * nt + jn
    conn = np.stack([np.stack([a, b, c], 1), np.stack([d, c, b], 1)], 1).reshape(-1, 3).astype(np.int32)
    return coords, conn
