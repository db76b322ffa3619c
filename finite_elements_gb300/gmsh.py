"""Gmsh 4.1 ASCII meshes: reading the triangle and tetrahedron meshes the reference's
scripts load (scripts/InputFiles/2D/*.msh and 3D/*.msh through volmdlr's GmshParser,
e.g. scripts/Elasticity/beam2d_example_3.py:52-73, beam3d_example_2.py:75-93) and
writing them back.

The reader follows the published MSH 4.1 ASCII layout:

* ``$Nodes``: ``numEntityBlocks numNodes minNodeTag maxNodeTag``, then per block
  ``entityDim entityTag parametric numNodesInBlock``, the block's node tags, then one
  ``x y z`` line per node;
* ``$Elements``: ``numEntityBlocks numElements minElementTag maxElementTag``, then per
  block ``entityDim entityTag elementType numElementsInBlock`` and one line per element,
  ``elementTag nodeTag ...``.  Type 2 is the 3-node triangle, type 4 the 4-node
  tetrahedron; the other types (points, lines) are skipped.

Nodes keep the file's order (the reference's scripts set ``mesh.nodes =
gmsh.nodes['all_nodes']`` "to keep Gmsh order"); triangles and tetrahedra keep file
order, one group per surface (volume) entity.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import ArrayMesh

TRIANGLE = 2
TETRAHEDRON = 4


@dataclass
class GmshMesh:
    coords: np.ndarray          # (n, 3) float64, file order
    node_tags: np.ndarray       # (n,) int64 Gmsh tags of those nodes
    triangles: np.ndarray       # (E, 3) int32 indices into coords
    group_ptr: np.ndarray       # (G+1,) triangles of surface entity g: group_ptr[g]:group_ptr[g+1]
    group_tags: np.ndarray      # (G,) the surface entity tags
    tetrahedra: np.ndarray = None      # (T, 4) int32 indices into coords
    tet_group_ptr: np.ndarray = None   # (V+1,) tetrahedra of volume entity v
    tet_group_tags: np.ndarray = None  # (V,) the volume entity tags

    def array_mesh(self) -> ArrayMesh:
        """The mesh for the analysis: the tetrahedra with (x, y, z) when the file has
        any (define_tetrahedron_element_mesh), else the planar triangles with (x, y);
        one element group per volume (surface) entity."""
        if self.tetrahedra is not None and self.tetrahedra.shape[0] > 0:
            return ArrayMesh(self.coords, self.tetrahedra, self.tet_group_ptr)
        return ArrayMesh(self.coords[:, :2], self.triangles, self.group_ptr)


def _section(lines, name):
    try:
        start = lines.index(f"${name}")
        end = lines.index(f"$End{name}", start)
    except ValueError:
        return None
    return lines[start + 1:end]


def read_msh(path) -> GmshMesh:
    """Parse a Gmsh 4.1 ASCII file."""
    with open(path, encoding="utf-8") as f:
        lines = [l.strip() for l in f]
    fmt = _section(lines, "MeshFormat")
    if not fmt:
        raise ValueError(f"{path}: no $MeshFormat section")
    version, file_type = fmt[0].split()[:2]
    if not version.startswith("4.") or file_type != "0":
        raise ValueError(f"{path}: MSH {version} (type {file_type}) is not MSH 4.x ASCII")

    nodes = _section(lines, "Nodes")
    if nodes is None:
        raise ValueError(f"{path}: no $Nodes section")
    n_blocks, n_nodes = (int(v) for v in nodes[0].split()[:2])
    tags = np.empty(n_nodes, np.int64)
    coords = np.empty((n_nodes, 3))
    pos, k = 1, 0
    for _ in range(n_blocks):
        _, _, parametric, count = (int(v) for v in nodes[pos].split())
        if parametric:
            raise ValueError(f"{path}: parametric nodes are not supported")
        pos += 1
        for j in range(count):
            tags[k + j] = int(nodes[pos + j])
        pos += count
        for j in range(count):
            coords[k + j] = [float(v) for v in nodes[pos + j].split()[:3]]
        pos += count
        k += count
    if k != n_nodes:
        raise ValueError(f"{path}: {k} nodes read, {n_nodes} declared")
    index = {int(t): i for i, t in enumerate(tags)}

    elems = _section(lines, "Elements")
    if elems is None:
        raise ValueError(f"{path}: no $Elements section")
    n_blocks = int(elems[0].split()[0])
    found = {TRIANGLE: ([], [0], []), TETRAHEDRON: ([], [0], [])}
    pos = 1
    for _ in range(n_blocks):
        dim, entity, etype, count = (int(v) for v in elems[pos].split())
        pos += 1
        if etype in found:
            rows, ptr, group_tags = found[etype]
            nn = 3 if etype == TRIANGLE else 4
            for j in range(count):
                v = elems[pos + j].split()
                rows.append([index[int(t)] for t in v[1:1 + nn]])
            ptr.append(len(rows))
            group_tags.append(entity)
        pos += count
    tri, tri_ptr, tri_tags = found[TRIANGLE]
    tet, tet_ptr, tet_tags = found[TETRAHEDRON]
    return GmshMesh(coords, tags, np.array(tri, dtype=np.int32).reshape(-1, 3), np.array(tri_ptr, np.int64),
                    np.array(tri_tags, np.int64), np.array(tet, dtype=np.int32).reshape(-1, 4),
                    np.array(tet_ptr, np.int64), np.array(tet_tags, np.int64))


def write_msh(path, coords, elements, node_tags=None):
    """Write a triangle mesh ((E, 3) elements, one block on surface entity 1) or a
    tetrahedron mesh ((E, 4) elements, one block on volume entity 1) as Gmsh 4.1 ASCII:
    one node block, one element block, no geometric entities section (which MSH 4.1
    allows)."""
    coords = np.asarray(coords, np.float64)
    if coords.shape[1] == 2:
        coords = np.hstack([coords, np.zeros((coords.shape[0], 1))])
    el = np.asarray(elements, np.int64)
    nn = el.shape[1] if el.ndim == 2 else 3
    el = el.reshape(-1, nn)
    etype, edim = (TETRAHEDRON, 3) if nn == 4 else (TRIANGLE, 2)
    n, e = coords.shape[0], el.shape[0]
    tags = np.arange(1, n + 1) if node_tags is None else np.asarray(node_tags, np.int64)
    out = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Nodes",
           f"1 {n} {int(tags.min()) if n else 0} {int(tags.max()) if n else 0}", f"{edim} 1 0 {n}"]
    out += [str(int(t)) for t in tags]
    out += [f"{x!r} {y!r} {z!r}" for x, y, z in coords.tolist()]
    out += ["$EndNodes", "$Elements", f"1 {e} 1 {e}", f"{edim} 1 {etype} {e}"]
    out += [f"{k + 1} " + " ".join(str(tags[i]) for i in row) for k, row in enumerate(el.tolist())]
    out += ["$EndElements"]
    with open(path, "w", encoding="utf-8") as f:
        f.write("\n".join(out) + "\n")
