"""Tensor-product meshes in the layout the sweep consumes.

A mesh is plain arrays: vertex coordinates, element-to-vertex connectivity in
MFEM's local vertex order (quad: (0,0),(1,0),(1,1),(0,1); hex: the bottom quad
then the top quad; segment: left, right) and the boundary faces with their
attributes.  ``cartesian`` follows MFEM's MakeCartesian{1,2,3}D with
``sfc_ordering = false`` (elements lexicographic, x fastest), which is how
allium's test suite and its Lua inputs build structured meshes
(src/io.cpp:345-368, test/test_sweep.cpp:64-108).  Boundary attributes follow
MFEM: 1D left=1, right=2; 2D bottom=1, right=2, top=3, left=4; 3D z=0 is 1,
y=0 is 2, x=1 is 3, y=1 is 4, x=0 is 5, z=1 is 6.

``jitter`` moves interior vertices by independent U[-jitter*h, jitter*h] offsets per
coordinate (seeded), keeping boundary vertices fixed.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    dim: int
    vertices: np.ndarray          # [nv, dim] float64
    elements: np.ndarray          # [ne, 2^dim] int32, MFEM local vertex order
    boundary_faces: np.ndarray    # [nbf, 2^(dim-1)] int32
    boundary_attributes: np.ndarray  # [nbf] int32
    shape: tuple = ()             # cells per axis when structured

    @property
    def num_elements(self) -> int:
        return int(self.elements.shape[0])

    @property
    def num_vertices(self) -> int:
        return int(self.vertices.shape[0])


def cartesian(cells, extents=None, jitter: float = 0.0, seed: int | None = None) -> Mesh:
    cells = tuple(int(c) for c in cells)
    dim = len(cells)
    if dim not in (1, 2, 3):
        raise ValueError("dimension must be 1, 2 or 3")
    extents = tuple(float(x) for x in (extents or (1.0,) * dim))
    nvx = [c + 1 for c in cells]
    axes = [np.linspace(0.0, extents[d], nvx[d]) for d in range(dim)]
    grids = np.meshgrid(*axes, indexing="ij")
    # vertex id = i + nvx0 * (j + nvx1 * k)  (x fastest)
    verts = np.stack([g.transpose(*reversed(range(dim))).reshape(-1) for g in grids], axis=1)
    verts = np.ascontiguousarray(verts, dtype=np.float64)

    def vid(*ijk):
        v = 0
        stride = 1
        for d in range(dim):
            v = v + ijk[d] * stride
            stride *= nvx[d]
        return v

    idx = np.meshgrid(*[np.arange(c) for c in cells], indexing="ij")
    idx = [a.transpose(*reversed(range(dim))).reshape(-1) for a in idx]   # element lexicographic
    if dim == 1:
        (i,) = idx
        elems = np.stack([vid(i), vid(i + 1)], axis=1)
    elif dim == 2:
        i, j = idx
        elems = np.stack([vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)], axis=1)
    else:
        i, j, k = idx
        elems = np.stack([vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                          vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)], axis=1)
    elems = np.ascontiguousarray(elems, dtype=np.int32)

    bf, ba = [], []
    if dim == 1:
        bf = [[vid(0)], [vid(cells[0])]]
        ba = [1, 2]
    elif dim == 2:
        nx, ny = cells
        for i in range(nx):
            bf.append([vid(i, 0), vid(i + 1, 0)]); ba.append(1)
        for j in range(ny):
            bf.append([vid(nx, j), vid(nx, j + 1)]); ba.append(2)
        for i in range(nx):
            bf.append([vid(i + 1, ny), vid(i, ny)]); ba.append(3)
        for j in range(ny):
            bf.append([vid(0, j + 1), vid(0, j)]); ba.append(4)
    else:
        nx, ny, nz = cells
        for j in range(ny):
            for i in range(nx):
                bf.append([vid(i, j, 0), vid(i, j + 1, 0), vid(i + 1, j + 1, 0), vid(i + 1, j, 0)]); ba.append(1)
        for k in range(nz):
            for i in range(nx):
                bf.append([vid(i, 0, k), vid(i + 1, 0, k), vid(i + 1, 0, k + 1), vid(i, 0, k + 1)]); ba.append(2)
        for k in range(nz):
            for j in range(ny):
                bf.append([vid(nx, j, k), vid(nx, j + 1, k), vid(nx, j + 1, k + 1), vid(nx, j, k + 1)]); ba.append(3)
        for k in range(nz):
            for i in range(nx):
                bf.append([vid(i + 1, ny, k), vid(i, ny, k), vid(i, ny, k + 1), vid(i + 1, ny, k + 1)]); ba.append(4)
        for k in range(nz):
            for j in range(ny):
                bf.append([vid(0, j + 1, k), vid(0, j, k), vid(0, j, k + 1), vid(0, j + 1, k + 1)]); ba.append(5)
        for j in range(ny):
            for i in range(nx):
                bf.append([vid(i, j, nz), vid(i + 1, j, nz), vid(i + 1, j + 1, nz), vid(i, j + 1, nz)]); ba.append(6)
    bfaces = np.ascontiguousarray(np.array(bf, dtype=np.int32).reshape(len(ba), -1))
    battr = np.array(ba, dtype=np.int32)

    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        h = np.array([extents[d] / cells[d] for d in range(dim)])
        interior = np.ones(verts.shape[0], dtype=bool)
        for d in range(dim):
            interior &= (verts[:, d] > 0.0) & (verts[:, d] < extents[d])
        offs = rng.uniform(-jitter, jitter, size=verts.shape) * h
        verts = verts + offs * interior[:, None]
    return Mesh(dim, verts, elems, bfaces, battr, cells)


def disjoint_union(meshes):
    """One mesh holding independent meshes side by side (no shared vertices, so
    no shared faces): elements, vertices and boundary faces concatenated in
    order.  Returns (mesh, element_offsets) with element_offsets[k] the first
    element of meshes[k] and element_offsets[-1] the total."""
    dim = meshes[0].dim
    verts, elems, bfs, bas = [], [], [], []
    voff, eoffs = 0, [0]
    for m in meshes:
        if m.dim != dim:
            raise ValueError("meshes of one union must share the dimension")
        verts.append(m.vertices)
        elems.append(m.elements + voff)
        bfs.append(m.boundary_faces + voff)
        bas.append(m.boundary_attributes)
        voff += m.num_vertices
        eoffs.append(eoffs[-1] + m.num_elements)
    mesh = Mesh(dim, np.ascontiguousarray(np.concatenate(verts), dtype=np.float64),
                np.ascontiguousarray(np.concatenate(elems), dtype=np.int32),
                np.ascontiguousarray(np.concatenate(bfs), dtype=np.int32),
                np.ascontiguousarray(np.concatenate(bas), dtype=np.int32))
    return mesh, np.array(eoffs, dtype=np.int64)
