"""Synthetic unstructured meshes in the mcfd_mesh_desc format.

The reference reads CGNS files partitioned by METIS (include/mini/mesh/part.hpp);
here the benchmark meshes are generated: a box of nx x ny x nz Hex8 cells with
optional periodic axes and optional jitter of interior nodes.  The output is a
plain unstructured description (node coordinates, CGNS-ordered cell nodes and
a face list with holder/sharer, local face indices, boundary groups and
periodic shifts), so nothing downstream relies on the structure.

Face conventions (coordinate/hexahedron.hpp:378-389): local face 0 is
zeta = -1 (z-), 1 eta = -1 (y-), 2 xi = +1 (x+), 3 eta = +1 (y+),
4 xi = -1 (x-), 5 zeta = +1 (z+).  The holder of an interior face is the cell
with the lower id; its face normal points to the sharer (part.hpp:957-967).
Boundary groups of a non-periodic box: 0 x-, 1 x+, 2 y-, 3 y+, 4 z-, 5 z+.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# local face index of the lower / upper side of each axis
LOWER_SIDE = (4, 1, 0)
UPPER_SIDE = (2, 3, 5)


@dataclass
class Mesh:
    xyz: np.ndarray          # [n_nodes, 3] float64
    cell_nodes: np.ndarray   # [n_cells, 8] int64
    face_cells: np.ndarray   # [n_faces, 2] int64
    face_sides: np.ndarray   # [n_faces, 2] int32
    face_group: np.ndarray   # [n_faces] int32
    face_shift: np.ndarray   # [n_faces, 3] float64
    cell_type: np.ndarray | None = None
    shape: tuple = ()
    lengths: tuple = ()
    origin: tuple = ()
    periodic: tuple = ()
    meta: dict = field(default_factory=dict)

    @property
    def n_cells(self) -> int:
        return int(self.cell_nodes.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.face_cells.shape[0])

    def cell_centers(self) -> np.ndarray:
        return self.xyz[self.cell_nodes].mean(axis=1)


def box(shape, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
        periodic=(False, False, False), jitter: float = 0.0, seed: int = 0) -> Mesh:
    """nx x ny x nz Hex8 cells on [origin, origin + lengths].

    jitter > 0 moves every node strictly inside the box by U(-jitter h, jitter h)
    per axis (h = cell size along that axis), drawn from numpy's PCG64 with
    ``seed``; boundary nodes stay put so periodic faces still match by a shift.
    """
    nx, ny, nz = (int(s) for s in shape)
    L = np.asarray(lengths, dtype=np.float64)
    O = np.asarray(origin, dtype=np.float64)
    h = L / np.array([nx, ny, nz], dtype=np.float64)
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    # node id = (k * (ny+1) + j) * (nx+1) + i
    xyz = np.empty(((nx + 1) * (ny + 1) * (nz + 1), 3), dtype=np.float64)
    nid = ((kk * (ny + 1) + jj) * (nx + 1) + ii).ravel()
    xyz[nid, 0] = O[0] + ii.ravel() * h[0]
    xyz[nid, 1] = O[1] + jj.ravel() * h[1]
    xyz[nid, 2] = O[2] + kk.ravel() * h[2]
    # exact end points
    xyz[nid[ii.ravel() == nx], 0] = O[0] + L[0]
    xyz[nid[jj.ravel() == ny], 1] = O[1] + L[1]
    xyz[nid[kk.ravel() == nz], 2] = O[2] + L[2]
    if jitter > 0:
        rng = np.random.default_rng(seed)
        inner = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)).ravel()
        ids = nid[inner]
        ids.sort()
        xyz[ids] += rng.uniform(-jitter, jitter, size=(ids.size, 3)) * h
    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    cid = (ck * ny + cj) * nx + ci
    order = np.argsort(cid)
    ci, cj, ck = ci[order], cj[order], ck[order]

    def node(i, j, k):
        return (k * (ny + 1) + j) * (nx + 1) + i

    cell_nodes = np.stack([
        node(ci, cj, ck), node(ci + 1, cj, ck), node(ci + 1, cj + 1, ck), node(ci, cj + 1, ck),
        node(ci, cj, ck + 1), node(ci + 1, cj, ck + 1), node(ci + 1, cj + 1, ck + 1), node(ci, cj + 1, ck + 1),
    ], axis=1).astype(np.int64)

    def cell(i, j, k):
        return (k * ny + j) * nx + i

    n = (nx, ny, nz)
    holders, sharers, hsides, ssides, shifts = [], [], [], [], []
    groups_b, holders_b, sides_b = [], [], []
    idx = (ci, cj, ck)
    for ax in range(3):
        ijk = [ci, cj, ck]
        inner = idx[ax] < n[ax] - 1
        nb = list(ijk)
        nb[ax] = idx[ax] + 1
        a = cell(*[v[inner] for v in ijk])
        b = cell(*[v[inner] for v in nb])
        holders.append(a); sharers.append(b)
        hsides.append(np.full(a.size, UPPER_SIDE[ax])); ssides.append(np.full(a.size, LOWER_SIDE[ax]))
        shifts.append(np.zeros((a.size, 3)))
        last = idx[ax] == n[ax] - 1
        first = idx[ax] == 0
        if periodic[ax]:
            lo = cell(*[v[first] for v in ijk])
            hi_ijk = [v[first].copy() for v in ijk]
            hi_ijk[ax] = np.full(hi_ijk[ax].shape, n[ax] - 1)
            hi = cell(*hi_ijk)
            # holder = lower cell id = the cell at index 0 along the axis
            sh = np.zeros((lo.size, 3))
            sh[:, ax] = -L[ax]
            holders.append(lo); sharers.append(hi)
            hsides.append(np.full(lo.size, LOWER_SIDE[ax])); ssides.append(np.full(lo.size, UPPER_SIDE[ax]))
            shifts.append(sh)
        else:
            lo = cell(*[v[first] for v in ijk])
            hi = cell(*[v[last] for v in ijk])
            holders_b += [lo, hi]
            sides_b += [np.full(lo.size, LOWER_SIDE[ax]), np.full(hi.size, UPPER_SIDE[ax])]
            groups_b += [np.full(lo.size, 2 * ax), np.full(hi.size, 2 * ax + 1)]
    h_i = np.concatenate(holders); s_i = np.concatenate(sharers)
    hs_i = np.concatenate(hsides); ss_i = np.concatenate(ssides)
    sh_i = np.concatenate(shifts)
    o = np.lexsort((hs_i, h_i))  # interior faces sorted by (holder, side)
    face_cells = [np.stack([h_i[o], s_i[o]], axis=1)]
    face_sides = [np.stack([hs_i[o], ss_i[o]], axis=1)]
    face_group = [np.full(o.size, -1)]
    face_shift = [sh_i[o]]
    if holders_b:
        hb = np.concatenate(holders_b); sb = np.concatenate(sides_b); gb = np.concatenate(groups_b)
        ob = np.lexsort((hb, gb))  # boundary faces by (group, holder)
        face_cells.append(np.stack([hb[ob], np.full(ob.size, -1)], axis=1))
        face_sides.append(np.stack([sb[ob], np.full(ob.size, -1)], axis=1))
        face_group.append(gb[ob])
        face_shift.append(np.zeros((ob.size, 3)))
    return Mesh(
        xyz=np.ascontiguousarray(xyz),
        cell_nodes=np.ascontiguousarray(cell_nodes),
        face_cells=np.ascontiguousarray(np.concatenate(face_cells).astype(np.int64)),
        face_sides=np.ascontiguousarray(np.concatenate(face_sides).astype(np.int32)),
        face_group=np.ascontiguousarray(np.concatenate(face_group).astype(np.int32)),
        face_shift=np.ascontiguousarray(np.concatenate(face_shift).astype(np.float64)),
        shape=(nx, ny, nz), lengths=tuple(L), origin=tuple(O), periodic=tuple(periodic),
    )


def gll_points(q: int) -> np.ndarray:
    """Gauss-Lobatto points on [-1, 1] (integrator/lobatto.hpp:37-83)."""
    if q == 2:
        return np.array([-1.0, 1.0])
    if q == 3:
        return np.array([-1.0, 0.0, 1.0])
    if q == 4:
        s = np.sqrt(1.0 / 5)
        return np.array([-1.0, -s, s, 1.0])
    raise ValueError("q must be 2, 3 or 4")


def node_coordinates(mesh: Mesh, degree: int) -> np.ndarray:
    """Global coordinates of the (p+1)^3 GLL nodes of every cell, [cells, N, 3],
    node order i*Q*Q + j*Q + k (integrator/hexahedron.hpp:66-80), through
    each cell's map (Hex8, Hex20 or Hex27)."""
    x = gll_points(degree + 1)
    a, b, c = np.meshgrid(x, x, x, indexing="ij")
    loc = np.stack([a.ravel(), b.ravel(), c.ravel()], axis=1)  # [N, 3]
    types = np.zeros(mesh.n_cells, np.int32) if mesh.cell_type is None else mesh.cell_type
    out = np.empty((mesh.n_cells, loc.shape[0], 3))
    for t in np.unique(types):
        sel = types == t
        shape = hex_shapes(int(t), loc)  # [N, nodes]
        xn = mesh.xyz[mesh.cell_nodes[sel, :shape.shape[1]]]
        out[sel] = np.einsum("nv,cvd->cnd", shape, xn)
    return out


HEX27, TET10, HEX20 = 2, 3, 4
# CGNS HEXA_27 local coordinates (coordinate/hexahedron.hpp Hexahedron27):
# corners, mid-edges bottom / vertical / top, face centres, centre
HEX27_LOCAL = np.array([
    [-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1],
    [0, -1, -1], [1, 0, -1], [0, 1, -1], [-1, 0, -1], [-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0],
    [0, -1, 1], [1, 0, 1], [0, 1, 1], [-1, 0, 1], [0, 0, -1], [0, -1, 0], [1, 0, 0], [0, 1, 0],
    [-1, 0, 0], [0, 0, 1], [0, 0, 0]], dtype=np.float64)
HEX_EDGES = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [0, 4], [1, 5], [2, 6], [3, 7],
                      [4, 5], [5, 6], [6, 7], [7, 4]])
HEX_FACE_CORNERS = np.array([[0, 3, 2, 1], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [0, 4, 7, 3], [4, 5, 6, 7]])
TET_EDGES = np.array([[0, 1], [1, 2], [2, 0], [3, 0], [3, 1], [3, 2]])  # AB BC CA DA DB DC


def hex_shapes(cell_type: int, loc: np.ndarray) -> np.ndarray:
    """Shape functions [points, nodes] of a hexahedron type at local points."""
    L = HEX27_LOCAL
    x, y, z = loc[:, 0:1], loc[:, 1:2], loc[:, 2:3]
    if cell_type == HEX8:
        return (1 + x * L[None, :8, 0]) * (1 + y * L[None, :8, 1]) * (1 + z * L[None, :8, 2]) / 8

    def q1(c, t):
        return np.where(c == 0, 1 - t * t, 0.5 * t * (t + c))
    if cell_type == HEX27:
        return q1(L[None, :, 0], x) * q1(L[None, :, 1], y) * q1(L[None, :, 2], z)
    if cell_type == HEX20:
        l = L[:20]
        f = [1 + x * l[None, :, 0], 1 + y * l[None, :, 1], 1 + z * l[None, :, 2]]
        corner = f[0] * f[1] * f[2] * (x * l[None, :, 0] + y * l[None, :, 1] + z * l[None, :, 2] - 2) / 8
        t = [x, y, z]
        out = corner.copy()
        for ax in range(3):
            mid = (l[:, ax] == 0)[None, :]
            o1, o2 = f[(ax + 1) % 3], f[(ax + 2) % 3]
            out = np.where(mid, (1 - t[ax] * t[ax]) * o1 * o2 / 4, out)
        return out
    raise ValueError("not a hexahedron type")


# CGNS PENTA_15 / PENTA_18 (coordinate/wedge.hpp Wedge15 / Wedge18): mid-edges
# 6-14 of the bottom triangle, the vertical edges and the top triangle, then
# the centres 15-17 of the quadrangles; PYRA_13 / PYRA_14 (coordinate/
# pyramid.hpp Pyramid13 / Pyramid14): mid-edges 5-8 of the base, 9-12 of the
# lateral edges, then the base centre 13.
WEDGE_EDGES = np.array([[0, 1], [1, 2], [2, 0], [0, 3], [1, 4], [2, 5], [3, 4], [4, 5], [5, 3]])
WEDGE_QUAD_CORNERS = np.array([[0, 1, 4, 3], [1, 2, 5, 4], [2, 0, 3, 5]])
PYRA_EDGES = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [0, 4], [1, 4], [2, 4], [3, 4]])
PYRA_BASE = np.array([[0, 1, 2, 3]])


def quadratic(m: Mesh, serendipity: bool = False) -> Mesh:
    """The same mesh with quadratic cells: Hex8 -> Hex27 (Hex20 with
    serendipity=True), Tet4 -> Tet10, Wedge6 -> Wedge18 (Wedge15), Pyra5 ->
    Pyra14 (Pyra13).  Mid-edge, mid-face and centre nodes sit at the averages
    of their corners and are shared between neighbours, so the geometry is
    unchanged until the nodes are moved (see deform())."""
    types = np.zeros(m.n_cells, np.int32) if m.cell_type is None else m.cell_type.astype(np.int32)
    fams = np.array([family(t) for t in types]) if m.cell_type is not None else np.full(m.n_cells, "hex")
    # family -> (corners, edges, quadrangles with centre nodes, cell centre?, new type, nodes)
    spec = {
        "hex": (8, HEX_EDGES, None if serendipity else HEX_FACE_CORNERS, not serendipity,
                HEX20 if serendipity else HEX27, 20 if serendipity else 27),
        "tet": (4, TET_EDGES, None, False, TET10, 10),
        "wedge": (6, WEDGE_EDGES, None if serendipity else WEDGE_QUAD_CORNERS, False,
                  WEDGE15 if serendipity else WEDGE18, 15 if serendipity else 18),
        "pyramid": (5, PYRA_EDGES, None if serendipity else PYRA_BASE, False,
                    PYRA13 if serendipity else PYRA14, 13 if serendipity else 14),
    }
    present = [f for f in spec if (fams == f).any()]
    width = max(spec[f][5] for f in present)
    cn = np.full((m.n_cells, width), -1, dtype=np.int64)
    new_types = types.copy()
    xyz = [m.xyz]
    n_nodes = m.xyz.shape[0]

    def shared(groups):  # groups [k, n]: corner sets -> new node ids (shared by sorted key)
        nonlocal n_nodes
        key = np.sort(groups, axis=1)
        uniq, inv = np.unique(key, axis=0, return_inverse=True)
        xyz.append(m.xyz[uniq].mean(axis=1))
        ids = n_nodes + np.arange(uniq.shape[0])
        n_nodes += uniq.shape[0]
        return ids[inv.ravel()]

    def gather(which):  # corner sets of every present family's table, one shared() call
        rows, where = [], []
        for f in present:
            table = spec[f][which]
            if table is None:
                continue
            cells = np.flatnonzero(fams == f)
            rows.append(m.cell_nodes[cells][:, table].reshape(-1, table.shape[1]))
            where.append((f, cells, table.shape[0]))
        return rows, where

    for f in present:
        cells = np.flatnonzero(fams == f)
        nc = spec[f][0]
        cn[cells, :nc] = m.cell_nodes[cells, :nc]
        new_types[cells] = spec[f][4]
    for which in (1, 2):  # mid-edges, then quadrangle centres
        rows, where = gather(which)
        if not rows:
            continue
        ids = shared(np.concatenate(rows))
        pos = 0
        for f, cells, k in where:
            nc, edges = spec[f][0], spec[f][1]
            first = nc + (0 if which == 1 else edges.shape[0])
            cn[cells, first:first + k] = ids[pos:pos + cells.size * k].reshape(cells.size, k)
            pos += cells.size * k
    hexes = np.flatnonzero(fams == "hex")
    if hexes.size and spec["hex"][3]:
        cn[hexes, 26] = shared(m.cell_nodes[hexes, :8])
    return Mesh(xyz=np.ascontiguousarray(np.concatenate(xyz)), cell_nodes=np.ascontiguousarray(cn),
                face_cells=m.face_cells, face_sides=m.face_sides, face_group=m.face_group,
                face_shift=m.face_shift, cell_type=new_types.astype(np.int32), shape=m.shape,
                lengths=m.lengths, origin=m.origin, periodic=m.periodic, meta=dict(m.meta))


def deform(m: Mesh, fn) -> Mesh:
    """The mesh with every node moved to fn(xyz) (vectorised over [n, 3]);
    keep fn periodic with the box for periodic meshes."""
    return Mesh(xyz=np.ascontiguousarray(fn(m.xyz), dtype=np.float64), cell_nodes=m.cell_nodes,
                face_cells=m.face_cells, face_sides=m.face_sides, face_group=m.face_group,
                face_shift=m.face_shift, cell_type=m.cell_type, shape=m.shape, lengths=m.lengths,
                origin=m.origin, periodic=m.periodic, meta=dict(m.meta))


# Tetrahedron4::faces_ (coordinate/tetrahedron.hpp:141-147): local face ->
# cell node slots, ordered so the normal points out of a positively oriented
# (CGNS) tetrahedron.
TET_FACES = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]], dtype=np.int64)
HEX8, TET4 = 0, 1
WEDGE6, PYRA5 = 5, 6
WEDGE15, WEDGE18, PYRA13, PYRA14 = 7, 8, 9, 10
# local faces of every cell type in the reference's node order (triangles end
# in -1): coordinate/hexahedron.hpp:353-390, tetrahedron.hpp:141-147,
# wedge.hpp:211-223, pyramid.hpp:110-121, 199-208
_HEX_FACES4 = [[0, 3, 2, 1], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [0, 4, 7, 3], [4, 5, 6, 7]]
CELL_FACES = {
    "hex": np.array(_HEX_FACES4, dtype=np.int64),
    "tet": np.array([[0, 2, 1, -1], [0, 1, 3, -1], [0, 3, 2, -1], [1, 2, 3, -1]], dtype=np.int64),
    "wedge": np.array([[0, 2, 1, -1], [3, 4, 5, -1], [0, 1, 4, 3], [1, 2, 5, 4], [0, 3, 5, 2]], dtype=np.int64),
    "pyramid": np.array([[0, 3, 2, 1], [0, 1, 4, -1], [1, 2, 4, -1], [2, 3, 4, -1], [3, 0, 4, -1]], dtype=np.int64),
}
CORNERS = {"hex": 8, "tet": 4, "wedge": 6, "pyramid": 5}


def family(cell_type: int) -> str:
    return {TET4: "tet", 3: "tet", WEDGE6: "wedge", 7: "wedge", 8: "wedge", PYRA5: "pyramid",
            9: "pyramid", 10: "pyramid"}.get(int(cell_type), "hex")

# Kuhn split of a hex into 6 tetrahedra sharing the (0,0,0)-(1,1,1) diagonal:
# for each axis permutation (a, b, c) the path 0 -> e_a -> e_a + e_b -> 1.
# Corner slot of offset (dx, dy, dz) in a CGNS Hex8: see box().
_HEX_SLOT = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3,
             (0, 0, 1): 4, (1, 0, 1): 5, (1, 1, 1): 6, (0, 1, 1): 7}


def _kuhn_tets():
    import itertools
    tets = []
    for perm in itertools.permutations(range(3)):
        path = [(0, 0, 0)]
        cur = [0, 0, 0]
        for ax in perm:
            cur[ax] = 1
            path.append(tuple(cur))
        slots = [_HEX_SLOT[v] for v in path]
        # positive orientation: det[v1 - v0, v2 - v0, v3 - v0] > 0
        v = np.array(path, dtype=np.float64)
        if np.linalg.det(v[1:] - v[0]) < 0:
            slots[1], slots[2] = slots[2], slots[1]
        tets.append(slots)
    return np.array(tets, dtype=np.int64)


KUHN_TETS = _kuhn_tets()


def tet_box(shape, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
            periodic=(False, False, False), jitter: float = 0.0, seed: int = 0) -> Mesh:
    """nx x ny x nz hexes of box() each split into 6 Tet4 cells (Kuhn split,
    conforming across cells and across periodic boundaries).

    cell_nodes keeps 8 slots per cell: the 4 tetrahedron nodes in CGNS order
    followed by -1.  Faces use the local face numbering of TET_FACES; holders
    are the lower cell id of each interior face, boundary groups as in box().
    """
    hexes = box(shape, lengths, origin, periodic, jitter, seed)
    nx, ny, nz = hexes.shape
    L = np.asarray(hexes.lengths)
    cn = hexes.cell_nodes[:, KUHN_TETS].reshape(-1, 4)           # [6 * cells, 4]
    n_cells = cn.shape[0]
    cell_nodes = np.full((n_cells, 8), -1, dtype=np.int64)
    cell_nodes[:, :4] = cn
    # node lattice indices and periodic canonical ids
    nid = np.arange(hexes.xyz.shape[0], dtype=np.int64)
    ii = nid % (nx + 1)
    jj = (nid // (nx + 1)) % (ny + 1)
    kk = nid // ((nx + 1) * (ny + 1))
    ci = np.where(periodic[0], ii % nx, ii) if periodic[0] else ii
    cj = np.where(periodic[1], jj % ny, jj) if periodic[1] else jj
    ck = np.where(periodic[2], kk % nz, kk) if periodic[2] else kk
    canon = (ck * (ny + 1) + cj) * (nx + 1) + ci
    # all (cell, side) faces
    fn = cn[:, TET_FACES]                                        # [cells, 4, 3]
    cells = np.repeat(np.arange(n_cells, dtype=np.int64), 4)
    sides = np.tile(np.arange(4, dtype=np.int64), n_cells)
    fn = fn.reshape(-1, 3)
    key = np.sort(canon[fn], axis=1)
    order = np.lexsort((cells, key[:, 2], key[:, 1], key[:, 0]))
    key, cells, sides, fn = key[order], cells[order], sides[order], fn[order]
    same = np.all(key[1:] == key[:-1], axis=1)
    if np.any(same[1:] & same[:-1]):
        # three faces share one periodic node set: the wrap is too short to
        # tell the faces apart by their nodes
        raise ValueError("periodic tetrahedral box too small: use at least 3 cells along "
                         "all but one periodic axis")
    first = np.flatnonzero(same)                                 # pairs (first, first + 1)
    paired = np.zeros(key.shape[0], dtype=bool)
    paired[first] = True
    paired[first + 1] = True
    # interior faces: holder = lower cell id (the sort puts it first)
    h, s = cells[first], cells[first + 1]
    hs, ss = sides[first], sides[first + 1]
    ch = hexes.xyz[fn[first]].mean(axis=1)
    cs = hexes.xyz[fn[first + 1]].mean(axis=1)
    shift = np.round((ch - cs) / L) * L
    o = np.lexsort((hs, h))
    face_cells = [np.stack([h[o], s[o]], axis=1)]
    face_sides = [np.stack([hs[o], ss[o]], axis=1)]
    face_group = [np.full(o.size, -1)]
    face_shift = [shift[o]]
    # boundary faces: group from the plane that holds all three nodes
    lone = np.flatnonzero(~paired)
    if lone.size:
        bn = fn[lone]
        grp = np.full(lone.size, -1, dtype=np.int64)
        for ax, (idx, n) in enumerate(((ii, nx), (jj, ny), (kk, nz))):
            v = idx[bn]
            grp = np.where(np.all(v == 0, axis=1), 2 * ax, grp)
            grp = np.where(np.all(v == n, axis=1), 2 * ax + 1, grp)
        if np.any(grp < 0):
            raise ValueError("unmatched interior tetrahedron face")
        hb, sb = cells[lone], sides[lone]
        ob = np.lexsort((hb, grp))
        face_cells.append(np.stack([hb[ob], np.full(ob.size, -1)], axis=1))
        face_sides.append(np.stack([sb[ob], np.full(ob.size, -1)], axis=1))
        face_group.append(grp[ob])
        face_shift.append(np.zeros((ob.size, 3)))
    return Mesh(
        xyz=hexes.xyz,
        cell_nodes=cell_nodes,
        face_cells=np.ascontiguousarray(np.concatenate(face_cells).astype(np.int64)),
        face_sides=np.ascontiguousarray(np.concatenate(face_sides).astype(np.int32)),
        face_group=np.ascontiguousarray(np.concatenate(face_group).astype(np.int32)),
        face_shift=np.ascontiguousarray(np.concatenate(face_shift).astype(np.float64)),
        cell_type=np.full(n_cells, TET4, dtype=np.int32),
        shape=hexes.shape, lengths=hexes.lengths, origin=hexes.origin, periodic=hexes.periodic,
    )


def _split_box(hexes: Mesh, cells: np.ndarray, cell_type: int, xyz: np.ndarray, periodic, lengths) -> Mesh:
    """Faces of a split box through the connectivity builder: the unsplit
    box's boundary quadrangles (z faces split along their 0-2 diagonal for
    wedges) as boundary elements, periodic axes paired by shift."""
    full = box(hexes.shape, hexes.lengths, hexes.origin, (False, False, False))
    full.xyz = hexes.xyz
    bn, bg = boundary_elements(full)
    if cell_type == WEDGE6:
        tri = []
        grp = []
        for q, g in zip(bn, bg):
            if g in (4, 5):
                tri += [[q[0], q[1], q[2], -1], [q[0], q[2], q[3], -1]]
                grp += [g, g]
            else:
                tri.append(list(q))
                grp.append(g)
        bn, bg = np.array(tri, dtype=np.int64), np.array(grp, dtype=np.int32)
    pairs = []
    for ax in range(3):
        if periodic[ax]:
            shift = [0.0, 0.0, 0.0]
            shift[ax] = -float(lengths[ax])
            pairs.append((2 * ax, 2 * ax + 1, tuple(shift)))
    m = build(xyz, cells, np.full(cells.shape[0], cell_type, dtype=np.int32), bn, bg, periodic=pairs)
    m.shape, m.lengths, m.origin, m.periodic = hexes.shape, hexes.lengths, hexes.origin, tuple(periodic)
    return m


def wedge_box(shape, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
              periodic=(False, False, False), jitter: float = 0.0, seed: int = 0) -> Mesh:
    """nx x ny x nz hexes of box() each split into 2 Wedge6 cells along the
    (0, 2) diagonal of their z faces: (0, 1, 2, 4, 5, 6) and (0, 2, 3, 4, 6, 7)
    in CGNS order.  Faces from the connectivity builder; boundary groups as in
    box() (0 x-, 1 x+, 2 y-, 3 y+, 4 z-, 5 z+), periodic axes paired."""
    hexes = box(shape, lengths, origin, (False, False, False), jitter, seed)
    hc = hexes.cell_nodes
    cells = np.full((2 * hexes.n_cells, 8), -1, dtype=np.int64)
    cells[0::2, :6] = hc[:, [0, 1, 2, 4, 5, 6]]
    cells[1::2, :6] = hc[:, [0, 2, 3, 4, 6, 7]]
    return _split_box(hexes, cells, WEDGE6, hexes.xyz, periodic, hexes.lengths)


def pyramid_box(shape, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
                periodic=(False, False, False), jitter: float = 0.0, seed: int = 0) -> Mesh:
    """nx x ny x nz hexes of box() each split into 6 Pyra5 cells, one per hex
    face, with the apex at an added node (the mean of the hex's corners): the
    base of the pyramid on hex face (f0, f1, f2, f3) is (f0, f3, f2, f1), so
    its outward base normal is the hex face's.  Faces from the connectivity
    builder; boundary groups as in box(), periodic axes paired."""
    hexes = box(shape, lengths, origin, (False, False, False), jitter, seed)
    hc = hexes.cell_nodes
    n0 = hexes.xyz.shape[0]
    apex = hexes.xyz[hc].mean(axis=1)
    xyz = np.concatenate([hexes.xyz, apex])
    cells = np.full((6 * hexes.n_cells, 8), -1, dtype=np.int64)
    for s, f in enumerate(_HEX_FACES4):
        cells[s::6, :4] = hc[:, [f[0], f[3], f[2], f[1]]]
        cells[s::6, 4] = n0 + np.arange(hexes.n_cells)
    out = _split_box(hexes, cells, PYRA5, xyz, periodic, hexes.lengths)
    return out


def concat(*meshes: Mesh) -> Mesh:
    """Disjoint union of meshes (independent blocks in one description):
    node and cell ids are offset; boundary groups of block b become
    b * 6 + group."""
    xyz, cn, fc, fs, fg, fsh, ct = [], [], [], [], [], [], []
    n_off = c_off = 0
    stride = max(m.cell_nodes.shape[1] for m in meshes)
    for b, m in enumerate(meshes):
        xyz.append(m.xyz)
        nodes = np.full((m.n_cells, stride), -1, dtype=np.int64)
        nodes[:, :m.cell_nodes.shape[1]] = m.cell_nodes
        nodes[nodes >= 0] += n_off
        cn.append(nodes)
        f = m.face_cells.copy()
        f[f >= 0] += c_off
        fc.append(f)
        fs.append(m.face_sides)
        g = m.face_group.copy()
        g[g >= 0] += 6 * b
        fg.append(g)
        fsh.append(m.face_shift)
        ct.append(m.cell_type if m.cell_type is not None else np.full(m.n_cells, HEX8, dtype=np.int32))
        n_off += m.xyz.shape[0]
        c_off += m.n_cells
    return Mesh(
        xyz=np.ascontiguousarray(np.concatenate(xyz)),
        cell_nodes=np.ascontiguousarray(np.concatenate(cn)),
        face_cells=np.ascontiguousarray(np.concatenate(fc)),
        face_sides=np.ascontiguousarray(np.concatenate(fs)),
        face_group=np.ascontiguousarray(np.concatenate(fg)),
        face_shift=np.ascontiguousarray(np.concatenate(fsh)),
        cell_type=np.ascontiguousarray(np.concatenate(ct).astype(np.int32)),
        meta={"blocks": [m.n_cells for m in meshes]},
    )


# ---------------------------------------------------------------------------
# Mesh ingest through the library's connectivity builder (mcfd_build_faces)
# and the Hilbert cell order (mcfd_hilbert_order).

def build(xyz, cell_nodes, cell_type=None, bface_nodes=None, bface_group=None,
          periodic=(), device: int | None = None) -> Mesh:
    """Mesh with faces built from the cells alone (Part::BuildLocalFaces /
    BuildBoundaryFaces).  cell_nodes [cells, stride] (CGNS order);
    bface_nodes [n, 4] boundary elements (triangles end in -1) with groups
    bface_group; periodic: ((group_a, group_b, shift), ...) with
    x(face of b) + shift = x(face of a).  device: pair the face slots on that
    GPU (mcfd_build_faces_gpu; the same faces)."""
    import ctypes as C
    from . import capi
    lib = capi.load()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    cn = np.ascontiguousarray(cell_nodes, dtype=np.int64)
    ct = None if cell_type is None else np.ascontiguousarray(cell_type, dtype=np.int32)
    bf = np.ascontiguousarray(np.zeros((0, 4)) if bface_nodes is None else bface_nodes, dtype=np.int64)
    bg = np.ascontiguousarray(np.zeros(0) if bface_group is None else bface_group, dtype=np.int32)
    pg = np.ascontiguousarray([[a, b] for a, b, _ in periodic] or np.zeros((0, 2)), dtype=np.int32)
    ps = np.ascontiguousarray([list(s) for _, _, s in periodic] or np.zeros((0, 3)), dtype=np.float64)
    P64, P32, PD = C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_double)
    ct_p = None if ct is None else ct.ctypes.data_as(P32)
    cap = int(lib.mcfd_face_slot_count(cn.shape[0], ct_p))
    fc = np.empty((cap, 2), np.int64)
    fs = np.empty((cap, 2), np.int32)
    fg = np.empty(cap, np.int32)
    fsh = np.empty((cap, 3), np.float64)
    n = C.c_int64()
    fn = lib.mcfd_build_faces if device is None else \
        (lambda *a: lib.mcfd_build_faces_gpu(int(device), *a))
    rc = fn(xyz.shape[0], xyz.ctypes.data_as(PD), cn.shape[0], cn.ctypes.data_as(P64), ct_p,
                              cn.shape[1], bf.shape[0], bf.ctypes.data_as(P64), bg.ctypes.data_as(P32), pg.shape[0],
                              pg.ctypes.data_as(P32), ps.ctypes.data_as(PD), cap, fc.ctypes.data_as(P64),
                              fs.ctypes.data_as(P32), fg.ctypes.data_as(P32), fsh.ctypes.data_as(PD),
                              C.byref(n))
    if rc != 0:
        raise capi.McfdError(rc, (lib.mcfd_build_error() or b"").decode())
    k = n.value
    return Mesh(xyz=xyz, cell_nodes=cn, face_cells=np.ascontiguousarray(fc[:k]),
                face_sides=np.ascontiguousarray(fs[:k]), face_group=np.ascontiguousarray(fg[:k]),
                face_shift=np.ascontiguousarray(fsh[:k]), cell_type=ct)


def cell_centroids(m: Mesh) -> np.ndarray:
    """Mean of each cell's corner nodes (8 Hex, 4 Tet, 6 Wedge, 5 Pyramid)."""
    if m.cell_type is None:
        return m.xyz[m.cell_nodes[:, :8]].mean(axis=1)
    out = np.empty((m.n_cells, 3))
    fam = np.array([family(t) for t in m.cell_type])
    for name, k in CORNERS.items():
        sel = fam == name
        if sel.any():
            out[sel] = m.xyz[m.cell_nodes[sel, :k]].mean(axis=1)
    return out


def hilbert_order(m: Mesh) -> np.ndarray:
    """Cells in the order of a 3D Hilbert curve through their centroids."""
    import ctypes as C
    from . import capi
    pts = np.ascontiguousarray(cell_centroids(m), dtype=np.float64)
    order = np.empty(m.n_cells, dtype=np.int64)
    capi.check(capi.load().mcfd_hilbert_order(m.n_cells, pts.ctypes.data_as(C.POINTER(C.c_double)),
                                              order.ctypes.data_as(C.POINTER(C.c_int64))))
    return order


def renumber_cells(m: Mesh, order: np.ndarray) -> Mesh:
    """The same mesh with cell k of the result = cell order[k] of m; faces
    keep their holder / sharer roles and sides and are re-sorted by (new
    holder, side), boundary faces after interior ones by (group, holder).
    A column of m maps to the result by column.reshape(cells, -1)[order]."""
    order = np.asarray(order, dtype=np.int64)
    new_id = np.empty_like(order)
    new_id[order] = np.arange(order.size, dtype=np.int64)
    fc = m.face_cells.copy()
    fc[:, 0] = new_id[fc[:, 0]]
    fc[:, 1] = np.where(fc[:, 1] >= 0, new_id[np.maximum(fc[:, 1], 0)], -1)
    inner = fc[:, 1] >= 0
    grp = m.face_group.astype(np.int64)
    key_group = np.where(inner, -1, np.where(grp < 0, np.iinfo(np.int64).max, grp))
    o = np.lexsort((m.face_sides[:, 0], fc[:, 0], key_group, ~inner))
    return Mesh(xyz=m.xyz, cell_nodes=np.ascontiguousarray(m.cell_nodes[order]),
                face_cells=np.ascontiguousarray(fc[o]), face_sides=np.ascontiguousarray(m.face_sides[o]),
                face_group=np.ascontiguousarray(m.face_group[o]), face_shift=np.ascontiguousarray(m.face_shift[o]),
                cell_type=None if m.cell_type is None else np.ascontiguousarray(m.cell_type[order]),
                shape=m.shape, lengths=m.lengths, origin=m.origin, periodic=m.periodic)


def boundary_elements(m: Mesh) -> tuple[np.ndarray, np.ndarray]:
    """Boundary faces of m as element node lists [n, 4] (the holder's local
    face; triangles end in -1) and their groups."""
    b = m.face_cells[:, 1] < 0
    cells, sides = m.face_cells[b, 0], m.face_sides[b, 0]
    nodes = np.full((cells.size, 4), -1, dtype=np.int64)
    for i, (c, sd) in enumerate(zip(cells, sides)):
        row = CELL_FACES[family(HEX8 if m.cell_type is None else m.cell_type[c])][sd]
        k = 3 if row[3] < 0 else 4
        nodes[i, :k] = m.cell_nodes[c, row[:k]]
    return nodes, m.face_group[b].astype(np.int32)


# Quadratic cells in VTK node order: type -> (VTK type, the CGNS slot of each
# VTK node); the inverse of the reader's tables (csrc/vtk_reader.cpp).  VTK
# has no 14-node pyramid: Pyra14 cells are written by their corners.  The
# quadratic wedges follow the solution writer's Wedge15 (mesh/vtk.hpp): CGNS
# corners unflipped, bottom, top, then vertical mid-edges.
_VTK_QUADRATIC = {
    HEX20: (25, [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 16, 17, 18, 19, 12, 13, 14, 15]),
    HEX27: (29, [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 16, 17, 18, 19, 12, 13, 14, 15, 24, 22, 21, 23, 20, 25, 26]),
    TET10: (24, list(range(10))),
    WEDGE15: (26, [0, 1, 2, 3, 4, 5, 6, 7, 8, 12, 13, 14, 9, 10, 11]),
    WEDGE18: (32, [0, 1, 2, 3, 4, 5, 6, 7, 8, 12, 13, 14, 9, 10, 11, 15, 16, 17]),
    PYRA13: (27, list(range(13))),
}


def write_vtk(path, m: Mesh, binary: bool = False, classic: bool = False) -> None:
    """Legacy VTK unstructured grid of m: its cells by their corners (Hex8 ->
    12, Tet4 -> 10, Wedge6 -> 13 in VTK's node order, Pyra5 -> 14; the
    quadratic types in VTK's quadratic cells, Pyra14 by its corners), its boundary faces as
    quads / triangles (9 / 5) and a CELL_DATA int array "group" (-1 on volume
    cells).  Version-5 OFFSETS / CONNECTIVITY layout, or the classic CELLS
    layout with classic=True (ASCII only)."""
    bn, bg = boundary_elements(m)
    ct = np.zeros(m.n_cells, np.int32) if m.cell_type is None else np.asarray(m.cell_type)
    if np.any(ct == PYRA14):
        import warnings
        warnings.warn("write_vtk: VTK has no 14-node pyramid; Pyra14 cells are written by their 5 corners "
                      "and read back as straight-sided Pyra5 cells", stacklevel=2)
    conn, offs, types = [], [0], []
    for c in range(m.n_cells):
        t = int(ct[c])
        fam = family(t)
        if t in _VTK_QUADRATIC:
            vtk_type, cgns_of_vtk = _VTK_QUADRATIC[t]
            nodes = m.cell_nodes[c, cgns_of_vtk]
        elif fam == "wedge":
            nodes = m.cell_nodes[c, [0, 2, 1, 3, 5, 4]]
        else:
            nodes = m.cell_nodes[c, :CORNERS[fam]]
        conn.append(nodes); offs.append(offs[-1] + nodes.size)
        types.append(vtk_type if t in _VTK_QUADRATIC else {"tet": 10, "wedge": 13, "pyramid": 14}.get(fam, 12))
    for f in range(bn.shape[0]):
        k = 3 if bn[f, 3] < 0 else 4
        conn.append(bn[f, :k]); offs.append(offs[-1] + k); types.append(5 if k == 3 else 9)
    conn = np.concatenate(conn).astype(np.int64) if conn else np.zeros(0, np.int64)
    offs = np.asarray(offs, dtype=np.int64)
    types = np.asarray(types, dtype=np.int32)
    groups = np.concatenate([np.full(m.n_cells, -1, np.int32), bg]).astype(np.int32)
    n = types.size
    with open(path, "wb") as f:
        w = lambda s: f.write(s.encode())  # noqa: E731
        w("# vtk DataFile Version 5.1\nmesh written by pvcriemannsolvers_gb300\n")
        w("BINARY\n" if binary else "ASCII\n")
        w("DATASET UNSTRUCTURED_GRID\n")
        w(f"POINTS {m.xyz.shape[0]} double\n")
        if binary:
            f.write(np.ascontiguousarray(m.xyz, dtype=">f8").tobytes()); w("\n")
        else:
            w("\n".join(" ".join(repr(float(v)) for v in p) for p in m.xyz) + "\n")
        if classic:
            if binary:
                raise ValueError("the classic CELLS layout is written in ASCII only")
            w(f"CELLS {n} {n + conn.size}\n")
            for c in range(n):
                ids = conn[offs[c]:offs[c + 1]]
                w(f"{ids.size} " + " ".join(str(int(i)) for i in ids) + "\n")
        else:
            w(f"CELLS {n + 1} {conn.size}\n")
            for name, arr in (("OFFSETS", offs), ("CONNECTIVITY", conn)):
                w(f"{name} vtktypeint64\n")
                if binary:
                    f.write(np.ascontiguousarray(arr, dtype=">i8").tobytes()); w("\n")
                else:
                    w(" ".join(str(int(v)) for v in arr) + "\n")
        w(f"CELL_TYPES {n}\n")
        if binary:
            f.write(np.ascontiguousarray(types, dtype=">i4").tobytes()); w("\n")
        else:
            w("\n".join(str(int(t)) for t in types) + "\n")
        w(f"CELL_DATA {n}\nSCALARS group int 1\nLOOKUP_TABLE default\n")
        if binary:
            f.write(np.ascontiguousarray(groups, dtype=">i4").tobytes()); w("\n")
        else:
            w("\n".join(str(int(g)) for g in groups) + "\n")


def read_vtk(path, periodic=(), group_array: str | None = None) -> Mesh:
    """Mesh from a legacy VTK unstructured grid (mcfd_vtk_read) with faces
    from the library's connectivity builder; periodic as in build()."""
    import ctypes as C
    from . import capi
    lib = capi.load()
    h = C.c_void_p()
    rc = lib.mcfd_vtk_read(str(path).encode(), None if group_array is None else group_array.encode(), C.byref(h))
    if rc != 0:
        raise capi.McfdError(rc, (lib.mcfd_vtk_error() or b"").decode())
    try:
        nn, nc, nb = C.c_int64(), C.c_int64(), C.c_int64()
        capi.check(lib.mcfd_vtk_mesh_sizes(h, C.byref(nn), C.byref(nc), C.byref(nb)))
        xyz = np.empty((nn.value, 3))
        stride = C.c_int32()
        capi.check(lib.mcfd_vtk_mesh_stride(h, C.byref(stride)))
        cn = np.empty((nc.value, stride.value), np.int64)
        ct = np.empty(nc.value, np.int32)
        bf = np.empty((nb.value, 4), np.int64)
        bg = np.empty(nb.value, np.int32)
        P64, P32 = C.POINTER(C.c_int64), C.POINTER(C.c_int32)
        capi.check(lib.mcfd_vtk_mesh_arrays(h, xyz.ctypes.data_as(C.POINTER(C.c_double)), cn.ctypes.data_as(P64),
                                            ct.ctypes.data_as(P32), bf.ctypes.data_as(P64), bg.ctypes.data_as(P32)))
    finally:
        lib.mcfd_vtk_mesh_destroy(h)
    return build(xyz, cn, ct if np.any(ct != HEX8) else None, bf, bg, periodic)
