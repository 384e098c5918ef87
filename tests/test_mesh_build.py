"""Mesh ingest on the host (no GPU): the library's connectivity builder
(mcfd_build_faces, the faces of Part::BuildLocalFaces / BuildBoundaryFaces)
reproduces the generators' face tables index for index from cells and
boundary elements alone, and the Hilbert cell order (mcfd_hilbert_order)
is a locality-preserving permutation."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import capi, cases, mesh as meshlib

HEX_FACE = np.array([[0, 3, 2, 1], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [0, 4, 7, 3], [4, 5, 6, 7]])


def boundary_elements(m):
    """Boundary faces of m as element node lists (holder's local face) and groups."""
    b = m.face_cells[:, 1] < 0
    cells, sides = m.face_cells[b, 0], m.face_sides[b, 0]
    nodes = np.full((cells.size, 4), -1, dtype=np.int64)
    tet = np.zeros(cells.size, bool) if m.cell_type is None else m.cell_type[cells] == meshlib.TET4
    hx = ~tet
    nodes[hx] = m.cell_nodes[cells[hx][:, None], HEX_FACE[sides[hx]]]
    nodes[tet, :3] = m.cell_nodes[cells[tet][:, None], meshlib.TET_FACES[sides[tet]]]
    return nodes, m.face_group[b]


def periodic_spec(m, periodic):
    L = m.lengths
    return [(2 * ax, 2 * ax + 1, tuple(-L[ax] if e == ax else 0.0 for e in range(3)))
            for ax in range(3) if periodic[ax]]


def same_faces(a, b):
    assert np.array_equal(a.face_cells, b.face_cells)
    assert np.array_equal(a.face_sides, b.face_sides)
    assert np.array_equal(a.face_group, b.face_group)
    assert np.array_equal(a.face_shift, b.face_shift)


@pytest.mark.parametrize("maker", ["box", "tet_box"])
@pytest.mark.parametrize("periodic", [(False, False, False), (True, False, True), (True, True, True)])
def test_builder_reproduces_generators(maker, periodic):
    make = getattr(meshlib, maker)
    shape = (4, 3, 5) if maker == "box" else (3, 4, 3)
    open_mesh = make(shape, lengths=(1.0, 0.8, 1.3), jitter=0.1, seed=7)
    want = make(shape, lengths=(1.0, 0.8, 1.3), periodic=periodic, jitter=0.1, seed=7)
    bn, bg = boundary_elements(open_mesh)
    got = meshlib.build(open_mesh.xyz, open_mesh.cell_nodes, open_mesh.cell_type, bn, bg,
                        periodic_spec(want, periodic))
    same_faces(got, want)


def canonical(m):
    """Faces of m as a sorted table (concat orders them block by block)."""
    t = np.column_stack([m.face_cells, m.face_sides, m.face_group, m.face_shift])
    return t[np.lexsort(t[:, ::-1].T)]


def test_builder_concat_and_ungrouped():
    m = meshlib.concat(meshlib.box((2, 2, 2), jitter=0.1, seed=1), meshlib.tet_box((3, 3, 3), jitter=0.1, seed=2))
    bn, bg = boundary_elements(m)
    assert np.array_equal(canonical(meshlib.build(m.xyz, m.cell_nodes, m.cell_type, bn, bg)), canonical(m))
    # without boundary elements every free face comes out ungrouped
    got = meshlib.build(m.xyz, m.cell_nodes, m.cell_type)
    assert np.all(got.face_group[got.face_cells[:, 1] < 0] == -1)
    assert (got.face_cells[:, 1] >= 0).sum() == (m.face_cells[:, 1] >= 0).sum()


def test_builder_errors():
    m = meshlib.box((2, 2, 1))
    bn, bg = boundary_elements(m)
    with pytest.raises(capi.McfdError, match="more than two"):
        meshlib.build(m.xyz, np.concatenate([m.cell_nodes, m.cell_nodes[:1]]))
    inner_face = m.cell_nodes[0, HEX_FACE[2]][None, :]  # shared by cells 0 and 1
    with pytest.raises(capi.McfdError, match="not a free face"):
        meshlib.build(m.xyz, m.cell_nodes, None, inner_face, np.array([0], np.int32))
    with pytest.raises(capi.McfdError, match="no partner"):
        meshlib.build(m.xyz, m.cell_nodes, None, bn, bg, [(0, 1, (-0.5, 0.0, 0.0))])
    bad = m.cell_nodes.copy()
    bad[0, 0] = m.xyz.shape[0]
    with pytest.raises(capi.McfdError, match="out of range"):
        meshlib.build(m.xyz, bad)


def test_hilbert_order_corners_form_a_gray_path():
    pts = np.array([[i, j, k] for i in (0, 1) for j in (0, 1) for k in (0, 1)], dtype=float)
    m = meshlib.Mesh(xyz=pts, cell_nodes=np.repeat(np.arange(8)[:, None], 8, axis=1),
                     face_cells=np.zeros((0, 2), np.int64), face_sides=np.zeros((0, 2), np.int32),
                     face_group=np.zeros(0, np.int32), face_shift=np.zeros((0, 3)))
    order = meshlib.hilbert_order(m)
    assert sorted(order.tolist()) == list(range(8))
    steps = np.abs(np.diff(pts[order], axis=0)).sum(axis=1)
    assert np.all(steps == 1)  # consecutive octants share a face


def test_hilbert_order_locality():
    m = meshlib.box((16, 16, 16))
    rng = np.random.default_rng(0)
    shuffled = meshlib.renumber_cells(m, rng.permutation(m.n_cells))
    order = meshlib.hilbert_order(shuffled)
    assert np.array_equal(np.sort(order), np.arange(m.n_cells))
    h = meshlib.renumber_cells(shuffled, order)
    inner = h.face_cells[:, 1] >= 0
    gap_h = np.abs(h.face_cells[inner, 0] - h.face_cells[inner, 1]).mean()
    gap_s = np.abs(shuffled.face_cells[inner, 0] - shuffled.face_cells[inner, 1]).mean()
    assert gap_h < gap_s / 10


@pytest.mark.parametrize("kind", ["hex", "mixed"])
def test_renumbered_residual_is_permuted(kind):
    """The oracle's residual on the renumbered mesh is the permuted residual."""
    if kind == "hex":
        m = meshlib.box((4, 3, 3), periodic=(True, False, True), jitter=0.1, seed=3)
        p = 2
        u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
        order = meshlib.hilbert_order(m)[::-1].copy()
        r = orc.Mesh(m, p).residual(orc.RUSANOV, u)
        mm = meshlib.renumber_cells(m, order)
        r2 = orc.Mesh(mm, p).residual(orc.RUSANOV, u.reshape(m.n_cells, -1)[order].ravel())
    else:
        m = meshlib.concat(meshlib.box((2, 2, 2), periodic=(True,) * 3, jitter=0.1, seed=4),
                           meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.1, seed=5))
        om = orc.Modal(m, 2)
        u = om.project(cases.smooth_ic(om.points()[0]))
        order = np.random.default_rng(1).permutation(m.n_cells)
        r = om.residual(orc.HLLC, u)
        mm = meshlib.renumber_cells(m, order)
        r2 = orc.Modal(mm, 2).residual(orc.HLLC, u.reshape(m.n_cells, -1)[order].ravel())
    want = r.reshape(m.n_cells, -1)[order].ravel()
    assert np.linalg.norm(r2 - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.parametrize("fmt", ["ascii", "binary", "classic"])
@pytest.mark.parametrize("maker", ["box", "tet_box"])
def test_vtk_round_trip(tmp_path, fmt, maker):
    """A mesh written as legacy VTK and read back through mcfd_vtk_read +
    mcfd_build_faces has the generator's faces, periodic planes included."""
    make = getattr(meshlib, maker)
    periodic = (True, False, True)
    open_mesh = make((3, 4, 3), lengths=(1.0, 0.8, 1.3), jitter=0.1, seed=9)
    want = make((3, 4, 3), lengths=(1.0, 0.8, 1.3), periodic=periodic, jitter=0.1, seed=9)
    path = tmp_path / "m.vtk"
    meshlib.write_vtk(path, open_mesh, binary=fmt == "binary", classic=fmt == "classic")
    got = meshlib.read_vtk(path, periodic_spec(want, periodic))
    assert np.array_equal(got.xyz, open_mesh.xyz)
    assert np.array_equal(got.cell_nodes, open_mesh.cell_nodes)
    same_faces(got, want)


def test_vtk_reader_errors(tmp_path):
    bad = tmp_path / "bad.vtk"
    bad.write_text("not a vtk file\n")
    with pytest.raises(capi.McfdError, match="legacy VTK"):
        meshlib.read_vtk(bad)
    with pytest.raises(capi.McfdError, match="cannot open"):
        meshlib.read_vtk(tmp_path / "missing.vtk")
    m = meshlib.box((2, 1, 1))
    meshlib.write_vtk(bad, m)
    text = bad.read_text().replace("CELL_TYPES", "CELL_TYPEZ")
    bad.write_text(text)
    with pytest.raises(capi.McfdError, match="unexpected keyword"):
        meshlib.read_vtk(bad)


@pytest.mark.parametrize("serendipity", [False, True])
@pytest.mark.parametrize("maker", ["wedge_box", "pyramid_box"])
def test_builder_quadratic_wedges_and_pyramids(maker, serendipity):
    """Wedge15 / Wedge18 / Pyra13 / Pyra14 cells (corners first, in CGNS
    order) give the faces of their linear cells."""
    make = getattr(meshlib, maker)
    periodic = (True, False, True)
    open_mesh = make((3, 2, 2), lengths=(1.0, 0.8, 1.3), jitter=0.1, seed=7)
    want = make((3, 2, 2), lengths=(1.0, 0.8, 1.3), periodic=periodic, jitter=0.1, seed=7)
    q = meshlib.quadratic(open_mesh, serendipity=serendipity)
    want_type = {("wedge_box", True): 7, ("wedge_box", False): 8, ("pyramid_box", True): 9,
                 ("pyramid_box", False): 10}[(maker, serendipity)]
    assert set(np.unique(q.cell_type).tolist()) == {want_type}
    bn, bg = meshlib.boundary_elements(open_mesh)
    got = meshlib.build(q.xyz, q.cell_nodes, q.cell_type, bn, bg, periodic_spec(want, periodic))
    same_faces(got, want)


@pytest.mark.parametrize("maker", ["box", "tet_box", "wedge_box", "pyramid_box"])
@pytest.mark.parametrize("serendipity", [False, True])
def test_vtk_round_trip_quadratic(tmp_path, maker, serendipity):
    """Quadratic cells through the legacy VTK writer and reader: VTK 25 / 29
    hexahedra, 24 tetrahedra, 26 / 32 wedges and 27 pyramids come back in CGNS
    order with their types (Pyra14, which VTK lacks, is written by its
    corners and comes back as Pyra5)."""
    q = meshlib.quadratic(getattr(meshlib, maker)((3, 3, 2), jitter=0.1, seed=4), serendipity=serendipity)
    path = tmp_path / "q.vtk"
    if maker == "pyramid_box" and not serendipity:
        with pytest.warns(UserWarning, match="Pyra14 cells are written by their 5 corners"):
            meshlib.write_vtk(path, q)
    else:
        meshlib.write_vtk(path, q)
    got = meshlib.read_vtk(path)
    if maker == "pyramid_box" and not serendipity:
        assert np.all(got.cell_type == meshlib.PYRA5)
        assert np.array_equal(got.cell_nodes[:, :5], q.cell_nodes[:, :5])
    else:
        assert np.array_equal(got.cell_type, q.cell_type)
        assert np.array_equal(got.cell_nodes, q.cell_nodes)
    same_faces(got, q)


@pytest.mark.parametrize("maker", ["box", "tet_box", "wedge_box"])
def test_vtk_quadratic_order_matches_the_writer(maker):
    """The VTK orders of the quadratic cells are the orders in which the
    solution writer (mesh/vtk.hpp Hexahedron27 / Tetrahedron10 / Wedge15,
    restated by the oracle) emits its sample points: on an undeformed
    quadratic mesh node k of a cell in VTK order sits at sample point k."""
    m = getattr(meshlib, maker)((3, 3, 3), jitter=0.1, seed=5)
    q = meshlib.quadratic(m)
    om = orc.Modal(m, 1)
    u = om.project(cases.smooth_ic(om.points()[0]))
    xyz, _, types = om.vtk_sample(u)
    t = int(q.cell_type[0])
    _, order = meshlib._VTK_QUADRATIC[t]
    n = {29: 27, 24: 10, 26: 15}[int(types[0])]
    pts = xyz.reshape(m.n_cells, n, 3)
    want = q.xyz[q.cell_nodes[:, order[:n]]]
    assert np.allclose(pts, want, rtol=0, atol=1e-13)


def write_classic_vtk(path, xyz, cells):
    """A legacy ASCII VTK file written directly: cells = [(vtk type, node
    ids, group)], CELL_DATA "group"."""
    lines = ["# vtk DataFile Version 3.0", "hand-written", "ASCII", "DATASET UNSTRUCTURED_GRID",
             f"POINTS {len(xyz)} double"]
    lines += [" ".join(repr(float(v)) for v in p) for p in xyz]
    size = sum(1 + len(n) for _, n, _ in cells)
    lines.append(f"CELLS {len(cells)} {size}")
    lines += [" ".join(str(int(v)) for v in [len(n), *n]) for _, n, _ in cells]
    lines.append(f"CELL_TYPES {len(cells)}")
    lines += [str(t) for t, _, _ in cells]
    lines += [f"CELL_DATA {len(cells)}", "SCALARS group int 1", "LOOKUP_TABLE default"]
    lines += [str(g) for _, _, g in cells]
    path.write_text("\n".join(lines) + "\n")


# VTK_QUADRATIC_WEDGE / VTK_BIQUADRATIC_QUADRATIC_WEDGE in VTK's own layout:
# CGNS slot i of the cell is VTK node VTK_WEDGE_OF_CGNS[i] (corners flipped
# as for VTK_WEDGE, mid-edges and quadrangle centres following them).
VTK_WEDGE_OF_CGNS = [0, 2, 1, 3, 5, 4, 8, 7, 6, 12, 14, 13, 11, 10, 9, 17, 16, 15]


def corner_wedge_volume(xyz, nodes):
    x0, x1, x2, x3 = (xyz[nodes[i]] for i in range(4))
    return float(np.dot(np.cross(x1 - x0, x2 - x0), x3 - x0))


@pytest.mark.parametrize("serendipity", [False, True])
def test_vtk_quadratic_wedges_in_vtk_layout(tmp_path, serendipity):
    """Quadratic wedges as ParaView, gmsh or meshio write them (VTK 26 / 32
    with VTK_WEDGE's corner orientation) and quadratic boundary elements
    (VTK 22 triangles, 23 / 28 quadrangles) come back in CGNS order with
    positive volumes, the same faces and the boundary groups."""
    m = meshlib.wedge_box((3, 2, 2), jitter=0.1, seed=9)
    q = meshlib.quadratic(m, serendipity=serendipity)
    n = 15 if serendipity else 18
    vtk_type = 26 if serendipity else 32
    cells = []
    for c in range(q.n_cells):
        vtk_nodes = np.empty(n, np.int64)
        vtk_nodes[VTK_WEDGE_OF_CGNS[:n]] = q.cell_nodes[c, :n]
        cells.append((vtk_type, vtk_nodes, -1))
    bn, bg = meshlib.boundary_elements(m)
    for nodes, g in zip(bn, bg):
        if nodes[3] < 0:  # quadratic triangle: corners, then any three mid-edge ids
            cells.append((22, [*nodes[:3], *nodes[:3]], int(g)))
        else:  # quadratic and biquadratic quadrangles
            cells.append((23 if g % 2 else 28, [*nodes, *nodes] + ([nodes[0]] if g % 2 == 0 else []), int(g)))
    cells.append((3, [0, 1], -1))  # a line: skipped
    path = tmp_path / "w.vtk"
    write_classic_vtk(path, q.xyz, cells)
    got = meshlib.read_vtk(path)
    assert np.array_equal(got.cell_nodes[:, :n], q.cell_nodes[:, :n])
    assert np.array_equal(got.cell_type, q.cell_type)
    assert all(corner_wedge_volume(got.xyz, got.cell_nodes[c]) > 0 for c in range(got.n_cells))
    same_faces(got, q)


def test_vtk_reader_rejects_unsupported_cells(tmp_path):
    m = meshlib.box((1, 1, 1))
    path = tmp_path / "u.vtk"
    write_classic_vtk(path, m.xyz, [(12, m.cell_nodes[0], -1), (38, list(range(8)), -1)])
    with pytest.raises(capi.McfdError, match="unsupported VTK cell type 38 with 8 nodes"):
        meshlib.read_vtk(path)
    write_classic_vtk(path, m.xyz, [(29, list(range(8)) * 2 + [0, 1, 2, 3], -1)])
    with pytest.raises(capi.McfdError, match="unsupported VTK cell type 29 with 20 nodes"):
        meshlib.read_vtk(path)
