"""The oracle's modal DG restatement (dg::General over Projection) on Hex8,
Tet4, Wedge6 and Pyra5 cells: quadrature exactness of the rules it uses,
orthonormality of the per-cell basis, projection exactness and free-stream
preservation.

Reference tests this mirrors: test/integrator/{hexahedron,tetrahedron,
triangle}.cpp (rule exactness), test/polynomial/projection.cpp (projection of
polynomials is exact), test/basis/linear.cpp (orthonormality).
"""
import math

import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import cases, mesh as meshlib


def _mesh(kind, periodic=(True, True, True), jitter=0.1, shape=(3, 3, 2), seed=3):
    if kind == "hex":
        return meshlib.box(shape, lengths=(1.0, 1.0, 1.0), periodic=periodic, jitter=jitter, seed=seed)
    if kind == "tet":
        return meshlib.tet_box(shape, lengths=(1.0, 1.0, 1.0), periodic=periodic, jitter=jitter, seed=seed)
    if kind == "wedge":
        return meshlib.wedge_box(shape, lengths=(1.0, 1.0, 1.0), periodic=periodic, jitter=jitter, seed=seed)
    if kind == "pyramid":
        return meshlib.pyramid_box(shape, lengths=(1.0, 1.0, 1.0), periodic=periodic, jitter=jitter, seed=seed)
    if kind == "all":
        blocks = [meshlib.box, meshlib.tet_box, meshlib.wedge_box, meshlib.pyramid_box]
        return meshlib.concat(*[fn(shape, lengths=(1.0, 1.0, 1.0), origin=(2.0 * i, 0.0, 0.0), periodic=periodic,
                                   jitter=jitter, seed=seed + i) for i, fn in enumerate(blocks)])
    a = meshlib.box(shape, lengths=(1.0, 1.0, 1.0), periodic=periodic, jitter=jitter, seed=seed)
    b = meshlib.tet_box(shape, lengths=(1.0, 1.0, 1.0), origin=(2.0, 0.0, 0.0), periodic=periodic,
                        jitter=jitter, seed=seed + 1)
    return meshlib.concat(a, b)


def _monomial_integral_unit_tet(e):
    # int over {x, y, z >= 0, x + y + z <= 1} of x^a y^b z^c = a! b! c! / (a + b + c + 3)!
    a, b, c = e
    return math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 3)


@pytest.mark.parametrize("p,degree", [(2, 5), (3, 6)])
def test_tet_rule_exactness(p, degree):
    """A single unit tetrahedron (affine map = identity on its first three
    barycentric axes) integrates every monomial up to the rule's degree."""
    xyz = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0], [0, 0, 0]])
    # CGNS-positive order: det[N1 - N0, N2 - N0, N3 - N0] > 0
    cn = np.array([[3, 0, 1, 2, -1, -1, -1, -1]], dtype=np.int64)
    m = meshlib.Mesh(xyz=xyz, cell_nodes=cn, face_cells=np.zeros((0, 2), np.int64),
                     face_sides=np.zeros((0, 2), np.int32), face_group=np.zeros(0, np.int32),
                     face_shift=np.zeros((0, 3)), cell_type=np.array([1], np.int32))
    o = orc.Modal(m, p)
    x, w = o.points()
    assert abs(w.sum() - 1 / 6) < 1e-15
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            for c in range(degree + 1 - a - b):
                got = float((w * x[:, 0] ** a * x[:, 1] ** b * x[:, 2] ** c).sum())
                assert abs(got - _monomial_integral_unit_tet((a, b, c))) < 1e-15, (a, b, c)


@pytest.mark.parametrize("p,degree", [(2, 4), (3, 6)])
def test_triangle_rule_exactness(p, degree):
    """The face rule on a tet face: integrate monomials over the boundary
    triangle z = 0 of the unit tetrahedron."""
    m = meshlib.tet_box((1, 1, 1), periodic=(False,) * 3)
    o = orc.Modal(m, p)
    fx, fw, fr = o.face_points()
    nf = len(fw) // m.n_faces
    # faces on the z = 0 plane: group 4
    sel = np.flatnonzero(m.face_group == 4)
    idx = (sel[:, None] * nf + np.arange(nf)[None, :]).ravel()
    x, w = fx[idx], fw[idx]
    assert abs(w.sum() - 1.0) < 1e-14
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            want = 1 / (a + 1) / (b + 1)   # over the unit square = two triangles
            got = float((w * x[:, 0] ** a * x[:, 1] ** b).sum())
            assert abs(got - want) < 1e-14, (a, b)
    # normals of that group point out of the box (-z)
    assert np.allclose(fr[idx, 0, :], [0, 0, -1])


@pytest.mark.parametrize("kind", ["hex", "tet", "mixed", "wedge", "pyramid", "all"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_projection_of_polynomials_is_exact(kind, p):
    """Projecting a polynomial of degree <= p and evaluating it back returns
    it at every quadrature point (the basis spans P_p; projection.hpp:28-42)."""
    m = _mesh(kind)
    o = orc.Modal(m, p)
    x, _ = o.points()
    rng = np.random.default_rng(p)
    vals = np.zeros((o.n_points, 5))
    for k in range(5):
        c = rng.uniform(-1, 1, 4)
        vals[:, k] = c[0] + c[1] * x[:, 0] ** p + c[2] * x[:, 1] * x[:, 2] ** (p - 1) + c[3] * x[:, 2]
    u = o.project(vals)
    back = o.values(u)
    assert np.abs(back - vals).max() < 1e-12 * max(1.0, np.abs(vals).max())


@pytest.mark.parametrize("kind", ["hex", "tet", "mixed", "wedge", "pyramid", "all"])
def test_free_stream_preservation(kind):
    """A uniform state has a zero residual (closed cells, consistent fluxes)."""
    m = _mesh(kind)
    for p in (1, 2, 3):
        o = orc.Modal(m, p)
        prim = np.tile([1.0, 0.3, -0.2, 0.5, 1.0], (o.n_points, 1))
        u = o.project(cases.prim_to_cons(*prim.T))
        for riemann in (orc.RUSANOV, orc.ROE, orc.HLLC, orc.AUSM):
            assert np.abs(o.residual(riemann, u)).max() < 1e-12


def test_tet_mesh_is_conforming_and_oriented():
    m = meshlib.tet_box((3, 2, 2), periodic=(True, False, True), jitter=0.1)
    cnt = np.bincount(m.face_cells[:, 0], minlength=m.n_cells)
    cnt += np.bincount(m.face_cells[m.face_cells[:, 1] >= 0, 1], minlength=m.n_cells)
    assert set(cnt.tolist()) == {4}
    x = m.xyz[m.cell_nodes[:, :4]]
    det = np.linalg.det(np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], 1))
    assert det.min() > 0
    # periodic faces carry a shift of one box length along x or z only
    sh = m.face_shift[m.face_group < 0]
    assert set(np.unique(np.round(sh, 12)).tolist()) <= {-1.0, 0.0}
    assert np.all(sh[:, 1] == 0)


def test_tet_box_rejects_ambiguous_periodic_wrap():
    with pytest.raises(ValueError):
        meshlib.tet_box((2, 2, 2), periodic=(True,) * 3)


def _single_cell(xyz, cell_type):
    """one cell with its faces as boundary elements (group 0)"""
    xyz = np.asarray(xyz, dtype=np.float64)
    fam = meshlib.family(cell_type)
    cells = np.full((1, 8), -1, dtype=np.int64)
    cells[0, :xyz.shape[0]] = np.arange(xyz.shape[0])
    bn = np.array([[r[0], r[1], r[2], r[3]] if r[3] >= 0 else [r[0], r[1], r[2], -1]
                   for r in meshlib.CELL_FACES[fam]], dtype=np.int64)
    return meshlib.build(xyz, cells, np.array([cell_type], np.int32), bn, np.zeros(bn.shape[0], np.int32))


@pytest.mark.parametrize("p", [1, 2, 3])
def test_wedge_and_pyramid_integrators(p):
    """test/integrator/wedge.cpp: the wedge on (-1,-1), (1,-1), (0,1) times
    [-1, 1] has volume 4; test/integrator/pyramid.cpp: the pyramid on the
    4 x 6 base at z = 0 with its apex at height 4 has volume 4 a b h / 3 = 32."""
    w = _single_cell([(-1, -1, -1), (1, -1, -1), (0, 1, -1), (-1, -1, 1), (1, -1, 1), (0, 1, 1)],
                     meshlib.WEDGE6)
    o = orc.Modal(w, p)
    _, wt = o.points()
    assert abs(wt.sum() - 4.0) < 1e-13
    a, b, h = 2.0, 3.0, 4.0
    pm = _single_cell([(-a, -b, 0), (a, -b, 0), (a, b, 0), (-a, b, 0), (0, 0, h)], meshlib.PYRA5)
    o = orc.Modal(pm, p)
    x, wt = o.points()
    assert abs(wt.sum() - 4 * a * b * h / 3) < 1e-12
    # the centroid of the pyramid is at h / 4 over the base
    assert abs((wt * x[:, 2]).sum() / wt.sum() - h / 4) < 1e-12


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_gauss_jacobi_rule_exactness(n):
    """integrator/jacobi.hpp (alpha 2, beta 0): sum w_i x_i^k equals
    int_{-1}^{1} (1 - x)^2 x^k dx for k <= 2n - 1."""
    lib = orc.load()
    lib.orc_gauss_jacobi20.restype = None
    lib.orc_gauss_jacobi20.argtypes = [orc.C.c_int, orc._D, orc._D]
    x, w = np.zeros(n), np.zeros(n)
    lib.orc_gauss_jacobi20(n, orc._p(x), orc._p(w))
    assert np.all(np.diff(x) > 0) and np.all(np.abs(x) < 1)
    for k in range(2 * n):
        exact = sum(c * (2.0 / (k + e + 1) if (k + e) % 2 == 0 else 0.0)
                    for c, e in ((1.0, 0), (-2.0, 1), (1.0, 2)))
        assert abs((w * x ** k).sum() - exact) < 1e-13


@pytest.mark.parametrize("kind", ["wedge", "pyramid"])
def test_split_boxes_tile_the_box(kind):
    """Cell volumes of the wedge and pyramid splits of a jittered box add up
    to the box (the rules integrate the maps' Jacobians exactly)."""
    m = _mesh(kind, periodic=(False, False, False))
    for p in (1, 2, 3):
        _, wt = orc.Modal(m, p).points()
        assert wt.min() > 0
        assert abs(wt.sum() - 1.0) < 1e-13
