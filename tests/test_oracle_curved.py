"""Curved cells in the oracle (Hex27 / Hex20 / Tet10 maps): an undeformed
quadratic mesh is the straight mesh, a volume-preserving shear keeps every
cell's volume, and a deformed periodic mesh stays conservative."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import cases, mesh as meshlib


def shear(eps=0.05, L=1.0):
    """x + eps sin(2 pi y / L): det J = 1, periodic in y (and x, z)."""
    def fn(x):
        y = x.copy()
        y[:, 0] += eps * np.sin(2 * np.pi * x[:, 1] / L)
        return y
    return fn


def wavy(eps=0.03, L=1.0):
    """A smooth periodic deformation of the unit box."""
    def fn(x):
        s = np.sin(2 * np.pi * x / L)
        y = x.copy()
        y[:, 0] += eps * s[:, 1] * s[:, 2]
        y[:, 1] += eps * s[:, 2] * s[:, 0]
        y[:, 2] += eps * s[:, 0] * s[:, 1]
        return y
    return fn


@pytest.mark.parametrize("serendipity", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_undeformed_quadratic_is_straight(p, serendipity):
    m = meshlib.box((3, 2, 2), periodic=(True, False, True), jitter=0.1, seed=2)
    q = meshlib.quadratic(m, serendipity=serendipity)
    u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    bcs = {2: (orc.BC_SMART, cases.SOD_LEFT), 3: (orc.BC_INVISCID_WALL, None)}
    a, b = orc.Mesh(m, p), orc.Mesh(q, p)
    a.set_bcs(bcs)
    b.set_bcs(bcs)
    r = a.residual(orc.ROE, u)
    assert np.linalg.norm(b.residual(orc.ROE, u) - r) <= 1e-12 * np.linalg.norm(r)


def test_undeformed_quadratic_modal_is_straight():
    m = meshlib.concat(meshlib.box((2, 2, 2), periodic=(True,) * 3, jitter=0.1, seed=3),
                       meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.1, seed=4))
    q = meshlib.quadratic(m)
    a, b = orc.Modal(m, 2), orc.Modal(q, 2)
    u = a.project(cases.smooth_ic(a.points()[0]))
    assert np.allclose(b.points()[0], a.points()[0], rtol=0, atol=1e-13)
    r = a.residual(orc.HLLC, u)
    assert np.linalg.norm(b.residual(orc.HLLC, u) - r) <= 1e-11 * np.linalg.norm(r)


@pytest.mark.parametrize("serendipity", [False, True])
def test_shear_keeps_volume(serendipity):
    m = meshlib.quadratic(meshlib.box((4, 4, 3), periodic=(True,) * 3), serendipity=serendipity)
    d = meshlib.deform(m, shear())
    for p in (1, 2, 3):
        _, w = orc.Mesh(d, p).node_geometry()
        assert np.allclose(w.sum(axis=1), 1.0 / 48, rtol=1e-13)
    om = orc.Modal(d, 2)
    assert abs(om.points()[1].sum() - 1.0) < 1e-13


@pytest.mark.parametrize("p", [2, 3])
def test_deformed_periodic_mesh_is_conservative(p):
    d = meshlib.deform(meshlib.quadratic(meshlib.box((3, 3, 3), periodic=(True,) * 3)), wavy())
    om = orc.Mesh(d, p)
    u = cases.smooth_ic(meshlib.node_coordinates(d, p).reshape(-1, 3)).ravel()
    r = om.residual(orc.RUSANOV, u).reshape(d.n_cells, -1, 5)
    _, w = om.node_geometry()
    total = np.einsum("cn,cnk->k", w, r)
    scale = np.einsum("cn,cnk->k", w, np.abs(r))
    assert np.all(np.abs(total) <= 1e-12 * scale)
    mm = meshlib.deform(meshlib.quadratic(meshlib.concat(
        meshlib.box((2, 2, 2), periodic=(True,) * 3), meshlib.tet_box((3, 3, 3), periodic=(True,) * 3))),
        wavy(0.02))
    o2 = orc.Modal(mm, p)
    uu = o2.project(cases.smooth_ic(o2.points()[0]))
    # the mean of each conserved variable changes only through faces, which
    # cancel: coefficient 0 of the orthonormal basis times the cell's volume^1/2
    rr = o2.residual(orc.HLLC, uu).reshape(mm.n_cells, -1, 5)
    x, w = o2.points()
    off = np.concatenate([[0], np.cumsum([(p + 1) ** 3 if t in (0, 2) else (14 if p <= 2 else 24)
                                          for t in mm.cell_type])])
    vol = np.array([w[off[c]:off[c + 1]].sum() for c in range(mm.n_cells)])
    total = (rr[:, 0, :] * np.sqrt(vol)[:, None]).sum(axis=0)
    assert np.all(np.abs(total) <= 1e-10 * np.abs(rr[:, 0, :] * np.sqrt(vol)[:, None]).sum(axis=0))


def _wedge_pyramid_blocks(jitter=0.1):
    return (meshlib.wedge_box((2, 2, 2), periodic=(True,) * 3, jitter=jitter, seed=3),
            meshlib.pyramid_box((2, 2, 2), periodic=(True,) * 3, jitter=jitter, seed=4))


@pytest.mark.parametrize("serendipity", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_undeformed_quadratic_wedge_pyramid_is_straight(p, serendipity):
    """Wedge15 / Wedge18 / Pyra13 / Pyra14 with their new nodes at the
    averages of the corners reproduce the straight Wedge6 / Pyra5 cells: the
    hierarchical maps interpolate every function of the linear span."""
    for m in _wedge_pyramid_blocks():
        q = meshlib.quadratic(m, serendipity=serendipity)
        a, b = orc.Modal(m, p), orc.Modal(q, p)
        assert np.allclose(b.points()[0], a.points()[0], rtol=0, atol=1e-13)
        assert np.allclose(b.points()[1], a.points()[1], rtol=1e-12, atol=0)
        u = a.project(cases.smooth_ic(a.points()[0]))
        r = a.residual(orc.HLLC, u)
        assert np.linalg.norm(b.residual(orc.HLLC, u) - r) <= 1e-12 * np.linalg.norm(r)


@pytest.mark.parametrize("serendipity", [False, True])
def test_quadratic_wedge_pyramid_integrators(serendipity):
    """test/integrator/wedge.cpp (Wedge15 / Wedge18 on the prism of volume 4)
    and test/integrator/pyramid.cpp (Pyramid13 / Pyramid14 on the 4 x 6 base,
    apex at height 4: volume 32), their node lists as in those tests."""
    wx = [(-1, -1, -1), (1, -1, -1), (0, 1, -1), (-1, -1, 1), (1, -1, 1), (0, 1, 1),
          (0, -1, -1), (0.5, 0, -1), (-0.5, 0, -1), (-1, -1, 0), (1, -1, 0), (0, 1, 0),
          (0, -1, 1), (0.5, 0, 1), (-0.5, 0, 1)]
    a, b, h = 2.0, 3.0, 4.0
    px = [(-a, -b, 0), (a, -b, 0), (a, b, 0), (-a, b, 0), (0, 0, h), (0, -b, 0), (a, 0, 0),
          (0, b, 0), (-a, 0, 0), (-a / 2, -b / 2, h / 2), (a / 2, -b / 2, h / 2),
          (a / 2, b / 2, h / 2), (-a / 2, b / 2, h / 2)]
    if not serendipity:
        wx += [(0, -1, 0), (0.5, 0, 0), (-0.5, 0, 0)]
        px += [(0, 0, 0)]
    w = _single_cell(wx, meshlib.WEDGE15 if serendipity else meshlib.WEDGE18)
    pm = _single_cell(px, meshlib.PYRA13 if serendipity else meshlib.PYRA14)
    for p in (1, 2, 3):
        assert abs(orc.Modal(w, p).points()[1].sum() - 4.0) < 1e-13
        x, wt = orc.Modal(pm, p).points()
        assert abs(wt.sum() - 4 * a * b * h / 3) < 1e-12
        assert abs((wt * x[:, 2]).sum() / wt.sum() - h / 4) < 1e-12


def _single_cell(xyz, cell_type):
    """one cell with its faces as boundary elements (group 0)"""
    xyz = np.asarray(xyz, dtype=np.float64)
    fam = meshlib.family(cell_type)
    cells = np.full((1, max(8, xyz.shape[0])), -1, dtype=np.int64)
    cells[0, :xyz.shape[0]] = np.arange(xyz.shape[0])
    bn = meshlib.CELL_FACES[fam]
    return meshlib.build(xyz, cells, np.array([cell_type], np.int32), bn, np.zeros(bn.shape[0], np.int32))


@pytest.mark.parametrize("serendipity", [False, True])
def test_deformed_quadratic_wedge_pyramid_meshes(serendipity):
    """Sheared periodic Wedge15/18 and Pyra13/14 meshes keep the box's volume
    and are conservative; at p = 1 they keep a free stream to rounding (the
    faces' own Triangle6 / Quadrangle8 / 9 maps close each cell exactly)."""
    fs = np.array([1.0, 0.3, 0.2, 0.1, 2.5])
    for gen in (meshlib.wedge_box, meshlib.pyramid_box):
        d = meshlib.deform(meshlib.quadratic(gen((4, 4, 3), periodic=(True,) * 3), serendipity=serendipity),
                           shear())
        om = orc.Modal(d, 1)
        assert abs(om.points()[1].sum() - 1.0) < 1e-13
        u = om.project(np.tile(fs, (om.points()[0].shape[0], 1)))
        assert np.abs(om.residual(orc.HLLC, u)).max() < 1e-12
        o2 = orc.Modal(d, 2)
        uu = o2.project(cases.smooth_ic(o2.points()[0]))
        rr = o2.residual(orc.HLLC, uu).reshape(d.n_cells, -1, 5)
        ctr, wt = o2.points()
        # mode 0 is the constant 1 / sqrt(volume): its residual times sqrt(volume) sums to 0
        npts = wt.size // d.n_cells
        vol = wt.reshape(d.n_cells, npts).sum(axis=1)
        total = (rr[:, 0, :] * np.sqrt(vol)[:, None]).sum(axis=0)
        assert np.abs(total).max() < 1e-12 * np.abs(rr[:, 0, :] * np.sqrt(vol)[:, None]).sum()
