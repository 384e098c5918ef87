"""Meshes from the connectivity builder and renumbered cells on the GPU: the
residual and a few SSP-RK3 steps on a Hilbert-renumbered mesh are the
permuted results of the original numbering, and a builder-made mesh runs
exactly like the generator's."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import General, Lobatto, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_renumbered_dgsem(precision):
    m = meshlib.box((6, 5, 4), periodic=(True, False, True), jitter=0.1, seed=3)
    p = 3
    u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    rng = np.random.default_rng(2)
    shuffled = meshlib.renumber_cells(m, rng.permutation(m.n_cells))
    for order in (meshlib.hilbert_order(m), rng.permutation(m.n_cells)):
        mm = meshlib.renumber_cells(m, order)
        a, b = Lobatto(m, p, "rusanov", precision=precision), Lobatto(mm, p, "rusanov", precision=precision)
        for s in (a, b):
            s.SetSmartBoundary(2, cases.SOD_LEFT)
            s.SetInviscidWall(3)
        a.SetSolutionColumn(u)
        b.SetSolutionColumn(u.reshape(m.n_cells, -1)[order].ravel())
        ra = a.GetResidualColumn().reshape(m.n_cells, -1)[order].ravel()
        assert rel(b.GetResidualColumn(), ra) <= 1e-14
        ta = a.advance(3, 1e9, 3, 0.0)
        tb = b.advance(3, 1e9, 3, 0.0)
        assert ta == tb
        ua = a.GetSolutionColumn().reshape(m.n_cells, -1)[order].ravel()
        assert rel(b.GetSolutionColumn(), ua) <= 1e-13
        a.close()
        b.close()
    assert shuffled.n_cells == m.n_cells


def test_builder_mesh_against_oracle():
    open_mesh = meshlib.tet_box((3, 3, 4), jitter=0.1, seed=5)
    b = open_mesh.face_cells[:, 1] < 0
    nodes = np.full((b.sum(), 4), -1, dtype=np.int64)
    nodes[:, :3] = open_mesh.cell_nodes[open_mesh.face_cells[b, 0][:, None],
                                        meshlib.TET_FACES[open_mesh.face_sides[b, 0]]]
    m = meshlib.build(open_mesh.xyz, open_mesh.cell_nodes, open_mesh.cell_type, nodes, open_mesh.face_group[b],
                      [(0, 1, (-1.0, 0.0, 0.0)), (4, 5, (0.0, 0.0, -1.0))])
    m = meshlib.renumber_cells(m, meshlib.hilbert_order(m))
    g = General(m, 2, "hllc")
    om = orc.Modal(m, 2)
    u = om.project(cases.smooth_ic(om.points()[0]))
    g.SetSolutionColumn(u)
    assert rel(g.GetResidualColumn(), om.residual(orc.HLLC, u)) <= 1e-12
    g.close()
