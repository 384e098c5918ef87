"""Curved cells on the GPU (Hex27 / Hex20 for the nodal schemes, Hex27 +
Tet10 for the modal scheme) against the oracle's restatement of the same
maps: residuals and SSP-RK3 steps to 1e-12, VTK samples, and the straight
equivalence of undeformed quadratic meshes."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import General, Lobatto, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def wavy(eps=0.03):
    def fn(x):
        s = np.sin(2 * np.pi * x)
        y = x.copy()
        y[:, 0] += eps * s[:, 1] * s[:, 2]
        y[:, 1] += eps * s[:, 2] * s[:, 0]
        y[:, 2] += eps * s[:, 0] * s[:, 1]
        return y
    return fn


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def nodal_mesh(serendipity):
    m = meshlib.box((4, 3, 3), periodic=(True, False, True), jitter=0.05, seed=5)
    return meshlib.deform(meshlib.quadratic(m, serendipity=serendipity), wavy())


@pytest.mark.parametrize("scheme", ["dgsem", "fr"])
@pytest.mark.parametrize("serendipity", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_curved_nodal_parity(p, serendipity, scheme):
    m = nodal_mesh(serendipity)
    s = Lobatto(m, p, "roe", scheme=scheme)
    om = orc.Mesh(m, p, scheme=scheme)
    s.SetSmartBoundary(2, cases.SOD_LEFT)
    s.SetInviscidWall(3)
    om.set_bcs({2: (orc.BC_SMART, cases.SOD_LEFT), 3: (orc.BC_INVISCID_WALL, None)})
    u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s.SetSolutionColumn(u)
    assert rel(s.GetResidualColumn(), om.residual(orc.ROE, u)) <= 1e-12
    dt = om.time_step(u, 1.0, 3)
    assert abs(s.GetTimeStep(1.0, 3) - dt) <= 1e-14 * dt
    s.close()


@pytest.mark.parametrize("p", [1, 2, 3])
def test_curved_rk3_step(p):
    from pvcriemannsolvers_gb300 import RungeKutta
    m = nodal_mesh(False)
    s = Lobatto(m, p, "hllc")
    om = orc.Mesh(m, p)
    s.SetInviscidWall(2)
    s.SetInviscidWall(3)
    om.set_bcs({2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None)})
    u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s.SetSolutionColumn(u)
    dt = om.time_step(u, 1.0, 3)
    RungeKutta(3).Update(s, 0.0, dt)
    assert rel(s.GetSolutionColumn(), om.rk_update(orc.HLLC, 3, 0.0, dt, u)) <= 1e-12
    s.close()


@pytest.mark.parametrize("p", [1, 2, 3])
def test_curved_modal_parity(p):
    m = meshlib.deform(meshlib.quadratic(meshlib.concat(
        meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=1),
        meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=2))), wavy(0.02))
    g = General(m, p, "hllc")
    om = orc.Modal(m, p)
    assert np.allclose(g.points(), om.points()[0], rtol=0, atol=1e-13)
    u = om.project(cases.smooth_ic(om.points()[0]))
    g.SetSolutionColumn(u)
    assert rel(g.GetResidualColumn(), om.residual(orc.HLLC, u)) <= 1e-12
    dt = om.time_step(u, 1.0, 3)
    g.advance(1, dt, 3, 0.0)
    u1 = om.rk_update(orc.HLLC, 3, 0.0, dt, u)
    assert rel(g.GetSolutionColumn(), u1) <= 1e-12
    xyz, values, types = g.vtk_sample()
    oxyz, ovalues, otypes = om.vtk_sample(g.GetSolutionColumn())
    assert np.array_equal(types, otypes)
    assert rel(xyz, oxyz) <= 1e-14 and rel(values, ovalues) <= 1e-13
    g.close()


def test_curved_vtk_sample_nodal():
    m = nodal_mesh(False)
    s = Lobatto(m, 2, "rusanov")
    om = orc.Mesh(m, 2)
    u = cases.smooth_ic(meshlib.node_coordinates(m, 2).reshape(-1, 3)).ravel()
    s.SetSolutionColumn(u)
    xyz, values, _ = s.vtk_sample()
    oxyz, ovalues, _ = om.vtk_sample(u)
    assert rel(xyz, oxyz) <= 1e-14 and rel(values, ovalues) <= 1e-13
    s.close()


def test_undeformed_quadratic_runs_like_straight():
    m = meshlib.box((4, 4, 3), periodic=(True,) * 3, jitter=0.1, seed=7)
    q = meshlib.quadratic(m)
    u = cases.smooth_ic(meshlib.node_coordinates(m, 3).reshape(-1, 3)).ravel()
    a, b = Lobatto(m, 3, "rusanov"), Lobatto(q, 3, "rusanov")
    for s in (a, b):
        s.SetSolutionColumn(u)
    # the same geometry through a different map: rounding only (parity bar 1e-12)
    assert rel(b.GetResidualColumn(), a.GetResidualColumn()) <= 1e-12
    a.close()
    b.close()


def test_curved_limiter_refused():
    with pytest.raises(capi.McfdError):
        Lobatto(nodal_mesh(False), 2, "roe", limiter="eigen")


@pytest.mark.parametrize("serendipity", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_curved_wedge_pyramid_modal_parity(p, serendipity):
    """Wedge15 / Wedge18 (faces through the cell map) and Pyra13 / Pyra14
    (faces through their own Triangle6 / Quadrangle8 / 9 maps) in one deformed
    mesh with Hex27 / Tet10 blocks: residual, SSP-RK3 step and dt against the
    oracle's nodal (serendipity / Vandermonde) form of the same maps."""
    m = meshlib.deform(meshlib.quadratic(meshlib.concat(
        meshlib.wedge_box((2, 3, 2), periodic=(True,) * 3, jitter=0.05, seed=1),
        meshlib.pyramid_box((2, 2, 2), periodic=(True,) * 3, jitter=0.05, seed=2),
        meshlib.box((2, 2, 2), periodic=(True,) * 3, jitter=0.05, seed=3)), serendipity=serendipity),
        wavy(0.02))
    g = General(m, p, "hllc")
    om = orc.Modal(m, p)
    assert np.allclose(g.points(), om.points()[0], rtol=0, atol=1e-13)
    u = om.project(cases.smooth_ic(om.points()[0]))
    g.SetSolutionColumn(u)
    assert rel(g.GetResidualColumn(), om.residual(orc.HLLC, u)) <= 1e-12
    dt = om.time_step(u, 1.0, 3)
    g.advance(1, dt, 3, 0.0)
    u1 = om.rk_update(orc.HLLC, 3, 0.0, dt, u)
    assert rel(g.GetSolutionColumn(), u1) <= 1e-12
    g.close()


@pytest.mark.parametrize("serendipity", [False, True])
def test_curved_wedge_vtk_sample(serendipity):
    """Quadratic wedges write Wedge15 samples through their own maps."""
    m = meshlib.deform(meshlib.quadratic(meshlib.wedge_box((3, 2, 2), periodic=(True,) * 3, jitter=0.05,
                                                           seed=6), serendipity=serendipity), wavy(0.02))
    g = General(m, 2, "hllc")
    om = orc.Modal(m, 2)
    u = om.project(cases.smooth_ic(om.points()[0]))
    g.SetSolutionColumn(u)
    xyz, values, types = g.vtk_sample()
    oxyz, ovalues, otypes = om.vtk_sample(u)
    assert np.array_equal(types, otypes) and set(types.tolist()) == {26}
    assert rel(xyz, oxyz) <= 1e-14 and rel(values, ovalues) <= 1e-13
    g.close()


def test_undeformed_quadratic_wedge_pyramid_runs_like_straight():
    m = meshlib.concat(meshlib.wedge_box((3, 2, 2), periodic=(True,) * 3, jitter=0.1, seed=7),
                       meshlib.pyramid_box((2, 2, 2), periodic=(True,) * 3, jitter=0.1, seed=8))
    q = meshlib.quadratic(m)
    om = orc.Modal(m, 3)
    u = om.project(cases.smooth_ic(om.points()[0]))
    a, b = General(m, 3, "rusanov"), General(q, 3, "rusanov")
    for s in (a, b):
        s.SetSolutionColumn(u)
    assert rel(b.GetResidualColumn(), a.GetResidualColumn()) <= 1e-12
    a.close()
    b.close()
