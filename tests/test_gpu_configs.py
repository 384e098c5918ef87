"""Parity on the benchmark configurations themselves: each case built with
its own mesh generator, boundary conditions, flux and limiter (at full size
where the oracle finishes in seconds, else scaled down with the same cell
size and data), stepped on the GPU and by the oracle with each side's own
time step.

* Sod shock tube at its full 100 x 4 x 4 size: DGSEM p = 2, Roe, weno::Lazy
  on every cell, smart ends and walls (demo/euler/shock_tube.cpp), CFL 0.1.
* Isentropic vortex on its 16^3 mesh: DGSEM p = 3, Rusanov, no limiter.
* Four-quadrant Riemann problem at 32 x 32 x 2 (the full case's cell size
  h = 1/256 scaled to 1/32): DGSEM p = 2, Roe, the moving-shock smart
  boundaries and walls of demo/euler/riemann2d.cpp:28-53, weno::Eigen.
* Mixed-element box at 6^3 Hex8 + 4^3 x 6 Tet4 (jittered, seed 0): modal
  DG p = 2, HLLC.
* Three members of the batched ensemble's seed-1 draw (its three smallest
  cases of different schemes), stepped together as an mcfd_ensemble.

FP64 bar: relative L2 <= 1e-12 after every step, identical troubled-cell
counts; time steps equal to 1e-12 relative.  Mixed form: density within
1e-6 relative L2 of the FP64 oracle.
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Ensemble, General, Lobatto, MovingSplit, RungeKutta, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MIXED_RHO_RTOL = 1e-6


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def density_rel_l2(a, b):
    a, b = a.reshape(-1, 5)[:, 0], b.reshape(-1, 5)[:, 0]
    return rel_l2(a, b)


SOD_ORC_BCS = {0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
               2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
               4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)}


def quadrant_orc_bcs():
    return {0: (orc.BC_SMART, MovingSplit(axis=1, position=0.8, speed=cases.SPEED_BC, a=cases.Q_C, b=cases.Q_B)),
            1: (orc.BC_INVISCID_WALL, None),
            2: (orc.BC_SMART, MovingSplit(axis=0, position=0.8, speed=cases.SPEED_CD, a=cases.Q_C, b=cases.Q_D)),
            3: (orc.BC_INVISCID_WALL, None), 4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)}


def step_limited_pair(s, om, lim, riemann, u, steps, cfl):
    """`steps` SSP-RK3 steps on both sides, each with its own time step."""
    t = 0.0
    troubled = []
    for k in range(steps):
        dt_orc = om.time_step(u, 1.0, 3, cfl)
        dt_gpu = s.GetTimeStep(1.0, 3)
        assert abs(dt_gpu - dt_orc) <= RTOL * dt_orc, (k, dt_gpu, dt_orc)
        s.troubled_cells()  # reset the count
        RungeKutta(3).Update(s, t, dt_orc)
        u = lim.rk_update(riemann, 3, t, dt_orc, u)
        t += dt_orc
        err = rel_l2(s.GetSolutionColumn(), u)
        assert err <= RTOL, (k, err)
        troubled.append(s.troubled_cells())
    return u, troubled


def test_sod_full_size_roe_weno_lazy(gpu):
    p, cfl = 2, 0.1
    m = cases.sod_mesh()  # 100 x 4 x 4
    assert m.n_cells == 1600
    u0 = cases.sod_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s = Lobatto(m, p, "roe", cfl=cfl, limiter="lazy")
    cases.sod_bc(s)
    s.SetSolutionColumn(u0)
    om = orc.Mesh(m, p)
    om.set_bcs(SOD_ORC_BCS)
    lim = orc.Limiter(om, orc.LIMITER_LAZY)
    u, n = lim.limit(u0)
    assert rel_l2(s.GetSolutionColumn(), u) <= RTOL
    assert n == m.n_cells  # weno::Lazy reconstructs every cell
    step_limited_pair(s, om, lim, orc.ROE, u, 8, cfl)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vortex_16_dgsem_p3_rusanov(gpu, precision):
    p = 3
    m = cases.vortex_mesh(16)
    u = cases.vortex_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s = Lobatto(m, p, "rusanov", cfl=0.1, precision=precision)
    s.SetSolutionColumn(u)
    om = orc.Mesh(m, p)
    t = 0.0
    for k in range(3):
        dt = om.time_step(u, 1.0, 3, 0.1)
        assert abs(s.GetTimeStep(1.0, 3) - dt) <= (RTOL if precision == "fp64" else 1e-6) * dt
        RungeKutta(3).Update(s, t, dt)
        u = om.rk_update(orc.RUSANOV, 3, t, dt, u)
        t += dt
        g = s.GetSolutionColumn()
        if precision == "fp64":
            assert rel_l2(g, u) <= RTOL, (k, rel_l2(g, u))
        else:
            assert density_rel_l2(g, u) <= MIXED_RHO_RTOL, (k, density_rel_l2(g, u))
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_four_quadrant_scaled_roe_weno_eigen(gpu, precision):
    p = 2
    m = cases.quadrant_mesh(32, 32, 2)
    u0 = cases.quadrant_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s = Lobatto(m, p, "roe", precision=precision, limiter="eigen")
    cases.quadrant_bc(s)
    s.SetSolutionColumn(u0)
    om = orc.Mesh(m, p)
    om.set_bcs(quadrant_orc_bcs())
    lim = orc.Limiter(om, orc.LIMITER_EIGEN)
    u, n0 = lim.limit(u0)
    assert s.troubled_cells() == n0 and 0 < n0 < m.n_cells
    if precision == "fp64":
        assert rel_l2(s.GetSolutionColumn(), u) <= RTOL
        _, troubled = step_limited_pair(s, om, lim, orc.ROE, u, 5, 0.0)
        assert all(0 < k < 3 * m.n_cells for k in troubled)
    else:
        t = 0.0
        for k in range(5):
            dt = om.time_step(u, 1.0, 3, 0.0)
            RungeKutta(3).Update(s, t, dt)
            u = lim.rk_update(orc.ROE, 3, t, dt, u)
            t += dt
        err = density_rel_l2(s.GetSolutionColumn(), u)
        assert err <= MIXED_RHO_RTOL, err
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mixed_box_scaled_modal_p2_hllc(gpu, precision):
    p = 2
    m = cases.mixed_box_mesh(6, 4)
    assert m.n_cells == 6 ** 3 + 6 * 4 ** 3
    s = General(m, p, "hllc", precision=precision)
    om = orc.Modal(m, p)
    u = om.project(cases.mixed_box_ic(om.points()[0]))
    s.SetSolutionColumn(u)
    t = 0.0
    for k in range(3):
        dt = om.time_step(u, 1.0, 3, 0.0)
        if precision == "fp64":
            assert abs(s.GetTimeStep(1.0, 3) - dt) <= RTOL * dt
        RungeKutta(3).Update(s, t, dt)
        u = om.rk_update(orc.HLLC, 3, t, dt, u)
        t += dt
    g = s.GetSolutionColumn()
    if precision == "fp64":
        assert rel_l2(g, u) <= RTOL, rel_l2(g, u)
    else:
        # modal coefficients: the density is the first component of every mode
        assert density_rel_l2(g, u) <= MIXED_RHO_RTOL, density_rel_l2(g, u)
    s.close()


def three_ensemble_members():
    """The ensemble's seed-1 draw; its smallest DGSEM hex case, smallest
    modal tet case and smallest modal hex case."""
    specs = cases.ensemble_spec()
    size = lambda sp: sp["n"] ** 3 * (6 if sp["tet"] else 1)
    picks = []
    for want in (("dgsem", False), ("modal", True), ("modal", False)):
        cand = [sp for sp in specs if (sp["scheme"], sp["tet"]) == want]
        picks.append(min(cand, key=size))
    return picks


def test_ensemble_members_seed1_through_one_graph(gpu):
    members = three_ensemble_members()
    systems, oracles, us = [], [], []
    for sp in members:
        q = cases.ensemble_mesh(sp)
        if sp["scheme"] == "modal":
            g = General(q, sp["p"], "rusanov")
            o = orc.Modal(q, sp["p"])
            u = o.project(cases.ensemble_state(o.points()[0], sp))
            g.SetSolutionColumn(u)
        else:
            g = Lobatto(q, sp["p"], "rusanov")
            o = orc.Mesh(q, sp["p"])
            u = cases.ensemble_state(meshlib.node_coordinates(q, sp["p"]).reshape(-1, 3), sp).ravel()
            g.SetSolutionColumn(u)
        systems.append(g)
        oracles.append(o)
        us.append(u)
    ens = Ensemble(systems)
    steps = 3
    ens.advance(steps, 1e9, 3)
    for g, o, u, sp in zip(systems, oracles, us, members):
        t = 0.0
        for _ in range(steps):
            dt = o.time_step(u, 1e9, 3, 0.0)
            u = o.rk_update(orc.RUSANOV, 3, t, dt, u)
            t += dt
        err = rel_l2(g.GetSolutionColumn(), u)
        assert err <= RTOL, (sp["case"], sp["scheme"], sp["p"], err)
    ens.close()
    for g in systems:
        g.close()
