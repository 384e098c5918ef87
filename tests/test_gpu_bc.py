"""Boundary values that depend on position and time (the reference's
std::function<Value(Global, double)> per boundary, spatial/fem.hpp:196-222)
on the GPU against the oracle:

* the oblique moving shock of demo/euler/double_mach.cpp:28-31 (a state
  program evaluated on the device at every face point and stage time) on
  the supersonic inlets of the double-Mach reflection, DGSEM and modal DG;
* a function of the position alone, sampled once at the group's face points
  into a table (as the right boundary of demo/euler/shu_osher.cpp:22-23,
  whose state is the initial sine profile), on smart boundaries, DGSEM, FR
  and modal DG.

Bar: relative L2 <= 1e-12 after three SSP-RK3 steps with each side's own
time step.
"""
import math

import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import General, Lobatto, ObliqueSplit, RungeKutta, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RIEMANN = {"roe": orc.ROE, "hllc": orc.HLLC, "exact": orc.EXACT, "rusanov": orc.RUSANOV}

# demo/euler/double_mach.cpp:5-31, at shock Mach 1.5 instead of 10: the
# boundary program is the same, and without the demo's limiter an
# unlimited p = 2 start from the Mach-10 discontinuity loses positivity in the
# reference algorithm (the oracle's own run turns non-finite within three
# steps), so the parity check takes a shock the scheme carries unlimited.
TAN60 = math.sqrt(3.0)
MACH = 1.5
RHO_AFTER = 1.4 * (MACH ** 2 * 2.4 / 2) / (1 + MACH ** 2 * 0.4 / 2)
P_AFTER = (MACH ** 2 * 1.4 - 0.4 / 2) / (2.4 / 2)
UN_AFTER = MACH * (RHO_AFTER - 1.4) / RHO_AFTER
AFTER = cases.prim_to_cons(RHO_AFTER, UN_AFTER * TAN60 * 0.5, -UN_AFTER * 0.5, 0.0, P_AFTER)
BEFORE = cases.prim_to_cons(1.4, 0.0, 0.0, 0.0, 1.0)
X_GAP = 1.0 / 6.0
U_X = MACH / (TAN60 * 0.5)
MOVING_SHOCK = ObliqueSplit(normal=np.array([TAN60, -1.0, 0.0]), position=TAN60 * X_GAP, speed=TAN60 * U_X,
                            a=AFTER, b=BEFORE)


def double_mach_ic(x):
    after = ((x[:, 0] - X_GAP) * TAN60 < x[:, 1])[:, None]
    return np.where(after, AFTER[None, :], BEFORE[None, :])


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def double_mach_bcs(s, om):
    """double_mach.cpp:33-51 on a box: left and top inlets with the moving
    shock, right outlet, walls at the bottom, front and back."""
    s.SetSupersonicInlet(0, MOVING_SHOCK)
    s.SetSupersonicInlet(3, MOVING_SHOCK)
    s.SetSupersonicOutlet(1)
    for g in (2, 4, 5):
        s.SetInviscidWall(g)
    om.set_bcs({0: (orc.BC_SUPERSONIC_INLET, MOVING_SHOCK), 3: (orc.BC_SUPERSONIC_INLET, MOVING_SHOCK),
                1: (orc.BC_SUPERSONIC_OUTLET, None), 2: (orc.BC_INVISCID_WALL, None),
                4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)})


def step_pair(s, om, u, riemann, steps=3, lim=None):
    t = 0.0
    for k in range(steps):
        dt = om.time_step(u, 1.0, 3, 0.0)
        assert abs(s.GetTimeStep(1.0, 3) - dt) <= RTOL * dt
        RungeKutta(3).Update(s, t, dt)
        u = (lim or om).rk_update(riemann, 3, t, dt, u)
        t += dt
        err = rel_l2(s.GetSolutionColumn(), u)
        assert err <= RTOL, (k, err)
    return u


@pytest.mark.parametrize("riemann", ["roe", "hllc"])
def test_double_mach_moving_shock_dgsem(gpu, riemann):
    p = 2
    m = meshlib.box((12, 4, 1), lengths=(4.0, 1.0, 0.25), jitter=0.05, seed=2)
    s = Lobatto(m, p, riemann)
    om = orc.Mesh(m, p)
    double_mach_bcs(s, om)
    u = double_mach_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s.SetSolutionColumn(u)
    step_pair(s, om, u, RIEMANN[riemann])
    s.close()


def test_double_mach_moving_shock_modal_tets(gpu):
    """Modal DG on tetrahedra with the weno::Eigen limiter (the projected
    discontinuity needs it on the modal scheme)."""
    p = 2
    m = meshlib.tet_box((8, 3, 1), lengths=(4.0, 1.0, 0.25), jitter=0.05, seed=3)
    s = General(m, p, "hllc", limiter="eigen")
    om = orc.Modal(m, p)
    lim = orc.ModalLimiter(om, orc.LIMITER_EIGEN)
    double_mach_bcs(s, om)
    u = om.project(double_mach_ic(om.points()[0]))
    s.SetSolutionColumn(u)
    u, n = lim.limit(u)
    assert s.troubled_cells() == n > 0
    step_pair(s, om, u, orc.HLLC, lim=lim)
    s.close()


# demo/euler/shu_osher.cpp:5-23: the right boundary's state is the initial
# profile at the boundary point, rho = 1 + 0.2 sin(5 x), a function of the
# position alone.  Here both ends take such a profile (with a uniform flow,
# so that the solution stays smooth for an unlimited scheme).
def shu_osher_profile(x):
    rho = 1.0 + 0.2 * np.sin(5.0 * x[:, 0]) * (1 + 0.1 * np.cos(3.0 * x[:, 1]))
    return cases.prim_to_cons(rho, 0.3, 0.0, 0.0, 1.0)


def shu_osher_bcs(s, om):
    s.SetSmartBoundary(0, shu_osher_profile)
    s.SetSmartBoundary(1, shu_osher_profile)
    for g in (2, 3, 4, 5):
        s.SetInviscidWall(g)
    om.set_bcs({0: (orc.BC_SMART, shu_osher_profile), 1: (orc.BC_SMART, shu_osher_profile),
                2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
                4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)})


@pytest.mark.parametrize("scheme", ["dgsem", "fr"])
def test_shu_osher_table_boundary_nodal(gpu, scheme):
    """Boundary points at x = 0 and x = 5 with y-dependent values."""
    p = 2
    m = meshlib.box((10, 2, 2), lengths=(5.0, 0.5, 0.5), origin=(0.0, 0.0, 0.0), jitter=0.1, seed=4)
    s = Lobatto(m, p, "roe", scheme=scheme)
    om = orc.Mesh(m, p, scheme)
    shu_osher_bcs(s, om)
    pts = s.bc_points(1)
    assert np.allclose(pts[:, 0], 5.0) and pts.shape[0] == 2 * 2 * (p + 1) ** 2
    u = shu_osher_profile(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s.SetSolutionColumn(u)
    step_pair(s, om, u, orc.ROE)
    s.close()


def test_shu_osher_table_boundary_modal(gpu):
    p = 2
    m = meshlib.concat(meshlib.box((6, 2, 2), lengths=(5.0, 0.5, 0.5), jitter=0.1, seed=5))
    s = General(m, p, "hllc")
    om = orc.Modal(m, p)
    shu_osher_bcs(s, om)
    u = om.project(shu_osher_profile(om.points()[0]))
    s.SetSolutionColumn(u)
    step_pair(s, om, u, orc.HLLC)
    s.close()


def test_table_boundary_replaced_and_recaptured(gpu):
    """A table set after a captured step graph takes effect at the next
    advance (the graph is captured again)."""
    p = 2
    m = meshlib.box((10, 2, 2), lengths=(5.0, 0.5, 0.5), jitter=0.1, seed=4)
    u = shu_osher_profile(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    const = cases.prim_to_cons(1.0, 0.3, 0.0, 0.0, 1.0)
    outs = []
    for late in (False, True):
        s = Lobatto(m, p, "roe")
        s.SetSmartBoundary(0, shu_osher_profile)
        s.SetSmartBoundary(1, const if late else shu_osher_profile)
        for g in (2, 3, 4, 5):
            s.SetInviscidWall(g)
        s.SetSolutionColumn(u)
        if late:
            s.advance(1, 1.0, 3, 0.0)  # captures the step graph with the constant state
            s.SetSmartBoundary(1, shu_osher_profile)
            s.SetSolutionColumn(u)
        s.advance(2, 1.0, 3, 0.0)
        outs.append(s.GetSolutionColumn())
        s.close()
    assert rel_l2(outs[1], outs[0]) <= 1e-14
