"""Parity of the GPU DGSEM path (through the C ABI) with the CPU oracle.

Bar: face/neighbour indexing bit-exact; FP64 residual, time step and RK
updates within 1e-12 relative L2 of the oracle (the tolerance the plain form
is specified against).
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Lobatto, MovingSplit, RungeKutta, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
KINDS = {"exact": orc.EXACT, "hllc": orc.HLLC, "ausm": orc.AUSM, "roe": orc.ROE, "rusanov": orc.RUSANOV}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def random_state(n_nodes, seed, amp=0.2):
    rng = np.random.default_rng(seed)
    rho = 1 + amp * rng.uniform(-1, 1, n_nodes)
    vel = 0.5 * rng.uniform(-1, 1, (3, n_nodes))
    p = 1 + amp * rng.uniform(-1, 1, n_nodes)
    return cases.prim_to_cons(rho, vel[0], vel[1], vel[2], p).ravel()


# Boundary set used on open boxes: groups 0..5 = x-, x+, y-, y+, z-, z+.
FREE = cases.prim_to_cons(1.0, 0.2, 0.1, -0.1, 1.0)
LOW = cases.prim_to_cons(0.8, -0.1, 0.0, 0.2, 0.7)


def bc_specs():
    return {
        0: ("smart", FREE),
        1: ("supersonic_outlet", None),
        2: ("smart", MovingSplit(axis=0, position=0.5, speed=0.3, a=FREE, b=LOW)),
        3: ("wall", None),
        4: ("subsonic_inlet", np.array([1.3, 0.0, 0.0, 1.0, 2.0 / 287.05])),
        5: ("subsonic_outlet", np.array([0, 0, 0, 0, 0.9])),
    }


ORC_KIND = {"smart": orc.BC_SMART, "supersonic_outlet": orc.BC_SUPERSONIC_OUTLET,
            "supersonic_inlet": orc.BC_SUPERSONIC_INLET, "wall": orc.BC_INVISCID_WALL,
            "subsonic_inlet": orc.BC_SUBSONIC_INLET, "subsonic_outlet": orc.BC_SUBSONIC_OUTLET}


def apply_bcs(system, om, specs, groups):
    used = {g: specs[g] for g in groups}
    om.set_bcs({g: (ORC_KIND[k], v) for g, (k, v) in used.items()})
    for g, (k, v) in used.items():
        if k == "smart":
            system.SetSmartBoundary(g, v)
        elif k == "supersonic_outlet":
            system.SetSupersonicOutlet(g)
        elif k == "supersonic_inlet":
            system.SetSupersonicInlet(g, v)
        elif k == "wall":
            system.SetInviscidWall(g)
        elif k == "subsonic_inlet":
            system.SetSubsonicInlet(g, v)
        elif k == "subsonic_outlet":
            system.SetSubsonicOutlet(g, v)


def make_case(p, periodic, jitter, riemann, shape=(4, 3, 3), seed=0):
    m = meshlib.box(shape, lengths=(1.0, 0.8, 0.6), periodic=periodic, jitter=jitter, seed=seed)
    sys_ = Lobatto(m, p, riemann)
    om = orc.Mesh(m, p)
    groups = sorted(set(int(g) for g in m.face_group if g >= 0))
    apply_bcs(sys_, om, bc_specs(), groups)
    return m, sys_, om


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("periodic,jitter", [((True, True, True), 0.0), ((True, False, True), 0.1),
                                             ((False, False, False), 0.1)])
def test_face_node_maps_bit_exact(gpu, p, periodic, jitter):
    m, s, om = make_case(p, periodic, jitter, "rusanov")
    gh, gs = s.face_node_maps()
    oh, os_ = om.face_node_maps()
    assert np.array_equal(gh, oh)
    assert np.array_equal(gs, os_)
    s.close()


@pytest.mark.parametrize("riemann", list(KINDS))
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("periodic,jitter", [((True, True, True), 0.1), ((False, False, False), 0.1)])
def test_residual_parity(gpu, riemann, p, periodic, jitter):
    m, s, om = make_case(p, periodic, jitter, riemann)
    u = random_state(m.n_cells * (p + 1) ** 3, seed=p)
    t = 0.37
    s.SetSolutionColumn(u)
    s.SetTime(t)
    r_gpu = s.GetResidualColumn()
    r_orc = om.residual(KINDS[riemann], u, t)
    assert np.all(np.isfinite(r_orc))
    err = rel_l2(r_gpu, r_orc)
    assert err <= RTOL, err
    # SetSolutionColumn / GetSolutionColumn round trip is exact
    assert np.array_equal(s.GetSolutionColumn(), u)
    s.close()


@pytest.mark.parametrize("riemann", ["rusanov", "roe", "hllc"])
def test_residual_deterministic(gpu, riemann):
    m, s, om = make_case(3, (True, False, False), 0.1, riemann)
    u = random_state(m.n_cells * 64, seed=11)
    s.SetSolutionColumn(u)
    a = s.GetResidualColumn()
    b = s.GetResidualColumn()
    assert a.tobytes() == b.tobytes()
    s.close()


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("p", [2, 3])
def test_time_step_and_rk_parity(gpu, order, p):
    m, s, om = make_case(p, (True, False, True), 0.1, "roe")
    u = random_state(m.n_cells * (p + 1) ** 3, seed=5)
    s.SetSolutionColumn(u)
    s.SetTime(0.1)
    dt_gpu = s.GetTimeStep(1.0, order)
    dt_orc = om.time_step(u, 1.0, order)
    assert abs(dt_gpu - dt_orc) <= 1e-14 * dt_orc
    RungeKutta(order).Update(s, 0.1, dt_orc)
    u_orc = om.rk_update(orc.ROE, order, 0.1, dt_orc, u)
    err = rel_l2(s.GetSolutionColumn(), u_orc)
    assert err <= RTOL, err
    s.close()


def test_advance_matches_oracle_loop(gpu):
    """mcfd_advance (device dt + graph-captured SSP-RK3) against the oracle
    driving GetTimeStep + RungeKutta<3>::Update step by step."""
    p, cfl, steps = 3, 0.1, 4
    m = meshlib.box((4, 4, 4), lengths=(10.0,) * 3, periodic=(True,) * 3, jitter=0.05, seed=0)
    s = Lobatto(m, p, "rusanov", cfl=cfl)
    om = orc.Mesh(m, p)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    s.SetSolutionColumn(u)
    t_end = s.advance(steps, 1e9, 3, 0.0)
    t = 0.0
    for _ in range(steps):
        dt = om.time_step(u, 1e9, 3, cfl)
        u = om.rk_update(orc.RUSANOV, 3, t, dt, u)
        t += dt
    assert abs(t_end - t) <= 1e-13 * t
    err = rel_l2(s.GetSolutionColumn(), u)
    assert err <= RTOL, err
    s.close()


def test_bad_inputs_fail_loudly(gpu):
    from pvcriemannsolvers_gb300 import capi
    m = meshlib.box((2, 2, 2), periodic=(True,) * 3)
    s = Lobatto(m, 2, "rusanov")
    with pytest.raises(capi.McfdError):
        s.SetSolutionColumn(np.zeros(7))
    bad = meshlib.box((2, 2, 2), periodic=(True,) * 3)
    bad.face_sides = bad.face_sides.copy()
    bad.face_sides[0, 1] = (bad.face_sides[0, 1] + 1) % 6  # wrong sharer side
    with pytest.raises(capi.McfdError):
        Lobatto(bad, 2, "rusanov")
    s.close()


@pytest.mark.parametrize("riemann", ["rusanov", "roe", "hllc", "exact"])
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("periodic,jitter", [((True, True, True), 0.1), ((False, False, False), 0.1)])
def test_fr_residual_parity(gpu, riemann, p, periodic, jitter):
    """fr::Lobatto (Huynh g2) residual against the oracle's FR restatement."""
    m = meshlib.box((4, 3, 3), lengths=(1.0, 0.8, 0.6), periodic=periodic, jitter=jitter, seed=0)
    s = Lobatto(m, p, riemann, scheme="fr")
    om = orc.Mesh(m, p, "fr")
    groups = sorted(set(int(g) for g in m.face_group if g >= 0))
    apply_bcs(s, om, bc_specs(), groups)
    u = random_state(m.n_cells * (p + 1) ** 3, seed=p + 10)
    s.SetSolutionColumn(u)
    s.SetTime(0.2)
    err = rel_l2(s.GetResidualColumn(), om.residual(KINDS[riemann], u, 0.2))
    assert err <= RTOL, err
    s.close()


def test_fr_rk_and_time_step_parity(gpu):
    m = meshlib.box((4, 4, 3), lengths=(10.0,) * 3, periodic=(True,) * 3, jitter=0.05, seed=2)
    p = 3
    s = Lobatto(m, p, "rusanov", cfl=0.1, scheme="fr")
    om = orc.Mesh(m, p, "fr")
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    s.SetSolutionColumn(u)
    t_end = s.advance(3, 1e9, 3, 0.0)
    t = 0.0
    for _ in range(3):
        dt = om.time_step(u, 1e9, 3, 0.1)
        u = om.rk_update(orc.RUSANOV, 3, t, dt, u)
        t += dt
    assert abs(t_end - t) <= 1e-13 * t
    assert rel_l2(s.GetSolutionColumn(), u) <= RTOL
    s.close()
