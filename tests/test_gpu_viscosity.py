"""GPU energy-based artificial viscosity on fr::Lobatto (through the C ABI)
against the oracle's restatement of EnergyBasedViscosity / WithViscosity.

Bar: cell viscosities, residuals, RK3 steps and time steps within 1e-12
relative (L2 for columns, max-norm for the viscosities, whose zero pattern
must match exactly); 1e-10 for steps with the exact Riemann solver (its
Newton tolerance, see the shock-tube test); initial limiters bit-exact
(majority) or to 1e-14 (average).
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Lobatto, RungeKutta, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RIEMANN = {"exact": orc.EXACT, "hllc": orc.HLLC, "roe": orc.ROE, "rusanov": orc.RUSANOV, "ausm": orc.AUSM}
SOD_BCS = {0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
           2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
           4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def shock_state(x, rng, noise=0.02):
    base = cases.sod_ic(x)
    base = base * (1 + noise * rng.uniform(-1, 1, (x.shape[0], 1)))
    base[:, 1] += 0.05 * rng.uniform(-1, 1, x.shape[0])
    return base.ravel()


def pair(m, p, riemann="exact", beta0=2.0, beta1=1.0 / 12, time_scale=0.05, bcs=None):
    s = Lobatto(m, p, riemann, scheme="fr")
    om = orc.Mesh(m, p, scheme="fr")
    if bcs:
        om.set_bcs(bcs)
        for g, (kind, val) in bcs.items():
            if kind == orc.BC_SMART:
                s.SetSmartBoundary(g, val)
            elif kind == orc.BC_INVISCID_WALL:
                s.SetInviscidWall(g)
            elif kind == orc.BC_NO_SLIP_WALL:
                s.SetNoSlipWall(g)
            elif kind == orc.BC_SUPERSONIC_OUTLET:
                s.SetSupersonicOutlet(g)
    s.SetViscosity(beta0, beta1, time_scale)
    ov = orc.Viscosity(om, beta0, beta1, time_scale)
    return s, om, ov


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("periodic", [False, True])
def test_viscosity_values_parity(gpu, p, periodic):
    m = meshlib.box((8, 3, 3), lengths=(1.0, 0.3, 0.3), periodic=(periodic,) * 3, jitter=0.1, seed=2)
    s, om, ov = pair(m, p)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = shock_state(x, np.random.default_rng(p))
    s.SetSolutionColumn(u)
    got = s.GetViscosity()
    want, _ = ov.properties(u)
    assert np.array_equal(got > 0, want > 0)
    assert want.max() > 0
    assert np.abs(got - want).max() <= RTOL * want.max(), np.abs(got - want).max() / want.max()
    s.close()


def test_viscosity_values_parity_many_listed_cells(gpu):
    """More cells over the jump threshold than the damping-rate kernel's
    persistent grid has warps (152 SMs x a few resident blocks x 4 warps), so
    its warps each take several listed cells; two passes are bitwise equal
    (the list's order does not reach the values)."""
    m = meshlib.box((40, 40, 4), lengths=(1.0, 1.0, 0.1), periodic=(True,) * 3, jitter=0.1, seed=5)
    s, om, ov = pair(m, 2)
    x = meshlib.node_coordinates(m, 2).reshape(-1, 3)
    u = shock_state(x, np.random.default_rng(11))
    s.SetSolutionColumn(u)
    got = s.GetViscosity()
    want, _ = ov.properties(u)
    assert (want.reshape(-1, 5).max(axis=1) > 0).sum() > 4000
    assert np.array_equal(got > 0, want > 0)
    assert np.abs(got - want).max() <= RTOL * want.max(), np.abs(got - want).max() / want.max()
    s.SetSolutionColumn(u)
    assert np.array_equal(s.GetViscosity(), got)
    s.close()


@pytest.mark.parametrize("riemann", ["exact", "hllc", "roe", "rusanov"])
@pytest.mark.parametrize("p", [2, 3])
def test_viscous_residual_parity(gpu, riemann, p):
    m = meshlib.box((8, 3, 2), lengths=(1.0, 0.3, 0.2), jitter=0.1, seed=5)
    s, om, ov = pair(m, p, riemann, bcs=SOD_BCS)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = shock_state(x, np.random.default_rng(7))
    s.SetSolutionColumn(u)
    got = s.GetResidualColumn()
    want = ov.residual(RIEMANN[riemann], u)
    nu, _ = ov.properties(u)
    assert nu.max() > 0
    err = rel_l2(got, want)
    assert err <= RTOL, err
    s.close()


def test_no_slip_wall_parity(gpu):
    p = 2
    m = meshlib.box((6, 3, 3), lengths=(1.0, 0.3, 0.3), jitter=0.1, seed=8)
    bcs = {0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SUPERSONIC_OUTLET, None),
           2: (orc.BC_NO_SLIP_WALL, None), 3: (orc.BC_NO_SLIP_WALL, None),
           4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_NO_SLIP_WALL, None)}
    s, om, ov = pair(m, p, "hllc", bcs=bcs)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = shock_state(x, np.random.default_rng(9))
    s.SetSolutionColumn(u)
    err = rel_l2(s.GetResidualColumn(), ov.residual(orc.HLLC, u))
    assert err <= RTOL, err
    s.close()


def test_no_slip_wall_without_viscosity_parity(gpu):
    """fr::Lobatto without the viscosity: a no-slip wall gets no correction."""
    p = 2
    m = meshlib.box((6, 3, 2), lengths=(1.0, 0.3, 0.2), jitter=0.1, seed=8)
    s = Lobatto(m, p, "roe", scheme="fr")
    om = orc.Mesh(m, p, scheme="fr")
    bcs = {0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
           2: (orc.BC_NO_SLIP_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
           4: (orc.BC_NO_SLIP_WALL, None), 5: (orc.BC_INVISCID_WALL, None)}
    om.set_bcs(bcs)
    s.SetSmartBoundary(0, cases.SOD_LEFT)
    s.SetSmartBoundary(1, cases.SOD_RIGHT)
    for g in (2, 4):
        s.SetNoSlipWall(g)
    for g in (3, 5):
        s.SetInviscidWall(g)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = shock_state(x, np.random.default_rng(3))
    s.SetSolutionColumn(u)
    err = rel_l2(s.GetResidualColumn(), om.residual(orc.ROE, u))
    assert err <= RTOL, err
    s.close()


def test_viscous_time_step_parity(gpu):
    p = 2
    m = cases.sod_mesh(20, 2, 2)
    s, om, ov = pair(m, p, bcs=SOD_BCS)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = shock_state(x, np.random.default_rng(4))
    s.SetSolutionColumn(u)
    for order, guess in ((3, 1.0), (3, 1e-5), (2, 1.0), (1, 1.0)):
        got = s.GetTimeStep(guess, order)
        want = ov.time_step(u, guess, order)
        assert abs(got - want) <= 1e-13 * want, (order, got, want)
    s.close()


@pytest.mark.parametrize("riemann,rtol", [("roe", RTOL), ("exact", 1e-10)])
def test_viscous_shock_tube_rk3_parity(gpu, riemann, rtol):
    """The viscous demos' configuration (fr::Lobatto p = 2 with the energy-
    based viscosity after the majority initial limiter) on a shock tube,
    through RungeKutta::Update (host-driven stages) and through the
    graph-captured mcfd_advance, each against the oracle.

    The tube carries a uniform background velocity so that no conserved
    component is exactly zero anywhere: the reference's viscosity jumps
    between 0 (damping rate -0.0 of an all-zero component) and its cap (the
    smallest positive rate) there (spatial/viscosity.hpp:521-526), so whether
    rounding leaves a zero exact decides the result.  The exact solver's
    Newton loop stops at a 1e-8 tolerance (riemann/euler/exact.hpp:140-152):
    a 1e-15 change of its input moves the oracle itself by ~1e-11 per step on
    this case, hence the looser bar for it."""
    p = 2
    m = meshlib.box((24, 2, 2), lengths=(1.0, 0.04, 0.04), periodic=(False, True, True))
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    left = cases.prim_to_cons(1.0, 0.1, 0.05, -0.07, 1.0)
    right = cases.prim_to_cons(0.125, 0.1, 0.05, -0.07, 0.1)
    u0 = np.where((x[:, 0] < 0.5)[:, None], left[None, :], right[None, :]).ravel()
    bcs = {0: (orc.BC_SMART, left), 1: (orc.BC_SMART, right)}
    s, om, ov = pair(m, p, riemann, bcs=bcs)
    s.SetSolutionColumn(u0)
    s.InitialLimiter("majority")
    u, missing = orc.initial_limiter(om, orc.INIT_MAJORITY, u0)
    assert missing == 0
    assert np.array_equal(s.GetSolutionColumn(), u)
    t = 0.0
    for _ in range(4):
        dt = ov.time_step(u, 1.0, 3)
        RungeKutta(3).Update(s, t, dt)
        u = ov.rk_update(RIEMANN[riemann], 3, t, dt, u)
        t += dt
    err = rel_l2(s.GetSolutionColumn(), u)
    assert err <= rtol, err
    assert ov.properties(u)[0].max() > 0
    # device-side dt and stages (graph)
    s.SetSolutionColumn(u)
    s.SetTime(t)
    t_dev = s.advance(3, 1.0, 3, t)
    for _ in range(3):
        dt = ov.time_step(u, 1.0, 3)
        u = ov.rk_update(RIEMANN[riemann], 3, t, dt, u)
        t += dt
    assert abs(t_dev - t) <= 1e-12 * t
    err = rel_l2(s.GetSolutionColumn(), u)
    assert err <= rtol, err
    s.close()


def test_initial_limiters_parity(gpu):
    p = 2
    m = meshlib.box((6, 3, 2), lengths=(1.0, 0.3, 0.2), jitter=0.1, seed=6)
    s = Lobatto(m, p, "roe", scheme="fr")
    om = orc.Mesh(m, p, scheme="fr")
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    rng = np.random.default_rng(12)
    u = (cases.sod_ic(x) * (1 + 0.1 * rng.uniform(-1, 1, (x.shape[0], 1)))).ravel()
    s.SetSolutionColumn(u)
    s.InitialLimiter("average")
    want, _ = orc.initial_limiter(om, orc.INIT_AVERAGE, u)
    assert np.abs(s.GetSolutionColumn() - want).max() <= 1e-14 * np.abs(want).max()
    st = cases.sod_ic(x).ravel()
    s.SetSolutionColumn(st)
    s.InitialLimiter("majority")
    want, missing = orc.initial_limiter(om, orc.INIT_MAJORITY, st)
    assert missing == 0 and np.array_equal(s.GetSolutionColumn(), want)
    # random states: no majority anywhere -> error, column unchanged
    s.SetSolutionColumn(u)
    with pytest.raises(capi.McfdError):
        s.InitialLimiter("majority")
    assert np.array_equal(s.GetSolutionColumn(), u)
    s.close()


def test_viscosity_rejections(gpu):
    m = meshlib.box((4, 2, 2), lengths=(1.0, 0.5, 0.5))
    s = Lobatto(m, 2, "roe")  # DGSEM
    with pytest.raises(capi.McfdError):
        s.SetViscosity()
    with pytest.raises(capi.McfdError):
        s.SetNoSlipWall(2)
    s.close()
    s = Lobatto(m, 2, "roe", scheme="fr", precision="mixed")
    with pytest.raises(capi.McfdError):
        s.SetViscosity()
    s.close()
    s = Lobatto(m, 2, "roe", scheme="fr", limiter="lazy")
    with pytest.raises(capi.McfdError):
        s.SetViscosity()
    s.close()


def _background_tube(p, nx=16, periodic=(False, True, True)):
    m = meshlib.box((nx, 2, 2), lengths=(1.0, 0.1, 0.1), periodic=periodic, jitter=0.05, seed=9)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    left = cases.prim_to_cons(1.0, 0.1, 0.05, -0.07, 1.0)
    right = cases.prim_to_cons(0.125, 0.1, 0.05, -0.07, 0.1)
    u0 = np.where((x[:, 0] < 0.5)[:, None], left[None, :], right[None, :]).ravel()
    return m, u0, left, right


@pytest.mark.parametrize("p", [1, 3])
def test_viscous_rk3_parity_other_degrees(gpu, p):
    """p = 1 and p = 3 (spatial factors 4 and 40, viscosity.hpp:581-601),
    HLLC, on a jittered tube with a background flow."""
    m, u0, left, right = _background_tube(p)
    s, om, ov = pair(m, p, "hllc", bcs={0: (orc.BC_SMART, left), 1: (orc.BC_SMART, right)})
    # the demos' initial limiter puts the jump on cell faces (majority is a
    # no-op below p = 2, limiter/majority.hpp:17-19)
    kind = "majority" if p >= 2 else "average"
    s.SetSolutionColumn(u0)
    s.InitialLimiter(kind)
    u, _ = orc.initial_limiter(om, orc.INIT_MAJORITY if p >= 2 else orc.INIT_AVERAGE, u0)
    assert np.abs(s.GetSolutionColumn() - u).max() <= 1e-14 * np.abs(u).max()
    s.SetSolutionColumn(u)
    t = 0.0
    for _ in range(3):
        dt = ov.time_step(u, 1.0, 3)
        assert abs(s.GetTimeStep(1.0, 3) - dt) <= 1e-13 * dt
        RungeKutta(3).Update(s, t, dt)
        u = ov.rk_update(orc.HLLC, 3, t, dt, u)
        t += dt
    assert ov.properties(u)[0].max() > 0
    err = rel_l2(s.GetSolutionColumn(), u)
    assert err <= RTOL, err
    s.close()


def test_viscous_stream_matches_advance(gpu):
    """mcfd_stream_step (per-slot job graphs: dt pass, then the stages reusing
    its viscosity properties) gives the columns of mcfd_advance."""
    p = 2
    m, u0, left, right = _background_tube(p)
    s, _, _ = pair(m, p, "roe", bcs={0: (orc.BC_SMART, left), 1: (orc.BC_SMART, right)})
    s.SetSolutionColumn(u0)
    s.InitialLimiter("majority")
    u0 = s.GetSolutionColumn()
    want = []
    t = 0.0
    for _ in range(3):
        t = s.advance(1, 1.0, 3, t)
        want.append(s.GetSolutionColumn())
    host_in = [u0.copy(), want[0].copy(), want[1].copy()]
    host_out = [np.empty_like(u0) for _ in range(3)]
    s.stream_begin()
    for k in range(3):
        s.stream_step(host_in[k], host_out[k], 0.0, 1, 1.0, 3)
    s.stream_end()
    for k in range(3):
        assert rel_l2(host_out[k], want[k]) <= 1e-15, k
    s.close()


def test_fr_degenerate_state_is_reported(gpu):
    """A state with negative pressure at a face point (clamped to zero
    primitives, riemann/euler/types.hpp:194-202) makes the HLLC flux NaN in the
    oracle; the GPU residual reports the non-finite value instead of treating
    that face as one without a boundary condition."""
    p = 2
    m = meshlib.box((4, 2, 2), lengths=(1.0, 0.5, 0.5), periodic=(True,) * 3)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = np.tile(cases.prim_to_cons(1.0, 0.1, 0.0, 0.0, 1.0), (x.shape[0], 1))
    u[0] = [0.16, 0.38, 0.008, -0.011, 0.379]   # kinetic energy above the total
    u = u.ravel()
    om = orc.Mesh(m, p, scheme="fr")
    assert not np.isfinite(om.residual(orc.HLLC, u)).all()
    s = Lobatto(m, p, "hllc", scheme="fr")
    s.SetSolutionColumn(u)
    with pytest.raises(capi.McfdError):
        s.GetResidualColumn()
    s.close()
