"""GPU WENO limiter (through the C ABI) against the oracle's restatement of
limiter::Reconstruct with weno::Lazy / the weno::Eigen jump detector.

Bar: 1e-12 relative L2 on the limited column and on limited SSP-RK3 steps;
identical troubled-cell counts.
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Lobatto, RungeKutta, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MODES = {"lazy": orc.LIMITER_LAZY, "detect_lazy": orc.LIMITER_DETECT_LAZY, "eigen": orc.LIMITER_EIGEN}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def sod_like(x, rng):
    base = cases.sod_ic(x)
    noise = 1 + 0.02 * rng.uniform(-1, 1, (x.shape[0], 1))
    return (base * noise).ravel()


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("periodic", [False, True])
def test_limiter_parity(gpu, mode, p, periodic):
    m = meshlib.box((8, 3, 2), lengths=(1.0, 0.3, 0.2), periodic=(periodic,) * 3, jitter=0.1, seed=4)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u = sod_like(x, np.random.default_rng(p))
    s = Lobatto(m, p, "roe", limiter=mode)
    om = orc.Mesh(m, p)
    lim = orc.Limiter(om, MODES[mode])
    s.SetSolutionColumn(u)            # WithLimiter::SetSolutionColumn limits
    got = s.GetSolutionColumn()
    want, n_orc = lim.limit(u)
    assert s.troubled_cells() == n_orc
    if mode != "lazy":
        assert 0 < n_orc < m.n_cells
    assert rel_l2(got, want) <= RTOL, rel_l2(got, want)
    s.close()


@pytest.mark.parametrize("mode", list(MODES))
def test_limited_rk3_parity(gpu, mode):
    """SSP-RK3 on WithLimiter<dg::Lobatto> (Sod tube, Roe, p = 2): the limiter
    runs after every stage."""
    p = 2
    m = cases.sod_mesh(20, 2, 2)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u0 = cases.sod_ic(x).ravel()
    s = Lobatto(m, p, "roe", limiter=mode)
    cases.sod_bc(s)
    om = orc.Mesh(m, p)
    om.set_bcs({0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
                2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
                4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)})
    lim = orc.Limiter(om, MODES[mode])
    s.SetSolutionColumn(u0)
    u, _ = lim.limit(u0)
    t = 0.0
    for _ in range(3):
        dt = om.time_step(u, 1.0, 3, 0.1)
        RungeKutta(3).Update(s, t, dt)
        u = lim.rk_update(orc.ROE, 3, t, dt, u)
        t += dt
    err = rel_l2(s.GetSolutionColumn(), u)
    assert err <= RTOL, err
    s.close()


def test_limiter_keeps_advance_graph_consistent(gpu):
    """mcfd_advance (graph-captured step incl. limiter passes) equals the
    step-by-step fused update."""
    p = 2
    m = cases.sod_mesh(16, 2, 2)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u0 = cases.sod_ic(x).ravel()
    out = []
    for fused in (True, False):
        s = Lobatto(m, p, "roe", cfl=0.1, limiter="lazy")
        cases.sod_bc(s)
        s.SetSolutionColumn(u0)
        if fused:
            s.advance(3, 1e9, 3, 0.0)
        else:
            t = 0.0
            for _ in range(3):
                dt = s.GetTimeStep(1e9, 3)
                RungeKutta(3).Update(s, t, dt)
                t += dt
        out.append(s.GetSolutionColumn())
        s.close()
    assert rel_l2(out[0], out[1]) <= 1e-14


def test_limited_fr_rk3_parity(gpu):
    """WithLimiter<fr::Lobatto>: the same Sod tube with the FR scheme."""
    p = 2
    m = cases.sod_mesh(20, 2, 2)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u0 = cases.sod_ic(x).ravel()
    s = Lobatto(m, p, "roe", limiter="detect_lazy", scheme="fr")
    cases.sod_bc(s)
    om = orc.Mesh(m, p, "fr")
    om.set_bcs({0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
                2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
                4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)})
    lim = orc.Limiter(om, MODES["detect_lazy"])
    s.SetSolutionColumn(u0)
    u, _ = lim.limit(u0)
    t = 0.0
    for _ in range(3):
        dt = om.time_step(u, 1.0, 3, 0.1)
        RungeKutta(3).Update(s, t, dt)
        u = lim.rk_update(orc.ROE, 3, t, dt, u)
        t += dt
    err = rel_l2(s.GetSolutionColumn(), u)
    assert err <= RTOL, err
    s.close()


@pytest.mark.parametrize("mode", ["eigen", "detect_lazy"])
def test_mixed_form_limiter_close_to_fp64(gpu, mode):
    """The mixed form's limiter (FP32 nodal-to-modal products of the momenta;
    density, energy, smoothness and reconstruction in FP64) tracks the FP64
    form on the Sod tube: about the same troubled cells, density within 1e-6
    after 10 steps."""
    p = 2
    m = cases.sod_mesh(40, 2, 2)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    u0 = cases.sod_ic(x).ravel()
    out = {}
    for precision in ("fp64", "mixed"):
        s = Lobatto(m, p, "roe", cfl=0.1, limiter=mode, precision=precision)
        cases.sod_bc(s)
        s.SetSolutionColumn(u0)
        s.troubled_cells()
        s.advance(10, 1.0, 3, 0.0)
        out[precision] = (s.GetSolutionColumn(), s.troubled_cells())
        s.close()
    a, b = out["mixed"][0].reshape(-1, 5)[:, 0], out["fp64"][0].reshape(-1, 5)[:, 0]
    assert rel_l2(a, b) <= 1e-6
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 0.02 * out["fp64"][1] + 2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_limited_steps_bitwise_reproducible(gpu, precision):
    """The troubled-cell list is appended in atomic order, so its order
    changes from run to run; every reconstruction reads only the modal
    buffer and writes only its own cell, so two runs of the same limited
    steps (captured graph: dt, stages, limiter passes) are bitwise equal.
    The four-quadrant problem with weno::Eigen, as in its workload."""
    p = 2
    m = cases.quadrant_mesh(16, 16, 2)
    u0 = cases.quadrant_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    outs = []
    for run in range(2):
        s = Lobatto(m, p, "roe", limiter="eigen", precision=precision)
        cases.quadrant_bc(s)
        s.SetSolutionColumn(u0)
        t = s.advance(6, 1.0, 3, 0.0)
        outs.append((s.GetSolutionColumn().tobytes(), t, s.troubled_cells()))
        s.close()
    assert outs[0] == outs[1]


def test_shock_cells_fp64_with_every_block_flagged_is_the_fp64_form(gpu):
    """weno::Lazy flags every cell, so with FP64 shock cells every block takes
    the FP64 cell update: with the same steps the result is the FP64 form's
    up to the mixed form's seeded square roots in the Riemann fluxes."""
    p = 2
    m = cases.sod_mesh(20, 2, 2)
    u0 = cases.sod_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    out = {}
    for name, kw in (("fp64", dict(precision="fp64")),
                     ("hybrid", dict(precision="mixed", shock_cells_fp64=1))):
        s = Lobatto(m, p, "roe", limiter="lazy", **kw)
        cases.sod_bc(s)
        s.SetSolutionColumn(u0)
        t = 0.0
        for _ in range(5):
            RungeKutta(3).Update(s, t, 2e-4)
            t += 2e-4
        out[name] = s.GetSolutionColumn()
        s.close()
    assert rel_l2(out["hybrid"], out["fp64"]) <= 1e-11, rel_l2(out["hybrid"], out["fp64"])


def test_shock_cells_fp64_track_the_fp64_form_closer(gpu):
    """The four-quadrant problem with weno::Eigen: the mixed form with FP64
    shock cells stays closer to the FP64 form than the plain mixed form."""
    p = 2
    m = cases.quadrant_mesh(32, 32, 2)
    u0 = cases.quadrant_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    out = {}
    for name, kw in (("fp64", dict(precision="fp64")), ("mixed", dict(precision="mixed")),
                     ("hybrid", dict(precision="mixed", shock_cells_fp64=1)),
                     ("hybrid2", dict(precision="mixed", shock_cells_fp64=2))):
        s = Lobatto(m, p, "roe", limiter="eigen", **kw)
        cases.quadrant_bc(s)
        s.SetSolutionColumn(u0)
        s.advance(60, 1.0, 3, 0.0)
        out[name] = s.GetSolutionColumn().reshape(-1, 5)[:, 0]
        s.close()
    e_mixed = rel_l2(out["mixed"], out["fp64"])
    e_hybrid = rel_l2(out["hybrid"], out["fp64"])
    e_hybrid2 = rel_l2(out["hybrid2"], out["fp64"])
    assert e_hybrid < e_mixed and e_hybrid2 <= e_hybrid * 1.5 and e_hybrid <= 1e-6, (e_hybrid, e_hybrid2, e_mixed)


def test_shock_cells_fp64_rejected_without_limiter(gpu):
    m = cases.sod_mesh(4, 2, 2)
    with pytest.raises(Exception):
        Lobatto(m, 2, "roe", precision="mixed", shock_cells_fp64=1)
    with pytest.raises(Exception):
        Lobatto(m, 2, "roe", precision="fp64", limiter="eigen", shock_cells_fp64=1)
