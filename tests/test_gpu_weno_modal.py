"""WENO limiter on the modal scheme (WithLimiter<dg::General> over
Projection, the reference's DGFEM build: demo/euler/sourceless.hpp:28-32,
74-80; limiter/reconstruct.hpp:21-54; limiter/weno.hpp:97-348) on the GPU
against the oracle's restatement, on every cell type: hexahedra,
tetrahedra, wedges, pyramids, curved cells and block meshes mixing them.

Bar: 1e-12 relative L2 on the limited column and on limited SSP-RK3 steps,
identical troubled-cell counts; the demo's second reconstruction of
tetrahedral meshes (sourceless.cpp:141-143); graph-captured steps equal to
the step-by-step updates; two runs of a limited step bitwise equal.
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import General, RungeKutta, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MODES = {"lazy": orc.LIMITER_LAZY, "detect_lazy": orc.LIMITER_DETECT_LAZY, "eigen": orc.LIMITER_EIGEN}
KINDS = ["hex", "tet", "wedge", "pyramid", "mixed", "all", "curved"]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def wavy(eps=0.02):
    """x + eps (sin 2 pi y sin 2 pi z, ...): a smooth deformation of the
    quadratic cells' nodes."""
    def fn(x):
        s = np.sin(2 * np.pi * x)
        y = x.copy()
        y[:, 0] += eps * s[:, 1] * s[:, 2]
        y[:, 1] += eps * s[:, 2] * s[:, 0]
        y[:, 2] += eps * s[:, 0] * s[:, 1]
        return y
    return fn


def make_mesh(kind, periodic, shape=(4, 3, 2), seed=0):
    """Blocks of [0, 1] x [0, 0.6] x [0, 0.4]; periodic in y and z when
    `periodic` (the jump along x is not wrapped)."""
    per = (False, periodic, periodic)
    kw = dict(lengths=(1.0, 0.6, 0.4), periodic=per, jitter=0.1)
    blocks = {"hex": meshlib.box, "tet": meshlib.tet_box, "wedge": meshlib.wedge_box,
              "pyramid": meshlib.pyramid_box}
    if kind in blocks:
        return blocks[kind](shape, seed=seed, **kw)
    if kind == "mixed":
        return meshlib.concat(meshlib.box(shape, seed=seed, **kw),
                              meshlib.tet_box(shape, origin=(2.0, 0, 0), seed=seed + 1, **kw))
    parts = [fn(shape, origin=(2.0 * i, 0, 0), seed=seed + i, **kw)
             for i, fn in enumerate(blocks.values())]
    m = meshlib.concat(*parts)
    if kind == "curved":
        m = meshlib.deform(meshlib.quadratic(m), wavy())
    return m


def jump_state(x, rng):
    """A Sod-like jump along x in every block (block i spans [2i, 2i + 1])
    with a small perturbation, so that the detector flags some cells."""
    xl = np.mod(x[:, 0], 2.0)
    rho = np.where(xl < 0.45, 1.0, 0.2) * (1 + 0.02 * rng.uniform(-1, 1, len(x)))
    p = np.where(xl < 0.45, 1.0, 0.15)
    n = len(x)
    return cases.prim_to_cons(rho, np.full(n, 0.1), np.full(n, -0.05), np.full(n, 0.02), p)


def mild_jump_state(x, rng):
    """A jump of density ratio 2 and pressure ratio 2.5: the limited scheme
    stays positive over the stepping tests' steps (with the 5:1 jump of
    jump_state the oracle's own limited run of the hexahedral and pyramid
    blocks turns non-finite within three steps)."""
    xl = np.mod(x[:, 0], 2.0)
    rho = np.where(xl < 0.45, 1.0, 0.5) * (1 + 0.02 * rng.uniform(-1, 1, len(x)))
    p = np.where(xl < 0.45, 1.0, 0.4)
    n = len(x)
    return cases.prim_to_cons(rho, np.full(n, 0.1), np.full(n, -0.05), np.full(n, 0.02), p)


def load_pair(m, p, mode, precision="fp64", seed=1, riemann="hllc", state=jump_state):
    s = General(m, p, riemann, precision=precision, limiter=mode)
    om = orc.Modal(m, p)
    lim = orc.ModalLimiter(om, MODES[mode])
    u = om.project(state(om.points()[0], np.random.default_rng(seed)))
    return s, om, lim, u


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("kind", KINDS)
def test_modal_limiter_parity(gpu, kind, p, mode):
    m = make_mesh(kind, periodic=(kind in ("hex", "tet", "mixed")))
    s, om, lim, u = load_pair(m, p, mode)
    s.SetSolutionColumn(u)  # WithLimiter::SetSolutionColumn limits
    got = s.GetSolutionColumn()
    want, n_orc = lim.limit(u)
    assert s.troubled_cells() == n_orc
    if mode == "lazy":
        assert n_orc == m.n_cells
    else:
        assert 0 < n_orc < m.n_cells
    assert rel_l2(got, want) <= RTOL, rel_l2(got, want)
    s.close()


@pytest.mark.parametrize("kind", ["tet", "mixed"])
def test_approximate_then_second_reconstruct_of_tetra_meshes(gpu, kind):
    """demo/euler/sourceless.cpp:134-143: Approximate (which limits, as
    WithLimiter::Approximate does) and, on tetrahedral meshes, a second
    limiter::Reconstruct."""
    p = 2
    m = make_mesh(kind, periodic=False)
    s = General(m, p, "exact", limiter="lazy")
    om = orc.Modal(m, p)
    lim = orc.ModalLimiter(om, orc.LIMITER_LAZY)
    rng = np.random.default_rng(3)
    vals = jump_state(om.points()[0], rng)
    s.project(vals)
    assert s.troubled_cells() == m.n_cells
    assert s.Limit() == m.n_cells
    want, _ = lim.limit(lim.limit(om.project(vals))[0])
    assert rel_l2(s.GetSolutionColumn(), want) <= RTOL
    s.close()


BC = {0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SUPERSONIC_OUTLET, None),
      2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
      4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)}


def set_bcs(s, om, n_blocks, groups=tuple(BC)):
    specs = {}
    for b in range(n_blocks):
        for g in groups:
            spec = BC[g]
            specs[b * 6 + g] = spec
            kind, value = spec
            if kind == orc.BC_SMART:
                s.SetSmartBoundary(b * 6 + g, value)
            elif kind == orc.BC_SUPERSONIC_OUTLET:
                s.SetSupersonicOutlet(b * 6 + g)
            else:
                s.SetInviscidWall(b * 6 + g)
    om.set_bcs(specs)


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("kind", ["tet", "mixed", "all"])
def test_limited_rk3_parity(gpu, kind, mode):
    """SSP-RK3 on WithLimiter<dg::General>: the limiter after every stage,
    smart inlet, outlet and walls; the GPU's own time step."""
    p = 2
    m = make_mesh(kind, periodic=False)
    s, om, lim, u = load_pair(m, p, mode, riemann="roe", state=mild_jump_state)
    set_bcs(s, om, {"tet": 1, "mixed": 2, "all": 4}[kind])
    s.SetSolutionColumn(u)
    u, _ = lim.limit(u)
    t = 0.0
    for k in range(3):
        dt = om.time_step(u, 1.0, 3, 0.0)
        assert abs(s.GetTimeStep(1.0, 3) - dt) <= RTOL * dt
        RungeKutta(3).Update(s, t, dt)
        u = lim.rk_update(orc.ROE, 3, t, dt, u)
        t += dt
        err = rel_l2(s.GetSolutionColumn(), u)
        assert err <= RTOL, (k, err)
    s.close()


def test_limited_advance_graph_equals_stepwise_and_is_deterministic(gpu):
    """mcfd_advance (captured step: dt, stages, limiter passes) equals the
    oracle's step loop, and two runs from the same state are bitwise equal
    (the troubled-cell list is filled in atomic order, but every
    reconstruction reads only the modal buffer and writes only its cell)."""
    p = 2
    m = make_mesh("mixed", periodic=True)
    outs = []
    for run in range(2):
        s, om, lim, u = load_pair(m, p, "eigen", riemann="hllc", state=mild_jump_state)
        set_bcs(s, om, 2, groups=(0, 1))  # y and z are periodic
        s.SetSolutionColumn(u)
        t = s.advance(4, 1.0, 3, 0.0)
        outs.append(s.GetSolutionColumn())
        s.close()
    assert outs[0].tobytes() == outs[1].tobytes()
    u, _ = lim.limit(u)
    t_orc = 0.0
    for _ in range(4):
        dt = om.time_step(u, 1.0, 3, 0.0)
        u = lim.rk_update(orc.HLLC, 3, t_orc, dt, u)
        t_orc += dt
    assert abs(t - t_orc) <= RTOL * t_orc
    assert rel_l2(outs[0], u) <= RTOL


def test_mixed_form_limited_density_close_to_fp64(gpu):
    p = 2
    m = make_mesh("mixed", periodic=True)
    res = {}
    for precision in ("fp64", "mixed"):
        s, om, lim, u = load_pair(m, p, "detect_lazy", precision=precision, riemann="hllc",
                                  state=mild_jump_state)
        set_bcs(s, om, 2, groups=(0, 1))  # y and z are periodic
        s.SetSolutionColumn(u)
        s.advance(5, 1.0, 3, 0.0)
        res[precision] = s.GetSolutionColumn().reshape(-1, om.m, 5)[:, :, 0]
        s.close()
    err = rel_l2(res["mixed"], res["fp64"])
    assert err <= 1e-6, err
