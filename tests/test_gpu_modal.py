"""Modal DG (dg::General over Projection) on the GPU against the oracle:
residual, time step, SSP-RK stages, the graph-captured step loop and the
projection, on Hex8, Tet4, Wedge6 and Pyra5 meshes and on block meshes of
several types.  FP64 bar: relative
L2 <= 1e-12."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import General, Lobatto, MovingSplit, RungeKutta, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

RTOL = 1e-12
KINDS = {"exact": orc.EXACT, "hllc": orc.HLLC, "ausm": orc.AUSM, "roe": orc.ROE, "rusanov": orc.RUSANOV}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_mesh(kind, periodic, jitter=0.1, shape=(3, 3, 2), seed=0):
    box = {"hex": meshlib.box, "tet": meshlib.tet_box, "wedge": meshlib.wedge_box,
           "pyramid": meshlib.pyramid_box}.get(kind)
    if kind == "all":
        blocks = [meshlib.box, meshlib.tet_box, meshlib.wedge_box, meshlib.pyramid_box]
        return meshlib.concat(*[fn(shape, origin=(2.0 * i, 0, 0), periodic=periodic, jitter=jitter, seed=seed + i)
                                for i, fn in enumerate(blocks)])
    if kind == "mixed":
        a = meshlib.box(shape, periodic=periodic, jitter=jitter, seed=seed)
        b = meshlib.tet_box(shape, origin=(2.0, 0, 0), periodic=periodic, jitter=jitter, seed=seed + 1)
        return meshlib.concat(a, b)
    return box(shape, periodic=periodic, jitter=jitter, seed=seed)


def smooth_values(x, seed):
    rng = np.random.default_rng(seed)
    rho = 1 + 0.2 * np.sin(2 * np.pi * x[:, 0] + rng.uniform()) * np.cos(2 * np.pi * x[:, 1])
    u = 0.3 + 0.1 * np.sin(2 * np.pi * x[:, 2])
    return cases.prim_to_cons(rho, u, -0.2 + 0.05 * x[:, 0], 0.1, 1.0 + 0.1 * x[:, 1])


# Boundary set on open boxes (group % 6 = x-, x+, y-, y+, z-, z+), the same
# data as the nodal parity tests.
FREE = cases.prim_to_cons(1.0, 0.2, 0.1, -0.1, 1.0).ravel()
LOW = cases.prim_to_cons(0.8, -0.1, 0.0, 0.2, 0.7).ravel()
SPLIT = MovingSplit(axis=0, position=0.5, speed=0.3, a=FREE, b=LOW)
BC_SPECS = [
    (capi.BC_SMART, FREE),
    (capi.BC_SUPERSONIC_OUTLET, None),
    (capi.BC_SMART, SPLIT),
    (capi.BC_INVISCID_WALL, None),
    (capi.BC_SUBSONIC_INLET, np.array([1.3, 0.0, 0.0, 1.0, 2.0 / 287.05])),
    (capi.BC_SUBSONIC_OUTLET, np.array([0, 0, 0, 0, 0.9])),
]
SETTERS = {
    capi.BC_INVISCID_WALL: lambda s, g, v: s.SetInviscidWall(g),
    capi.BC_SUPERSONIC_OUTLET: lambda s, g, v: s.SetSupersonicOutlet(g),
    capi.BC_SMART: lambda s, g, v: s.SetSmartBoundary(g, v),
    capi.BC_SUPERSONIC_INLET: lambda s, g, v: s.SetSupersonicInlet(g, v),
    capi.BC_SUBSONIC_OUTLET: lambda s, g, v: s.SetSubsonicOutlet(g, v),
    capi.BC_SUBSONIC_INLET: lambda s, g, v: s.SetSubsonicInlet(g, v),
}


def apply_bcs(s, o, m):
    specs = {}
    for g in sorted(set(int(g) for g in m.face_group if g >= 0)):
        kind, value = BC_SPECS[g % 6]
        SETTERS[kind](s, g, value)
        specs[g] = (kind, value)
    o.set_bcs(specs)


def build(kind, p, riemann, periodic, seed=0):
    m = make_mesh(kind, periodic, seed=seed)
    s = General(m, p, riemann)
    o = orc.Modal(m, p)
    apply_bcs(s, o, m)
    x, _ = o.points()
    u = o.project(smooth_values(x, seed))
    return m, s, o, u


def test_points_and_projection_match_oracle(gpu):
    for kind in ("hex", "tet", "mixed", "wedge", "pyramid", "all"):
        for p in (1, 2, 3):
            m = make_mesh(kind, (True, True, True))
            s = General(m, p)
            o = orc.Modal(m, p)
            xo, _ = o.points()
            xg = s.points()
            assert np.abs(xg - xo).max() <= 1e-14
            vals = smooth_values(xo, 1)
            s.project(vals)
            assert rel_l2(s.GetSolutionColumn(), o.project(vals)) <= RTOL
            s.close()


@pytest.mark.parametrize("riemann", ["rusanov", "roe", "hllc", "ausm", "exact"])
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("kind", ["hex", "tet", "mixed", "wedge", "pyramid", "all"])
@pytest.mark.parametrize("periodic", [(True, True, True), (False, False, False)])
def test_modal_residual_parity(gpu, riemann, p, kind, periodic):
    """The exact solver's Newton loop stops once f(p) >= -1e-8
    (riemann/euler/exact.hpp:140-152); on smooth fields the face jumps are so
    small that the first f already sits near that threshold, so a last-bit
    difference of pow (CUDA's against the C library's) can add or skip one
    Newton step at a face point and move its flux by up to ~1e-8: the bar for
    that solver is 1e-9."""
    m, s, o, u = build(kind, p, riemann, periodic)
    s.SetSolutionColumn(u)
    s.SetTime(0.1)
    r = s.GetResidualColumn()
    ro = o.residual(KINDS[riemann], u, 0.1)
    bar = 1e-9 if riemann == "exact" else RTOL
    assert rel_l2(r, ro) <= bar, rel_l2(r, ro)
    s.close()


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("kind", ["hex", "tet", "mixed", "wedge", "pyramid", "all"])
def test_modal_time_step_and_rk_parity(gpu, order, kind):
    p = 2
    m, s, o, u = build(kind, p, "hllc", (True, False, True), seed=2)
    s.SetSolutionColumn(u)
    s.SetTime(0.0)
    dt_gpu = s.GetTimeStep(1.0, order)
    dt_orc = o.time_step(u, 1.0, order)
    assert abs(dt_gpu - dt_orc) <= 1e-14 * dt_orc
    RungeKutta(order).Update(s, 0.0, dt_orc)
    uo = o.rk_update(orc.HLLC, order, 0.0, dt_orc, u)
    assert rel_l2(s.GetSolutionColumn(), uo) <= RTOL
    s.close()


def test_modal_advance_matches_oracle_loop(gpu):
    """mcfd_advance (device dt + graph-captured SSP-RK3) on the mixed mesh."""
    m, s, o, u = build("mixed", 2, "hllc", (True, True, True), seed=4)
    s.SetSolutionColumn(u)
    t_end = s.advance(5, 1e9, 3, 0.0)
    t = 0.0
    for _ in range(5):
        dt = o.time_step(u, 1e9, 3, 0.0)
        u = o.rk_update(orc.HLLC, 3, t, dt, u)
        t += dt
    assert abs(t_end - t) <= 1e-13 * t
    assert rel_l2(s.GetSolutionColumn(), u) <= RTOL
    s.close()


def test_modal_rejections(gpu):
    m = meshlib.tet_box((3, 3, 2), periodic=(True,) * 3)
    with pytest.raises(capi.McfdError):
        Lobatto(m, 2)                            # Tet4 cells need the modal scheme
    hexes = meshlib.box((2, 2, 2), periodic=(True,) * 3)
    with pytest.raises(capi.McfdError):
        Lobatto(hexes, 4, scheme="modal")            # degree beyond 3


@pytest.mark.parametrize("kind", ["hex", "tet", "mixed", "wedge", "pyramid"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_modal_mixed_form_accuracy(gpu, kind, p):
    """Mixed modal form (FP32 contractions, FP64 Riemann and RK): residual
    within 1e-4 of the oracle (the residual of this near-uniform field is
    ~1e-3 of the fluxes whose FP32 contraction error it inherits), and 20
    SSP-RK3 steps within 1e-6 density L2 of the FP64 GPU path (the bar of the
    mixed form)."""
    m = make_mesh(kind, (True, True, True), seed=3)
    o = orc.Modal(m, p)
    x, _ = o.points()
    u0 = o.project(smooth_values(x, 5))
    s = General(m, p, "hllc", precision="mixed")
    s.SetSolutionColumn(u0)
    r = s.GetResidualColumn()
    assert rel_l2(r, o.residual(orc.HLLC, u0)) < 1e-4
    out = {}
    for prec in ("fp64", "mixed"):
        sys_ = General(m, p, "hllc", precision=prec)
        sys_.SetSolutionColumn(u0)
        t = sys_.advance(20, 1e9, 3, 0.0)
        out[prec] = (sys_.GetSolutionColumn(), t)
        sys_.close()
    a = out["mixed"][0].reshape(-1, 5)
    b = out["fp64"][0].reshape(-1, 5)
    # density coefficients on the orthonormal basis: their L2 is the field's L2
    assert np.linalg.norm(a[:, 0] - b[:, 0]) / np.linalg.norm(b[:, 0]) <= 1e-6
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 1e-6 * out["fp64"][1]
    s.close()
