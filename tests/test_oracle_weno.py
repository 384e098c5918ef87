"""The oracle's WENO limiter against the reference's limiter tests.

* smoothness indicator of the Taylor monomials on [-1,1]^3
  (test/limiter/weno.cpp:45-88: first-order monomials give volume * w1,
  x^2 gives 32/3 w1 + 32 w2, xy gives 16/3 w1 + 8 w2),
* cell averages are preserved by the reconstruction
  (test/limiter/weno.cpp:172-176, 301-305: 1e-13),
* a globally linear field is reproduced exactly (every candidate equals it),
* the jump detector flags the cells next to a discontinuity only.
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import cases, mesh as meshlib

EXPS = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]


def monomial_field(x, exps):
    return np.stack([x[:, 0] ** a * x[:, 1] ** b * x[:, 2] ** c for a, b, c in exps], axis=1)


def test_smoothness_kat():
    m = meshlib.box((1, 1, 1), lengths=(2, 2, 2), origin=(-1, -1, -1))
    om = orc.Mesh(m, 2)
    lim = orc.Limiter(om)
    x = meshlib.node_coordinates(m, 2).reshape(-1, 3)
    volume = 8.0
    w1 = volume ** (2 / 3 - 1)
    w2 = volume ** (4 / 3 - 1) / 4
    want = {(1, 0, 0): volume * w1, (0, 1, 0): volume * w1, (0, 0, 1): volume * w1,
            (2, 0, 0): 32 / 3 * w1 + 32 * w2, (0, 2, 0): 32 / 3 * w1 + 32 * w2, (0, 0, 2): 32 / 3 * w1 + 32 * w2,
            (1, 1, 0): 16 / 3 * w1 + 8 * w2, (1, 0, 1): 16 / 3 * w1 + 8 * w2, (0, 1, 1): 16 / 3 * w1 + 8 * w2}
    for group in (EXPS[:5], EXPS[4:]):
        u = monomial_field(x, group).ravel()
        beta = lim.smoothness(0, lim.modal(u)[0])
        for e, b in zip(group, beta):
            assert abs(b - want[e]) < 1e-12, (e, b, want[e])
    # a constant has zero smoothness indicator
    u = np.ones((x.shape[0], 5)).ravel()
    assert np.abs(lim.smoothness(0, lim.modal(u)[0])).max() < 1e-14


def cell_averages(om, u):
    _, w = om.node_geometry()
    uu = u.reshape(w.shape[0], w.shape[1], 5)
    return (uu * w[..., None]).sum(axis=1) / w.sum(axis=1)[:, None]


@pytest.mark.parametrize("p", [1, 2, 3])
def test_lazy_preserves_cell_averages(p):
    m = meshlib.box((5, 4, 3), lengths=(1, 0.8, 0.6), jitter=0.1, seed=2)
    om = orc.Mesh(m, p)
    lim = orc.Limiter(om, orc.LIMITER_LAZY)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    rng = np.random.default_rng(p)
    u = cases.prim_to_cons(1 + 0.3 * rng.uniform(-1, 1, len(x)), 0.2, 0.1, 0.0, 1 + 0.3 * rng.uniform(-1, 1, len(x))).ravel()
    # first make u a modal (total degree p) field, as after any limiter pass
    u1, n1 = lim.limit(u)
    assert n1 == m.n_cells
    u2, _ = lim.limit(u1)
    np.testing.assert_allclose(cell_averages(om, u2), cell_averages(om, u1), rtol=0, atol=1e-13)


def test_lazy_reproduces_linear_fields():
    m = meshlib.box((4, 3, 3), lengths=(1, 0.8, 0.6), jitter=0.1, seed=5)
    for p in (1, 2):
        om = orc.Mesh(m, p)
        lim = orc.Limiter(om, orc.LIMITER_LAZY)
        x = meshlib.node_coordinates(m, p).reshape(-1, 3)
        u = cases.prim_to_cons(1 + 0.1 * x[:, 0] - 0.2 * x[:, 1], 0.0, 0.0, 0.0, 1 + 0.05 * x[:, 2]).ravel()
        # density and energy are linear in x here; momentum is zero
        v, _ = lim.limit(u)
        np.testing.assert_allclose(v, u, rtol=0, atol=1e-12)


def test_jump_detector_flags_cells_next_to_a_shock():
    m = meshlib.box((12, 2, 2), lengths=(1, 0.2, 0.2))
    om = orc.Mesh(m, 2)
    lim = orc.Limiter(om, orc.LIMITER_DETECT_LAZY)
    x = meshlib.node_coordinates(m, 2).reshape(-1, 3)
    smooth = cases.prim_to_cons(1 + 0.01 * x[:, 0], 0, 0, 0, 1.0).ravel()
    assert not lim.troubled(smooth).any()
    sod = cases.sod_ic(x).ravel()
    flags = lim.troubled(sod)
    centers = m.cell_centers()[:, 0]
    assert flags.any()
    assert np.all(np.abs(centers[flags] - 0.5) < 2 / 12)  # within two cells of the jump


def test_eigen_matrices_are_inverse():
    """test/riemann/euler/eigen.cpp:13-23: L R = R L = I to 1e-15 (scaled)."""
    rng = np.random.default_rng(31415926)
    for _ in range(32):
        prim = [rng.uniform(0.5, 2), *rng.uniform(-1, 1, 3), rng.uniform(0.5, 2)]
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        t = np.cross(n, rng.normal(size=3))
        t /= np.linalg.norm(t)
        frame = np.stack([n, t, np.cross(n, t)])
        L, R = orc.eigen_matrices(orc.prim_to_cons(prim), frame)
        assert np.abs(L @ R - np.eye(5)).max() < 1e-14
        assert np.abs(R @ L - np.eye(5)).max() < 1e-14


@pytest.mark.parametrize("p", [1, 2, 3])
def test_eigen_reconstruction_preserves_means_and_linear_fields(p):
    """weno::Eigen reconstruction (on every cell) keeps every cell average: the
    candidates share it, the weights of a component sum to one and R L = I.
    A linear field is reproduced: every candidate is the same polynomial."""
    m = meshlib.box((4, 3, 3), lengths=(1.0, 1.0, 1.0), periodic=(False,) * 3, jitter=0.1, seed=2)
    om = orc.Mesh(m, p)
    lim = orc.Limiter(om, orc.LIMITER_EIGEN_ALL)
    x = meshlib.node_coordinates(m, p).reshape(-1, 3)
    rng = np.random.default_rng(p)
    n = len(x)
    rho = 1 + 0.5 * (x[:, 0] > 0.5) + 0.05 * rng.uniform(-1, 1, n)
    u = cases.prim_to_cons(rho, np.full(n, 0.2), np.full(n, -0.1), np.zeros(n),
                           1 + 0.3 * (x[:, 1] > 0.4)).ravel()
    before = lim.modal(u)
    out, count = lim.limit(u)
    assert count == m.n_cells
    after = lim.modal(out)
    assert np.abs(after[:, :, 0] - before[:, :, 0]).max() < 1e-12 * np.abs(before[:, :, 0]).max()
    assert not np.allclose(after, before)
    lin = cases.prim_to_cons(1 + 0.1 * x[:, 0], np.full(n, 0.2), np.full(n, 0.1), np.zeros(n),
                             1 + 0.05 * x[:, 1]).ravel()
    out_l, _ = lim.limit(lin)
    assert np.abs(out_l - lin).max() < 1e-12 * np.abs(lin).max()


# ---------------------------------------------------------------- modal scheme
# WithLimiter<dg::General> over Projection (the reference's DGFEM build,
# demo/euler/sourceless.hpp:28-32, 74-80): the same limiter on every cell
# type of the modal scheme, the column holding the modal coefficients.

def modal_mesh(kind, periodic=False, shape=(3, 3, 2), seed=0, lengths=(1.0, 1.0, 1.0)):
    per = (periodic,) * 3
    kw = dict(lengths=lengths, periodic=per, jitter=0.1)
    if kind == "mixed":
        return meshlib.concat(meshlib.box(shape, seed=seed, **kw),
                              meshlib.tet_box(shape, origin=(2.0, 0, 0), seed=seed + 1, **kw))
    make = {"hex": meshlib.box, "tet": meshlib.tet_box, "wedge": meshlib.wedge_box,
            "pyramid": meshlib.pyramid_box}[kind]
    return make(shape, seed=seed, **kw)


@pytest.mark.parametrize("kind", ["hex", "tet", "wedge", "pyramid", "mixed"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_modal_lazy_preserves_averages_and_reproduces_linear_fields(kind, p):
    m = modal_mesh(kind)
    om = orc.Modal(m, p)
    lim = orc.ModalLimiter(om, orc.LIMITER_LAZY)
    x, _ = om.points()
    n = len(x)
    rng = np.random.default_rng(p)
    u = om.project(cases.prim_to_cons(1 + 0.3 * rng.uniform(-1, 1, n), 0.2, 0.1, 0.0,
                                      1 + 0.3 * rng.uniform(-1, 1, n)))
    v, count = lim.limit(u)
    assert count == m.n_cells
    # the constant mode carries the average: psi_0 is the only basis function
    # with a non-zero mean, so the mean of every component is preserved iff
    # coefficient 0 is (limiter/weno.hpp:172-176, 301-305: 1e-13)
    c0_u, c0_v = u.reshape(-1, om.m, 5)[:, 0], v.reshape(-1, om.m, 5)[:, 0]
    assert np.abs(c0_v - c0_u).max() <= 1e-13 * np.abs(c0_u).max()
    assert not np.allclose(v, u)
    # every candidate of a globally linear field is that field
    lin = om.project(cases.prim_to_cons(1 + 0.1 * x[:, 0] - 0.2 * x[:, 1], 0.0, 0.0, 0.0, 1 + 0.05 * x[:, 2]))
    w, _ = lim.limit(lin)
    assert np.abs(w - lin).max() <= 1e-12 * np.abs(lin).max()


@pytest.mark.parametrize("kind", ["tet", "wedge", "pyramid"])
def test_modal_smoothness_of_linear_fields(kind):
    """beta of a linear field g.x on any cell is vol^(2/3 - 1) * vol * |g|^2
    per component (limiter/weno.hpp:25-95 with only first derivatives)."""
    m = modal_mesh(kind, shape=(2, 2, 2))
    om = orc.Modal(m, 2)
    lim = orc.ModalLimiter(om)
    x, w = om.points()
    g = np.array([[0.3, -0.2, 0.5], [1.0, 0.0, 0.0], [0.0, 2.0, 0.0], [0.0, 0.0, -1.5], [0.7, 0.7, 0.7]])
    u = om.project(x @ g.T)
    modal = lim.modal(u)
    # cell volumes from the quadrature: psi_0 = S00 is constant, 1 / S00^2 = vol
    for c in range(m.n_cells):
        vol = 1.0 / lim_s00(modal, u, om, c) ** 2
        beta = lim.smoothness(c, modal[c])
        want = vol ** (2 / 3) * (g * g).sum(axis=1)
        np.testing.assert_allclose(beta, want, rtol=1e-12)


def lim_s00(modal, u, om, c):
    """psi_0 of cell c from a projected constant: coefficient 0 of the
    constant 1 is integral(psi_0) = psi_0 * vol = 1 / psi_0."""
    one = om.project(np.ones((om.n_points, 5)))
    return 1.0 / one.reshape(-1, om.m, 5)[c, 0, 0]


@pytest.mark.parametrize("kind", ["hex", "tet", "mixed"])
def test_modal_eigen_preserves_means_and_detector_flags_the_jump(kind):
    m = modal_mesh(kind, shape=(12, 2, 2), lengths=(1.0, 0.2, 0.2))
    om = orc.Modal(m, 2)
    x, _ = om.points()
    n = len(x)
    smooth = om.project(cases.prim_to_cons(1 + 0.01 * x[:, 0], 0.1, 0.0, 0.0, 1.0 + 0.0 * x[:, 0]))
    lim = orc.ModalLimiter(om, orc.LIMITER_EIGEN)
    assert not lim.troubled(smooth).any()
    jump = om.project(cases.prim_to_cons(1 + 0.8 * (x[:, 0] > 0.53), 0.1, 0.0, 0.0, 1 + 0.5 * (x[:, 0] > 0.53)))
    flags = lim.troubled(jump)
    assert flags.any() and not flags.all()
    out, count = lim.limit(jump)
    assert count == flags.sum()
    c0_in, c0_out = jump.reshape(-1, om.m, 5)[:, 0], out.reshape(-1, om.m, 5)[:, 0]
    assert np.abs(c0_out - c0_in).max() <= 1e-12 * np.abs(c0_in).max()
    # unflagged cells are untouched
    keep = ~flags
    assert np.array_equal(out.reshape(-1, om.m * 5)[keep], jump.reshape(-1, om.m * 5)[keep])
