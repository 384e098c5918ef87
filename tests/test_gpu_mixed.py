"""The mixed-precision form (FP32 volume flux + contraction, FP64 Riemann
fluxes, lift and RK accumulation) against the FP64 oracle.

Bar (BASELINE the benchmark spec): relative L2 density error <= 1e-6 against the
FP64 path after the stated step count, smooth-case convergence preserved.
"""
import math

import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Lobatto, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

MIXED_L2_BAR = 1e-6


def density_l2(a, b):
    ra, rb = a.reshape(-1, 5)[:, 0], b.reshape(-1, 5)[:, 0]
    return float(np.linalg.norm(ra - rb) / np.linalg.norm(rb))


def test_mixed_residual_close_to_oracle(gpu):
    m = meshlib.box((4, 4, 4), lengths=(10.0,) * 3, periodic=(True,) * 3, jitter=0.1, seed=1)
    s = Lobatto(m, 3, "rusanov", precision="mixed")
    om = orc.Mesh(m, 3)
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    s.SetSolutionColumn(u)
    r = s.GetResidualColumn()
    ro = om.residual(orc.RUSANOV, u)
    err = np.linalg.norm(r - ro) / np.linalg.norm(ro)
    assert err < 1e-5, err
    s.close()


@pytest.mark.parametrize("n,steps", [(8, 100), (16, 100)])
def test_mixed_vortex_density_error(gpu, n, steps):
    """100 SSP-RK3 steps of the vortex (DGSEM p=3, Rusanov, CFL 0.1): mixed vs
    FP64 (the FP64 GPU path equals the oracle to 1e-12, test_gpu_dgsem_parity)."""
    m = cases.vortex_mesh(n)
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    u0 = cases.vortex_ic(x).ravel()
    out = {}
    for prec in ("fp64", "mixed"):
        s = Lobatto(m, 3, "rusanov", cfl=0.1, precision=prec)
        s.SetSolutionColumn(u0)
        t = s.advance(steps, 1e9, 3, 0.0)
        out[prec] = (s.GetSolutionColumn(), t)
        s.close()
    err = density_l2(out["mixed"][0], out["fp64"][0])
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 1e-6 * out["fp64"][1]
    assert err <= MIXED_L2_BAR, err


def test_mixed_oracle_direct_small(gpu):
    """20 steps on 6^3 against the CPU oracle itself."""
    n, steps, cfl = 6, 20, 0.1
    m = cases.vortex_mesh(n)
    om = orc.Mesh(m, 3)
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    s = Lobatto(m, 3, "rusanov", cfl=cfl, precision="mixed")
    s.SetSolutionColumn(u)
    s.advance(steps, 1e9, 3, 0.0)
    t = 0.0
    for _ in range(steps):
        dt = om.time_step(u, 1e9, 3, cfl)
        u = om.rk_update(orc.RUSANOV, 3, t, dt, u)
        t += dt
    assert density_l2(s.GetSolutionColumn(), u) <= MIXED_L2_BAR
    s.close()


def test_mixed_convergence_order_preserved(gpu):
    """Error against the exact advected vortex drops between 8^3 and 16^3 at
    the same rate for both forms (fixed final time)."""
    errs = {"fp64": [], "mixed": []}
    t_end = 0.5
    for n in (8, 16):
        m = cases.vortex_mesh(n)
        x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
        w1 = np.array([1 / 6, 5 / 6, 5 / 6, 1 / 6])
        w = np.tile(np.einsum("i,j,k->ijk", w1, w1, w1).ravel(), m.n_cells)
        rho_ex = cases.vortex_prim(x, t_end)[0]
        for prec in errs:
            s = Lobatto(m, 3, "rusanov", precision=prec)
            s.SetSolutionColumn(cases.vortex_ic(x).ravel())
            dt = 0.1 * (10.0 / n) / 4.0
            steps = int(math.ceil(t_end / dt))
            dt = t_end / steps
            t = 0.0
            for _ in range(steps):
                from pvcriemannsolvers_gb300 import RungeKutta
                RungeKutta(3).Update(s, t, dt)
                t += dt
            rho = s.GetSolutionColumn().reshape(-1, 5)[:, 0]
            errs[prec].append(math.sqrt(np.sum(w * (rho - rho_ex) ** 2) / np.sum(w * rho_ex ** 2)))
            s.close()
    order = {k: math.log2(v[0] / v[1]) for k, v in errs.items()}
    assert order["fp64"] > 2.5, errs
    assert abs(order["mixed"] - order["fp64"]) < 0.1, (order, errs)


def test_mixed_fr_vortex_density_error(gpu):
    """fr::Lobatto in the mixed form: 50 steps on 8^3 against the FP64 FR path."""
    m = cases.vortex_mesh(8)
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    u0 = cases.vortex_ic(x).ravel()
    out = {}
    for prec in ("fp64", "mixed"):
        s = Lobatto(m, 3, "rusanov", cfl=0.1, precision=prec, scheme="fr")
        s.SetSolutionColumn(u0)
        t = s.advance(50, 1e9, 3, 0.0)
        out[prec] = (s.GetSolutionColumn(), t)
        s.close()
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 1e-6 * out["fp64"][1]
    err = density_l2(out["mixed"][0], out["fp64"][0])
    assert err <= MIXED_L2_BAR, err


@pytest.mark.parametrize("scheme", ["dg", "fr"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_mixed_affine_metric_terms(gpu, scheme, p):
    """Uniform boxes have affine cells, and the mixed form then keeps its FP32
    metric terms once per cell (adj(J), 1/det(J)) scaled by the node weights.
    Its residual must match the oracle to FP32 accuracy, and match the
    per-node metric path of a box whose nodes moved by 1e-9 of a cell (not
    affine any more) to the size of that move."""
    kw = {} if scheme == "dg" else {"scheme": "fr"}
    om_kw = () if scheme == "dg" else ("fr",)
    res = {}
    for jitter in (0.0, 1e-9):
        m = meshlib.box((5, 4, 3), lengths=(10.0, 8.0, 6.0), periodic=(True,) * 3, jitter=jitter, seed=3)
        s = Lobatto(m, p, "rusanov", precision="mixed", **kw)
        x = meshlib.node_coordinates(m, p).reshape(-1, 3)
        u = cases.vortex_ic(x).ravel()
        s.SetSolutionColumn(u)
        res[jitter] = s.GetResidualColumn()
        if jitter == 0.0:
            ro = orc.Mesh(m, p, *om_kw).residual(orc.RUSANOV, u)
            err = np.linalg.norm(res[jitter] - ro) / np.linalg.norm(ro)
            assert err < 1e-5, err
        s.close()
    d = np.linalg.norm(res[0.0] - res[1e-9]) / np.linalg.norm(res[1e-9])
    assert d < 1e-5, d
