"""The FP64 time step of the nodal forms on states that stress its two passes.

The FP64 dt reduction first brackets every node's rate max(|u| + c, 1e-5) *
cell_rate in FP32 interval arithmetic and forms the FP64 rate only where a
node can hold the maximum.  Each case below plants the node of the largest
rate (or a node that must not become it) in one of the forms the bracket
treats specially: a pressure cancelling against the kinetic energy, values
above the FP32 range, momenta below it, a state the positivity clamp zeroes,
zero density, and a near-tie of many nodes.  The bar is the plain FP64
step's own: within 1e-14 of the oracle's dt (the GetTimeStep rule of
spatial/dg/lobatto.hpp:213-233 with the cell lengths of the oracle).
"""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Lobatto, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

P = 2
N = (P + 1) ** 3


def base_state(n_nodes, seed):
    rng = np.random.default_rng(seed)
    rho = 1 + 0.2 * rng.uniform(-1, 1, n_nodes)
    vel = 0.5 * rng.uniform(-1, 1, (3, n_nodes))
    p = 1 + 0.2 * rng.uniform(-1, 1, n_nodes)
    return cases.prim_to_cons(rho, vel[0], vel[1], vel[2], p)  # [nodes][5]


def cons(rho, u, v, w, p):
    return np.asarray(cases.prim_to_cons(rho, u, v, w, p), dtype=np.float64).ravel()


def plant(kind, u, rng):
    n = u.shape[0]
    k = int(rng.integers(n))
    if kind == "cancelling_pressure":
        # p / E about 1e-9: the bracket cannot bound the pressure, FP64 decides
        q = cons(1.0, 40.0, -3.0, 2.0, 1.0)
        ke = 0.5 * (q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]
        q[4] = ke * (1 + 2.5e-9)
        u[k] = q
    elif kind == "moderate_cancellation":
        # p / E about 1e-5: bracketed, within the widening of the bounds
        q = cons(1.0, 30.0, 1.0, -1.0, 1.0)
        ke = 0.5 * (q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]
        q[4] = ke * (1 + 2.5e-5)
        u[k] = q
    elif kind == "above_fp32_range":
        u[k] = cons(1.0, 0.1, 0.0, 0.0, 1e40)
    elif kind == "density_above_fp32_range":
        u[k] = cons(1e39, 3.0, 0.0, 0.0, 1e39)
    elif kind == "tiny_momenta":
        u[:, 1:4] = np.sign(u[:, 1:4]) * 1e-42
        u[k] = cons(0.5, 0.0, 0.0, 0.0, 4.0)
        u[k, 1:4] = -3e-41
    elif kind == "clamped_state":
        # large momentum and E below the kinetic energy: the clamp zeroes the
        # state and its rate is the floor, not the largest
        q = cons(1.0, 80.0, 0.0, 0.0, 1.0)
        q[4] = 0.5 * q[1] ** 2 * 0.9
        u[k] = q
        u[(k + 7) % n, 4] = -1.0       # negative energy: clamped too
    elif kind == "zero_density":
        u[k] = [0.0, 0.0, 0.0, 0.0, 1.0]
    elif kind == "near_tie":
        idx = rng.choice(n, 96, replace=False)
        q = cons(1.0, 2.0, 0.5, -0.5, 1.5)
        for j, i in enumerate(idx):
            u[i] = q * (1 + 1e-15 * (j % 7 - 3))
    else:
        raise ValueError(kind)


KINDS = ["cancelling_pressure", "moderate_cancellation", "above_fp32_range",
         "density_above_fp32_range", "tiny_momenta", "clamped_state", "zero_density", "near_tie"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("shape", [(4, 3, 3), (9, 8, 7)])
def test_fp64_time_step_matches_oracle(gpu, kind, shape):
    m = meshlib.box(shape, lengths=(1.0, 0.8, 0.6), periodic=(True,) * 3, jitter=0.1, seed=1)
    s = Lobatto(m, P, "rusanov")
    om = orc.Mesh(m, P)
    rng = np.random.default_rng(KINDS.index(kind))
    u = base_state(m.n_cells * N, seed=4)
    plant(kind, u, rng)
    col = u.ravel()
    s.SetSolutionColumn(col)
    dt_gpu = s.GetTimeStep(1.0, 3)
    dt_orc = om.time_step(col, 1.0, 3)
    assert dt_orc > 0
    assert abs(dt_gpu - dt_orc) <= 1e-14 * dt_orc, (dt_gpu, dt_orc)
    # repeated calls give the same bits (no state carried between reductions)
    assert s.GetTimeStep(1.0, 3) == dt_gpu
    s.close()
