"""Initial and boundary data of the benchmark configurations.

Every function maps points [M, 3] to conservative states [M, 5]
(rho, rho u, rho v, rho w, rho E) of an ideal gas with gamma = 1.4.
"""
from __future__ import annotations

import math

import numpy as np

from . import mesh as meshlib
from .system import MovingSplit

GAMMA = 1.4


def prim_to_cons(rho, u, v, w, p) -> np.ndarray:
    """PrimitiveToConservative (include/mini/riemann/euler/types.hpp:302-311)."""
    rho, u, v, w, p = np.broadcast_arrays(*(np.asarray(a, dtype=np.float64) for a in (rho, u, v, w, p)))
    e = p * (1.0 / (GAMMA - 1.0)) + rho * (0.5 * (u * u + v * v + w * w))
    return np.stack([rho, rho * u, rho * v, rho * w, e], axis=-1)


# ---------------------------------------------------------------- Sod
SOD_LEFT = prim_to_cons(1.0, 0.0, 0.0, 0.0, 1.0)
SOD_RIGHT = prim_to_cons(0.125, 0.0, 0.0, 0.0, 0.1)


def sod_mesh(nx=100, ny=4, nz=4) -> meshlib.Mesh:
    """[0,1] x [0,0.04]^2 with 100 x 4 x 4 hexahedra (h = 0.01)."""
    return meshlib.box((nx, ny, nz), lengths=(1.0, 0.04, 0.04))


def sod_ic(x: np.ndarray) -> np.ndarray:
    """demo/euler/shock_tube.cpp MyIC with the split at x = 0.5."""
    return np.where((x[:, 0] < 0.5)[:, None], SOD_LEFT[None, :], SOD_RIGHT[None, :])


def sod_bc(system) -> None:
    """shock_tube.cpp MyBC: smart boundaries at both ends, walls elsewhere."""
    system.SetSmartBoundary(0, SOD_LEFT)
    system.SetSmartBoundary(1, SOD_RIGHT)
    for g in (2, 3, 4, 5):
        system.SetInviscidWall(g)


# ---------------------------------------------------------------- vortex
VORTEX_BETA = 5.0
VORTEX_CENTER = (5.0, 5.0)
VORTEX_FREE = (1.0, 1.0, 1.0, 0.0, 1.0)
VORTEX_BOX = 10.0


def vortex_mesh(n: int) -> meshlib.Mesh:
    """[0,10]^3, n^3 hexahedra, periodic in every direction."""
    return meshlib.box((n, n, n), lengths=(VORTEX_BOX,) * 3, periodic=(True, True, True))


def vortex_prim(x: np.ndarray, t: float = 0.0):
    """Shu's isentropic vortex advected by (1, 1, 0) with periodic wrap."""
    rho0, u0, v0, w0, p0 = VORTEX_FREE
    xs = np.mod(x[:, 0] - u0 * t, VORTEX_BOX) - VORTEX_CENTER[0]
    ys = np.mod(x[:, 1] - v0 * t, VORTEX_BOX) - VORTEX_CENTER[1]
    r2 = xs * xs + ys * ys
    b = VORTEX_BETA
    du = -b / (2 * math.pi) * ys * np.exp((1 - r2) / 2)
    dv = b / (2 * math.pi) * xs * np.exp((1 - r2) / 2)
    temp = 1 - (GAMMA - 1) * b * b / (8 * GAMMA * math.pi ** 2) * np.exp(1 - r2)
    rho = temp ** (1 / (GAMMA - 1))
    p = rho ** GAMMA
    return rho, u0 + du, v0 + dv, np.full_like(rho, w0), p


def vortex_ic(x: np.ndarray, t: float = 0.0) -> np.ndarray:
    return prim_to_cons(*vortex_prim(x, t))


# ---------------------------------------------------------------- four quadrants
# demo/euler/riemann2d.cpp:5-25
Q_A = prim_to_cons(1.5, 0.0, 0.0, 0.0, 1.5)
Q_B = prim_to_cons(0.5323, 1.206, 0.0, 0.0, 0.3)
Q_C = prim_to_cons(0.1380, 1.206, 1.206, 0.0, 0.029)
Q_D = prim_to_cons(0.5323, 0.0, 1.206, 0.0, 0.3)
SPEED_CD = (Q_D[1] - Q_C[1]) / (0.5323 - 0.1380)
SPEED_BC = (Q_C[2] - Q_B[2]) / (0.1380 - 0.5323)


def quadrant_mesh(nx=256, ny=256, nz=16) -> meshlib.Mesh:
    return meshlib.box((nx, ny, nz), lengths=(1.0, 1.0, 0.0625))


def quadrant_ic(x: np.ndarray) -> np.ndarray:
    left = (x[:, 0] < 0.8)[:, None]
    low = (x[:, 1] < 0.8)[:, None]
    return np.where(left, np.where(low, Q_C, Q_B), np.where(low, Q_D, Q_A))


def quadrant_bc(system) -> None:
    """riemann2d.cpp:28-53: walls on top/right/front/back, moving-shock smart
    states on the left (x = 0) and bottom (y = 0)."""
    system.SetSmartBoundary(0, MovingSplit(axis=1, position=0.8, speed=SPEED_BC, a=Q_C, b=Q_B))
    system.SetInviscidWall(1)
    system.SetSmartBoundary(2, MovingSplit(axis=0, position=0.8, speed=SPEED_CD, a=Q_C, b=Q_D))
    system.SetInviscidWall(3)
    system.SetInviscidWall(4)
    system.SetInviscidWall(5)


# ---------------------------------------------------------------- smooth
def smooth_ic(x: np.ndarray) -> np.ndarray:
    """rho = 1 + 0.2 sin(2 pi x) cos(2 pi y), u = (0.5, 0.3, 0.1), p = 1."""
    rho = 1 + 0.2 * np.sin(2 * math.pi * x[:, 0]) * np.cos(2 * math.pi * x[:, 1])
    return prim_to_cons(rho, 0.5, 0.3, 0.1, 1.0)


# ---------------------------------------------------------------- mixed box
def mixed_box_mesh(n_hex: int, n_tet: int) -> meshlib.Mesh:
    """Two independent periodic unit-cube blocks: n_hex^3 Hex8 and
    n_tet^3 x 6 Tet4 (Kuhn split), interior nodes jittered U(-0.1 h, 0.1 h)
    with seed 0 (the mixed-element box; 100 / 64 at full size)."""
    a = meshlib.box((n_hex,) * 3, periodic=(True,) * 3, jitter=0.1, seed=0)
    b = meshlib.tet_box((n_tet,) * 3, periodic=(True,) * 3, jitter=0.1, seed=0)
    return meshlib.concat(a, b)


mixed_box_ic = smooth_ic


# ---------------------------------------------------------------- ensemble
def ensemble_spec(n_cases: int = 64, seed: int = 1, scale: float = 1.0) -> list[dict]:
    """The batched ensemble's draw (numpy PCG64): per case an element count
    log-uniform in [4k, 200k] (times scale), Hex8 or 6-tet-split (fair
    draw), p in {1, 2, 3}, DGSEM or modal DG for Hex8 cases (fair draw;
    Tet4 cases are modal), rho = 1 + sum of 3 modes a sin(2 pi k.x + phi)
    with a ~ U(0, 0.1), |k|_inf <= 3, phi ~ U(0, 2 pi), and a uniform
    velocity of magnitude U(0, 0.5) in a direction on the sphere; p = 1."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n_cases):
        count = float(np.exp(rng.uniform(np.log(4000), np.log(200000)))) * scale
        tet = bool(rng.integers(0, 2))
        p = int(rng.integers(1, 4))
        modal_hex = bool(rng.integers(0, 2))
        waves = [(rng.uniform(0, 0.1), rng.integers(-3, 4, 3), rng.uniform(0, 2 * np.pi)) for _ in range(3)]
        d = rng.normal(size=3)
        vel = rng.uniform(0, 0.5) * d / np.linalg.norm(d)
        n = max(3, int(round((count / 6) ** (1 / 3)))) if tet else max(3, int(round(count ** (1 / 3))))
        scheme = "modal" if (tet or modal_hex) else "dgsem"
        specs.append({"case": k, "tet": tet, "p": p, "scheme": scheme, "n": n, "waves": waves, "vel": vel})
    return specs


def ensemble_state(x: np.ndarray, spec: dict) -> np.ndarray:
    """Initial state of one ensemble case at points x."""
    rho = np.ones(len(x))
    for a, kv, phi in spec["waves"]:
        rho += a * np.sin(2 * np.pi * (x @ kv) + phi)
    n = len(x)
    v = spec["vel"]
    return prim_to_cons(rho, np.full(n, v[0]), np.full(n, v[1]), np.full(n, v[2]), np.ones(n))


def ensemble_mesh(spec: dict) -> meshlib.Mesh:
    """Periodic unit cube of one ensemble case (n^3 Hex8 or n^3 x 6 Tet4)."""
    make = meshlib.tet_box if spec["tet"] else meshlib.box
    return make((spec["n"],) * 3, periodic=(True,) * 3)
