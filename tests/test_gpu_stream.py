"""Streamed stepping (mcfd_stream_*): each job's result equals the sequential
mcfd_set_solution + mcfd_advance + mcfd_get_solution, bit for bit, while the
uploads and downloads of neighbouring jobs overlap its compute."""
import numpy as np
import pytest
import torch

from pvcriemannsolvers_gb300 import General, Lobatto, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def pinned(n):
    return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()


def job_inputs(system, m, n_jobs, modal):
    out = []
    for j in range(n_jobs):
        rng = np.random.default_rng(j)
        x = system.points() if modal else meshlib.node_coordinates(m, system.degree).reshape(-1, 3)
        rho = 1 + 0.1 * np.sin(2 * np.pi * (x @ rng.integers(-2, 3, 3)) + rng.uniform(0, 6))
        n = len(x)
        v = rng.uniform(-0.3, 0.3, 3)
        cons = cases.prim_to_cons(rho, np.full(n, v[0]), np.full(n, v[1]), np.full(n, v[2]), np.ones(n))
        if modal:
            system.project(cons)
            col = system.GetSolutionColumn()
        else:
            col = cons.ravel()
        buf = pinned(col.size)
        buf[:] = col
        out.append(buf)
    return out


@pytest.mark.parametrize("kind,precision,n_steps", [("dgsem", "fp64", 2), ("dgsem", "mixed", 1),
                                                    ("modal", "fp64", 2), ("fr", "fp64", 1)])
def test_stream_matches_sequential(kind, precision, n_steps):
    modal = kind == "modal"
    if modal:
        m = meshlib.concat(meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=1),
                           meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=2))
        s = General(m, 2, "hllc", precision=precision)
    else:
        m = meshlib.box((5, 4, 3), periodic=(True,) * 3, jitter=0.1, seed=0)
        s = Lobatto(m, 3, "rusanov", precision=precision, scheme=kind)
    n_jobs = 5
    inputs = job_inputs(s, m, n_jobs, modal)
    times = [0.25 * j for j in range(n_jobs)]
    want = []
    for u, t in zip(inputs, times):
        s.SetSolutionColumn(u)
        s.advance(n_steps, 1e9, 3, t)
        want.append(s.GetSolutionColumn())
    own = s.GetSolutionColumn()
    outs = [pinned(s.column_size) for _ in range(n_jobs)]
    for o in outs:
        o[:] = np.nan
    s.stream_begin()
    for u, o, t in zip(inputs, outs, times):
        s.stream_step(u, o, t, n_steps, 1e9, 3)
    s.stream_end()
    for j in range(n_jobs):
        assert np.array_equal(outs[j], want[j]), f"job {j}"
    # the handle's own solution is untouched, and stepping it afterwards
    # (fresh node traces after the jobs overwrote them) gives the same bits
    assert np.array_equal(s.GetSolutionColumn(), own)
    s.SetSolutionColumn(inputs[1])
    s.advance(n_steps, 1e9, 3, times[1])
    assert np.array_equal(s.GetSolutionColumn(), want[1])
    # a second stream reuses the staging and graphs
    s.stream_begin()
    s.stream_step(inputs[0], outs[0], times[0], n_steps, 1e9, 3)
    s.stream_end()
    assert np.array_equal(outs[0], want[0])
    s.close()


def test_stream_with_limiter():
    """With a limiter the loaded column is limited first, as by SetSolutionColumn."""
    m = meshlib.box((6, 4, 3), periodic=(True,) * 3, jitter=0.05, seed=3)
    s = Lobatto(m, 2, "roe", limiter="eigen")
    x = meshlib.node_coordinates(m, 2).reshape(-1, 3)
    n = len(x)
    inputs, want = [], []
    for j in range(3):
        left = x[:, 0] < 0.3 + 0.1 * j
        rho = np.where(left, 1.0, 0.125)
        p = np.where(left, 1.0, 0.1)
        buf = pinned(5 * n)
        buf[:] = cases.prim_to_cons(rho, np.zeros(n), np.zeros(n), np.zeros(n), p).ravel()
        inputs.append(buf)
        s.SetSolutionColumn(buf)
        s.advance(2, 1e9, 3, 0.0)
        want.append(s.GetSolutionColumn())
    outs = [pinned(s.column_size) for _ in inputs]
    s.stream_begin()
    for u, o in zip(inputs, outs):
        s.stream_step(u, o, 0.0, 2, 1e9, 3)
    s.stream_end()
    for j in range(len(inputs)):
        assert np.array_equal(outs[j], want[j]), f"job {j}"
    s.close()


def test_stream_errors():
    m = meshlib.box((3, 3, 3), periodic=(True,) * 3)
    s = Lobatto(m, 1, "rusanov")
    a = pinned(s.column_size)
    b = pinned(s.column_size)
    with pytest.raises(capi.McfdError):
        s.stream_step(a, b, 0.0, 1, 1e9, 3)  # not begun
    s.stream_begin()
    with pytest.raises(ValueError):
        s.stream_step(a[:-1], b, 0.0, 1, 1e9, 3)
    with pytest.raises(capi.McfdError):
        s.stream_step(a, b, 0.0, 1, 1e9, 4)  # RK order
    s.stream_end()
    s.stream_end()  # a second end is a no-op
    s.close()


def test_stream_reports_nonfinite():
    m = meshlib.box((3, 3, 3), periodic=(True,) * 3)
    s = Lobatto(m, 1, "rusanov")
    x = meshlib.node_coordinates(m, 1).reshape(-1, 3)
    a = pinned(s.column_size)
    a[:] = cases.smooth_ic(x).ravel()
    a[7] = np.nan
    b = pinned(s.column_size)
    s.stream_begin()
    s.stream_step(a, b, 0.0, 1, 1e9, 3)
    with pytest.raises(capi.McfdError):
        s.stream_end()
    s.close()
