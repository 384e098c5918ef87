"""Batching: independent cases inside one handle (mcfd_set_cases) and
ensembles of handles stepped by one CUDA graph (mcfd_ensemble).  A case must
evolve exactly as it does alone: same per-case time step, same bits."""
import numpy as np
import pytest

from pvcriemannsolvers_gb300 import Ensemble, General, Lobatto, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def wavy_state(x, seed):
    rng = np.random.default_rng(seed)
    rho = np.ones(len(x))
    for _ in range(3):
        k = rng.integers(-2, 3, 3)
        rho += rng.uniform(0, 0.1) * np.sin(2 * np.pi * (x @ k) + rng.uniform(0, 2 * np.pi))
    d = rng.normal(size=3)
    v = rng.uniform(0, 0.5) * d / np.linalg.norm(d)
    n = len(x)
    return cases.prim_to_cons(rho, np.full(n, v[0]), np.full(n, v[1]), np.full(n, v[2]), np.ones(n))


def blocks(kind, shapes, seeds):
    make = meshlib.box if kind == "hex" else meshlib.tet_box
    return [make(s, periodic=(True,) * 3, jitter=0.05, seed=sd) for s, sd in zip(shapes, seeds)]


def load(system, m, seed, modal):
    if modal:
        system.project(wavy_state(system.points(), seed))
    else:
        x = meshlib.node_coordinates(m, system.degree).reshape(-1, 3)
        system.SetSolutionColumn(wavy_state(x, seed).ravel())


def batched(kind, p, scheme, shapes, seeds, riemann="rusanov"):
    parts = blocks(kind, shapes, seeds)
    m = meshlib.concat(*parts)
    modal = scheme == "modal"
    s = General(m, p, riemann) if modal else Lobatto(m, p, riemann, scheme=scheme)
    offsets = np.concatenate([[0], np.cumsum([q.n_cells for q in parts])])
    cols = []
    for q, sd in zip(parts, seeds):
        one = General(q, p, riemann) if modal else Lobatto(q, p, riemann, scheme=scheme)
        load(one, q, sd, modal)
        cols.append(one.GetSolutionColumn())
        one.close()
    s.SetSolutionColumn(np.concatenate(cols))
    s.set_cases(offsets)
    return s, parts


def alone(q, p, scheme, seed, steps, riemann="rusanov"):
    modal = scheme == "modal"
    one = General(q, p, riemann) if modal else Lobatto(q, p, riemann, scheme=scheme)
    load(one, q, seed, modal)
    t = one.advance(steps, 1e9, 3, 0.0)
    out = one.GetSolutionColumn()
    one.close()
    return out, t


@pytest.mark.parametrize("kind,p,scheme", [("hex", 2, "dgsem"), ("hex", 3, "fr"), ("tet", 2, "modal"),
                                           ("hex", 1, "modal")])
def test_cases_evolve_as_alone(gpu, kind, p, scheme):
    shapes, seeds = [(3, 3, 3), (4, 2, 3), (3, 3, 2)], [1, 2, 3]
    s, parts = batched(kind, p, scheme, shapes, seeds)
    steps = 4
    s.advance(steps, 1e9, 3, 0.0)
    sol = s.GetSolutionColumn()
    t_cases, _ = s.case_times()
    off = 0
    for k, (q, sd) in enumerate(zip(parts, seeds)):
        ref, t_ref = alone(q, p, scheme, sd, steps)
        assert t_cases[k] == t_ref
        assert np.array_equal(sol[off:off + ref.size], ref)
        off += ref.size
    s.close()


def test_ensemble_matches_members_alone(gpu):
    a, pa = batched("hex", 3, "dgsem", [(3, 3, 3), (2, 3, 2)], [4, 5])
    b, pb = batched("tet", 2, "modal", [(3, 3, 2), (3, 2, 3)], [6, 7], riemann="hllc")
    c = Lobatto(meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=8), 1, "roe", scheme="fr")
    load(c, meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=8), 8, False)
    ens = Ensemble([a, b, c])
    ens.advance(3, 1e9, 3)
    ens.advance(2, 1e9, 3)
    for sysm, parts, seeds, scheme, p, riemann in ((a, pa, [4, 5], "dgsem", 3, "rusanov"),
                                                   (b, pb, [6, 7], "modal", 2, "hllc")):
        sol = sysm.GetSolutionColumn()
        t_cases, _ = sysm.case_times()
        off = 0
        for k, (q, sd) in enumerate(zip(parts, seeds)):
            ref, t_ref = alone(q, p, scheme, sd, 5, riemann)
            assert t_cases[k] == t_ref
            assert np.array_equal(sol[off:off + ref.size], ref)
            off += ref.size
    qc = meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=8)
    ref, _ = alone(qc, 1, "fr", 8, 5, "roe")
    assert np.array_equal(c.GetSolutionColumn(), ref)
    ens.close()
    for sysm in (a, b, c):
        sysm.close()


def test_cases_must_not_share_faces(gpu):
    m = meshlib.box((4, 2, 2), periodic=(True,) * 3)
    s = Lobatto(m, 1)
    with pytest.raises(capi.McfdError):
        s.set_cases([0, 8, 16])
    with pytest.raises(capi.McfdError):
        s.set_cases([0, 20])
    s.close()


def test_ensemble_stream_matches_sequential(gpu):
    """Streamed ensemble jobs (mcfd_ensemble_stream_*) give the columns of
    set-solution + mcfd_ensemble_advance + get-solution, bit for bit."""
    import torch

    def members():
        a, _ = batched("hex", 2, "dgsem", [(3, 3, 3), (2, 3, 2)], [4, 5])
        b, _ = batched("tet", 2, "modal", [(3, 3, 2), (3, 2, 3)], [6, 7], riemann="hllc")
        c = Lobatto(meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=8), 3, "rusanov",
                    precision="mixed")
        load(c, meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.05, seed=8), 8, False)
        return [a, b, c]

    def pinned(n):
        return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()

    seq = members()
    start = [s.GetSolutionColumn() for s in seq]
    ens = Ensemble(seq)
    want = []
    cols = start
    for job in range(4):
        for s, col in zip(seq, cols):
            s.SetSolutionColumn(col)
        ens.advance(1, 1e9, 3)
        cols = [s.GetSolutionColumn() for s in seq]
        want.append(cols)
    ens.close()
    for s in seq:
        s.close()
    # streamed: job k's input is job k-1's expected output
    stm = members()
    ens = Ensemble(stm)
    ins = [[pinned(c.size) for c in start] for _ in range(4)]
    outs = [[pinned(c.size) for c in start] for _ in range(4)]
    for j in range(4):
        src = start if j == 0 else want[j - 1]
        for dst, col in zip(ins[j], src):
            dst[:] = col
    ens.stream_begin()
    for j in range(4):
        ens.stream_step(ins[j], outs[j], 1, 1e9, 3)
    ens.stream_end()
    for j in range(4):
        for got, ref in zip(outs[j], want[j]):
            assert np.array_equal(got, ref), f"job {j}"
    ens.close()
    for s in stm:
        s.close()
