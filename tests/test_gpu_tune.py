"""mcfd_autotune: launch shapes change no result bit, and the JSON-lines
cache answers a second request for the same configuration."""
import numpy as np
import pytest

from pvcriemannsolvers_gb300 import General, Lobatto, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def _run(system, u0, steps=3):
    system.SetSolutionColumn(u0)
    system.advance(steps, 1e9, 3, 0.0)
    return system.GetSolutionColumn()


@pytest.mark.parametrize("kind", ["dgsem_mixed", "sod_eigen", "modal"])
def test_autotune_keeps_results_and_caches(gpu, kind, tmp_path):
    if kind == "dgsem_mixed":
        m = meshlib.box((6, 6, 6), lengths=(10.0,) * 3, periodic=(True,) * 3)
        make = lambda: Lobatto(m, 3, "rusanov", cfl=0.1, precision="mixed")
        u0 = cases.vortex_ic(meshlib.node_coordinates(m, 3).reshape(-1, 3)).ravel()
    elif kind == "sod_eigen":
        m = cases.sod_mesh(30, 2, 2)
        def make():
            s = Lobatto(m, 2, "roe", limiter="eigen")
            cases.sod_bc(s)
            return s
        u0 = cases.sod_ic(meshlib.node_coordinates(m, 2).reshape(-1, 3)).ravel()
    else:
        m = meshlib.concat(meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.1),
                           meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.1))
        make = lambda: General(m, 2, "hllc")
        g = make()
        g.Approximate(cases.smooth_ic)
        u0 = g.GetSolutionColumn()
        g.close()
    a = make()
    want = _run(a, u0)
    a.close()
    b = make()
    b.SetSolutionColumn(u0)
    cache = str(tmp_path / "tune.jsonl")
    first = b.autotune(cache)
    assert not first["from_cache"]
    assert first["face_block"] in (128, 256, 512) and first["dt_block"] in (128, 256, 512)
    assert np.array_equal(_run(b, u0), want)
    c = make()
    c.SetSolutionColumn(u0)
    second = c.autotune(cache)
    assert second["from_cache"] and second["face_block"] == first["face_block"]
    assert np.array_equal(_run(c, u0), want)
    b.close()
    c.close()
