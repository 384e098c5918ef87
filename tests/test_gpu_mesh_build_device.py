"""The GPU connectivity builder (mcfd_build_faces_gpu) gives the host
builder's faces index for index, errors included."""
import numpy as np
import pytest

from pvcriemannsolvers_gb300 import capi, mesh as meshlib

pytestmark = pytest.mark.gpu


def periodic_spec(m, periodic):
    return [(2 * ax, 2 * ax + 1, tuple(-m.lengths[ax] if e == ax else 0.0 for e in range(3)))
            for ax in range(3) if periodic[ax]]


def same(a, b):
    for f in ("face_cells", "face_sides", "face_group", "face_shift"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


@pytest.mark.parametrize("maker,quad", [("box", False), ("tet_box", False), ("box", True), ("tet_box", True)])
@pytest.mark.parametrize("periodic", [(False, False, False), (True, False, True)])
def test_gpu_builder_matches_host(maker, quad, periodic):
    make = getattr(meshlib, maker)
    open_mesh = make((5, 4, 3), lengths=(1.0, 0.8, 1.3), jitter=0.1, seed=11)
    want = make((5, 4, 3), lengths=(1.0, 0.8, 1.3), periodic=periodic, jitter=0.1, seed=11)
    src = meshlib.quadratic(open_mesh) if quad else open_mesh
    bn, bg = meshlib.boundary_elements(open_mesh)
    spec = periodic_spec(want, periodic)
    host = meshlib.build(src.xyz, src.cell_nodes, src.cell_type, bn, bg, spec)
    gpu = meshlib.build(src.xyz, src.cell_nodes, src.cell_type, bn, bg, spec, device=0)
    same(gpu, host)
    same(gpu, want)


def test_gpu_builder_large_mixed():
    m = meshlib.concat(meshlib.box((30, 30, 30), jitter=0.1, seed=1), meshlib.tet_box((12, 12, 12), jitter=0.1, seed=2))
    bn, bg = meshlib.boundary_elements(m)
    host = meshlib.build(m.xyz, m.cell_nodes, m.cell_type, bn, bg)
    gpu = meshlib.build(m.xyz, m.cell_nodes, m.cell_type, bn, bg, device=0)
    same(gpu, host)


def test_gpu_builder_errors():
    m = meshlib.box((2, 2, 1))
    with pytest.raises(capi.McfdError, match="more than two"):
        meshlib.build(m.xyz, np.concatenate([m.cell_nodes, m.cell_nodes[:1]]), device=0)
    bad = m.cell_nodes.copy()
    bad[0, 0] = m.xyz.shape[0]
    with pytest.raises(capi.McfdError, match="out of range"):
        meshlib.build(m.xyz, bad, device=0)


@pytest.mark.parametrize("quad", [False, True])
@pytest.mark.parametrize("maker", ["wedge_box", "pyramid_box"])
@pytest.mark.parametrize("periodic", [(False, False, False), (True, False, True)])
def test_gpu_builder_wedges_and_pyramids(maker, periodic, quad):
    """Wedge6 / Pyra5 cells (triangle and quadrangle faces of one cell) and
    their quadratic Wedge18 / Pyra14 forms."""
    host = getattr(meshlib, maker)((4, 3, 3), lengths=(1.0, 0.8, 1.3), periodic=periodic, jitter=0.1, seed=5)
    bn, bg = meshlib.boundary_elements(getattr(meshlib, maker)((4, 3, 3), lengths=(1.0, 0.8, 1.3),
                                                               jitter=0.1, seed=5))
    spec = periodic_spec(host, periodic)
    src = meshlib.quadratic(host) if quad else host
    gpu = meshlib.build(src.xyz, src.cell_nodes, src.cell_type, bn, bg, spec, device=0)
    same(gpu, host)
