"""Output and restart on the GPU through the C ABI: VTK sampling against the
oracle's Writer<Part>::Prepare, the written files, the DataOnCells field
gather / scatter (Part::GatherSolutions / ScatterSolutions) and the restart
file (Part::WriteSolutions / ReadSolutions)."""
import numpy as np
import pytest
import torch

import oracle.orc as orc
from pvcriemannsolvers_gb300 import General, Lobatto, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def nodal(p, scheme="dgsem", precision="fp64"):
    m = meshlib.box((4, 3, 2), lengths=(1.0, 0.8, 0.6), periodic=(True, False, True), jitter=0.1, seed=0)
    s = Lobatto(m, p, "rusanov", scheme=scheme, precision=precision)
    om = orc.Mesh(m, p, scheme=scheme)
    u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    s.SetSolutionColumn(u)
    return s, om, u


def modal(p, precision="fp64"):
    m = meshlib.concat(meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.1, seed=1),
                       meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.1, seed=2))
    s = General(m, p, "hllc", precision=precision)
    om = orc.Modal(m, p)
    u = om.project(cases.smooth_ic(om.points()[0]))
    s.SetSolutionColumn(u)
    return s, om, u


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def modal_wedges(p):
    m = meshlib.concat(meshlib.box((2, 2, 2), periodic=(True,) * 3, jitter=0.1, seed=1),
                       meshlib.wedge_box((3, 2, 2), periodic=(True,) * 3, jitter=0.1, seed=3))
    s = General(m, p, "hllc")
    om = orc.Modal(m, p)
    u = om.project(cases.smooth_ic(om.points()[0]))
    s.SetSolutionColumn(u)
    return s, om, u


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("kind", ["dgsem", "fr", "modal", "modal_wedges"])
def test_vtk_sample_matches_oracle(kind, p):
    """Writer<Part>::Prepare: Hexahedron27 / Tetrahedron10 / Wedge15 points
    (mesh/vtk.hpp:400-493)."""
    if kind == "modal_wedges":
        s, om, u = modal_wedges(p)
    else:
        s, om, u = modal(p) if kind == "modal" else nodal(p, kind)
    xyz, values, types = s.vtk_sample()
    oxyz, ovalues, otypes = om.vtk_sample(u)
    assert np.array_equal(types, otypes)
    assert xyz.shape == oxyz.shape
    assert rel(xyz, oxyz) <= 1e-14
    assert rel(values, ovalues) <= 1e-13
    s.close()


def test_written_files(tmp_path):
    import xml.etree.ElementTree as ET
    s, om, u = modal(2)
    s.WriteSolutions(tmp_path, "step0")
    assert (tmp_path / "step0.pvtu").read_text() == orc.pvtu_text("step0")
    root = ET.parse(tmp_path / "step0" / "0.vtu").getroot()
    oxyz, ovalues, otypes = om.vtk_sample(u)
    arrays = {da.get("Name"): da for da in root.iter("DataArray")}
    for k, f in enumerate(orc.FIELD_NAMES):
        v = np.array(arrays[f].text.split(), dtype=float)
        # 6 significant digits, as the reference's stream output
        assert np.allclose(v, ovalues[:, k], rtol=1e-5, atol=1e-300)
    assert np.array_equal(np.array(arrays["types"].text.split(), dtype=int), otypes)
    s.WriteSolutions(tmp_path, "step0b", binary=True)
    assert (tmp_path / "step0b" / "0.vtu").exists()
    with pytest.raises(capi.McfdError):
        s.WriteSolutions("/proc/no/such/dir", "x")
    s.close()


@pytest.mark.parametrize("kind", ["dgsem", "modal"])
def test_gather_scatter_fields(kind):
    s, _, u = modal(2) if kind == "modal" else nodal(3)
    n = s.column_size
    cells = s.mesh.n_cells
    fields = torch.empty(n, dtype=torch.float64, device="cuda")
    s.gather_fields_device(fields.data_ptr(), n)
    want = u.reshape(cells, n // cells).T.ravel()  # field i of cell c = value i of its block
    assert np.array_equal(fields.cpu().numpy(), want)
    s.SetSolutionColumn(np.zeros(n))
    s.scatter_fields_device(fields.data_ptr(), n)
    assert np.array_equal(s.GetSolutionColumn(), u)
    with pytest.raises(capi.McfdError):
        s.gather_fields_device(fields.data_ptr(), n - 1)
    s.close()


@pytest.mark.parametrize("kind", ["dgsem", "modal"])
def test_restart_round_trip(tmp_path, kind):
    s, _, u = modal(2) if kind == "modal" else nodal(2)
    t = s.advance(2, 1e9, 3, 0.0)
    path = tmp_path / "state.rst"
    s.write_restart(path, t)
    saved = s.GetSolutionColumn()
    s.SetSolutionColumn(saved)  # both continuations start from a freshly loaded column
    t2 = s.advance(3, 1e9, 3, t)
    after = s.GetSolutionColumn()
    s.SetSolutionColumn(np.zeros(s.column_size))
    assert s.read_restart(path) == t
    assert np.array_equal(s.GetSolutionColumn(), saved)
    # the restarted run continues bit for bit
    assert s.advance(3, 1e9, 3, t) == t2
    assert np.array_equal(s.GetSolutionColumn(), after)
    # a damaged file is refused and the solution kept
    raw = bytearray(path.read_bytes())
    raw[-5] ^= 0x40
    bad = tmp_path / "bad.rst"
    bad.write_bytes(bytes(raw))
    with pytest.raises(capi.McfdError):
        s.read_restart(bad)
    assert np.array_equal(s.GetSolutionColumn(), after)
    s.close()


def test_restart_refuses_other_mesh(tmp_path):
    s, _, _ = nodal(2)
    s.write_restart(tmp_path / "a.rst", 0.0)
    other, _, _ = nodal(3)
    with pytest.raises(capi.McfdError):
        other.read_restart(tmp_path / "a.rst")
    with pytest.raises(capi.McfdError):
        other.read_restart(tmp_path / "missing.rst")
    s.close()
    other.close()


def test_pyramids_have_no_vtk_cell(tmp_path):
    """The reference's writer has no pyramid element (mesh/vtk.hpp:400-414):
    sampling or writing a mesh with pyramids is refused."""
    m = meshlib.pyramid_box((2, 2, 2), periodic=(True,) * 3)
    s = General(m, 2, "hllc")
    with pytest.raises(capi.McfdError):
        s.vtk_sample()
    with pytest.raises(capi.McfdError):
        s.WriteSolutions(str(tmp_path), "frame")
    s.close()
