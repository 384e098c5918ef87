"""Output on the host (no GPU): the library's base64 against the reference's
known-answer vectors (test/mesh/vtk.cpp:17-55), and the .pvtu / .vtu writer
against the oracle's restatement of Writer<Part>::WriteSolutions
(mesh/vtk.hpp:526-669) on oracle-sampled solutions."""
import base64
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import base64_encode, cases, mesh as meshlib, write_vtu_arrays

# (input, encoded) pairs of the reference's EncodeBase64 test
KAT = [("A", "QQ=="), ("AB", "QUI="), ("ABC", "QUJD"), ("ABCD", "QUJDRA=="), ("ABCDE", "QUJDREU="),
       ("ABCDEF", "QUJDREVG"), ("1", "MQ=="), ("12", "MTI="), ("123", "MTIz"), ("1234", "MTIzNA=="),
       ("12345", "MTIzNDU="), ("123456", "MTIzNDU2")]


@pytest.mark.parametrize("text,enc", KAT)
def test_base64_reference_vectors(text, enc):
    assert base64_encode(text.encode()) == enc


def test_base64_binary_bytes():
    rng = np.random.default_rng(0)
    for n in (0, 1, 2, 3, 7, 64, 1001):
        data = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        assert base64_encode(data) == base64.b64encode(data).decode()


def sampled(kind, p):
    if kind == "hex":
        m = meshlib.box((3, 2, 2), periodic=(False, True, True), jitter=0.1, seed=1)
        om = orc.Mesh(m, p)
        u = cases.smooth_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel()
    else:
        m = meshlib.concat(meshlib.box((3, 3, 3), periodic=(True,) * 3, jitter=0.1, seed=1),
                           meshlib.tet_box((3, 3, 3), periodic=(True,) * 3, jitter=0.1, seed=2))
        om = orc.Modal(m, p)
        u = om.project(cases.smooth_ic(om.points()[0]))
    return om, u


@pytest.mark.parametrize("kind,p", [("hex", 2), ("mixed", 2)])
def test_writer_matches_restated_layout(tmp_path, kind, p):
    om, u = sampled(kind, p)
    xyz, values, types = om.vtk_sample(u)
    write_vtu_arrays(tmp_path, "frame", xyz, values, types)
    assert (tmp_path / "frame.pvtu").read_text() == orc.pvtu_text("frame")
    assert (tmp_path / "frame" / "0.vtu").read_text() == orc.vtu_text(xyz, values, types)


def _array(root, name):
    for da in root.iter("DataArray"):
        if da.get("Name") == name:
            return da
    raise KeyError(name)


def _decode(da, dtype):
    text = da.text.strip()
    n = struct.unpack("<Q", base64.b64decode(text[:12]))[0]
    raw = base64.b64decode(text[12:])
    assert len(raw) == n
    return np.frombuffer(raw, dtype=dtype)


def test_binary_writer_round_trip(tmp_path):
    om, u = sampled("mixed", 1)
    xyz, values, types = om.vtk_sample(u)
    write_vtu_arrays(tmp_path, "bin", xyz, values, types, binary=True)
    root = ET.parse(tmp_path / "bin" / "0.vtu").getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == len(xyz) and int(piece.get("NumberOfCells")) == len(types)
    assert np.array_equal(_decode(_array(root, "Points"), "<f8").reshape(-1, 3), xyz)
    for k, f in enumerate(orc.FIELD_NAMES):
        assert np.array_equal(_decode(_array(root, f), "<f8"), values[:, k])
    sizes = np.where(types == 29, 27, 10)
    assert np.array_equal(_decode(_array(root, "offsets"), "<i4"), np.cumsum(sizes))
    assert np.array_equal(_decode(_array(root, "types"), "u1"), types)


def test_writer_rejects_bad_input(tmp_path):
    from pvcriemannsolvers_gb300 import capi
    xyz, values = np.zeros((27, 3)), np.zeros((27, 5))
    with pytest.raises(capi.McfdError):
        write_vtu_arrays(tmp_path, "x", xyz, values, np.array([24], np.uint8))  # 10 != 27 points
    with pytest.raises(capi.McfdError):
        write_vtu_arrays(tmp_path, "x", xyz, values, np.array([12], np.uint8))  # not a written type


def test_oracle_sampling_reproduces_polynomials():
    """The sampled interpolant / projection of a linear field is exact at the
    VTK nodes."""
    a = np.array([0.3, -0.2, 0.5])
    lin = lambda x: 1.0 + x @ a  # noqa: E731
    m = meshlib.box((3, 2, 2), jitter=0.1, seed=3)
    for p in (1, 2, 3):
        om = orc.Mesh(m, p)
        x = meshlib.node_coordinates(m, p).reshape(-1, 3)
        u = np.repeat(lin(x)[:, None], 5, axis=1).ravel()
        xyz, v, _ = om.vtk_sample(u)
        assert np.allclose(v, lin(xyz)[:, None], rtol=0, atol=1e-13)
    mm = meshlib.concat(meshlib.box((2, 2, 2), jitter=0.1, seed=4), meshlib.tet_box((3, 3, 3), jitter=0.1, seed=5))
    for p in (1, 2):
        om = orc.Modal(mm, p)
        u = om.project(np.repeat(lin(om.points()[0])[:, None], 5, axis=1))
        xyz, v, types = om.vtk_sample(u)
        assert len(xyz) == 27 * 8 + 10 * 162 and set(types.tolist()) == {24, 29}
        assert np.allclose(v, lin(xyz)[:, None], rtol=0, atol=1e-12)
