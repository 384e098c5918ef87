"""Synthetic mesh builder and the oracle's reference-style face matching."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import mesh as meshlib


@pytest.mark.parametrize("periodic", [(False, False, False), (True, True, True), (True, False, True)])
def test_box_faces_closed(periodic):
    m = meshlib.box((3, 4, 2), lengths=(1, 2, 3), periodic=periodic)
    # every local face of every cell appears exactly once
    seen = np.zeros((m.n_cells, 6), dtype=int)
    for (h, s), (sh, ss) in zip(m.face_cells, m.face_sides):
        seen[h, sh] += 1
        if s >= 0:
            seen[s, ss] += 1
    assert np.all(seen == 1)
    inner = m.face_cells[:, 1] >= 0
    assert np.all(m.face_cells[inner, 0] < m.face_cells[inner, 1]) or any(periodic)
    assert np.all(m.face_group[inner] == -1)
    assert np.all(m.face_group[~inner] >= 0)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_oracle_near_matching_on_jittered_periodic_mesh(p):
    """spatial/dg/lobatto.hpp:58-78: every face point matches a node of the
    holder and of the sharer (through the periodic shift)."""
    m = meshlib.box((3, 3, 3), lengths=(1, 1, 1), periodic=(True, False, True), jitter=0.1, seed=0)
    om = orc.Mesh(m, p)
    h, s = om.face_node_maps()
    assert h.min() >= 0
    inner = m.face_cells[:, 1] >= 0
    assert s[inner].min() >= 0
    assert np.all(s[~inner] == -1)


def test_jitter_is_seeded_and_bounded():
    a = meshlib.box((4, 4, 4), jitter=0.1, seed=0)
    b = meshlib.box((4, 4, 4), jitter=0.1, seed=0)
    c = meshlib.box((4, 4, 4))
    assert np.array_equal(a.xyz, b.xyz)
    assert np.abs(a.xyz - c.xyz).max() <= 0.1 * 0.25 + 1e-15
