"""The mixed form's DGSEM differentiation on the tensor cores (TF32x3
compensated mma.sync products with FP32 accumulation, p = 3) against the
FP32 SIMT path and the oracle: the residual within the mixed form's
tolerance of both, and the density after 20 SSP-RK3 steps within the mixed
form's 1e-6 bar of the FP64 form."""
import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import Lobatto, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tensor_contraction_residual(gpu):
    m = meshlib.box((5, 4, 3), lengths=(10.0, 8.0, 6.0), periodic=(True,) * 3, jitter=0.1, seed=1)
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    res = {}
    for contraction in ("simt", "tensor"):
        s = Lobatto(m, 3, "rusanov", precision="mixed", contraction=contraction)
        s.SetSolutionColumn(u)
        res[contraction] = s.GetResidualColumn()
        s.close()
    ro = orc.Mesh(m, 3).residual(orc.RUSANOV, u)
    # the SIMT and tensor paths differ by FP32-level rounding of the
    # contraction (TF32x3 is not FP32 FMA bit for bit), which the residual of
    # this near-uniform field magnifies as it does for the SIMT path's own
    # deviation from the oracle: both within the mixed form's 1e-5
    assert rel_l2(res["tensor"], res["simt"]) <= 1e-5, rel_l2(res["tensor"], res["simt"])
    assert rel_l2(res["tensor"], ro) <= 1e-5, rel_l2(res["tensor"], ro)


def test_tensor_contraction_steps(gpu):
    m = cases.vortex_mesh(8)
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    out = {}
    for name, precision, contraction in (("fp64", "fp64", "simt"), ("tensor", "mixed", "tensor")):
        s = Lobatto(m, 3, "rusanov", cfl=0.1, precision=precision, contraction=contraction)
        s.SetSolutionColumn(u)
        s.advance(20, 1e9, 3, 0.0)
        out[name] = s.GetSolutionColumn().reshape(-1, 5)[:, 0]
        s.close()
    assert rel_l2(out["tensor"], out["fp64"]) <= 1e-6, rel_l2(out["tensor"], out["fp64"])


def test_tensor_contraction_rejected_outside_its_scope(gpu):
    m = meshlib.box((2, 2, 2), periodic=(True,) * 3)
    for kw in (dict(degree=2, precision="mixed"), dict(degree=3, precision="fp64"),
               dict(degree=3, precision="mixed", scheme="fr")):
        deg = kw.pop("degree")
        with pytest.raises(capi.McfdError):
            Lobatto(m, deg, "rusanov", contraction="tensor", **kw)
