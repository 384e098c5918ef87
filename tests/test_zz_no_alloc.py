"""mcfd_residual_device_noalloc: the residual for callers that cannot
allocate device memory while they run (a program whose memory pool owns the
whole device after start-up, or a time-critical loop that cannot afford the
device synchronisation of cudaMalloc).  Its face-flux scratch is a fixed
16 MiB array inside the library, so it must agree with the ordinary residual
entry point on every call, and reject meshes too large for that array.

This file is collected last on purpose; it passes alone in a fresh process
and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from pvcriemannsolvers_gb300 import Lobatto, capi, cases, mesh as meshlib

pytestmark = pytest.mark.gpu

# the parity tolerances of the residual tests: the FP64 form, and the mixed
# form (FP32 contractions and an FP32 flux store)
RTOL = {"fp64": 1e-12, "mixed": 1e-5}


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("riemann", ["hllc", "rusanov"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("scheme", ["dgsem", "fr"])
def test_noalloc_residual_matches_residual_device_twice(gpu, scheme, precision, riemann):
    """DGSEM and FR (whose face points without a boundary carry the no-flux
    NaN marker through the scratch), FP64 and mixed (FP32 fluxes in the
    scratch), HLLC and Rusanov (whose ordinary stepping path reads node
    traces that the no-allocation path does not use); two calls in a row."""
    import torch
    m = meshlib.box((4, 3, 3), lengths=(1.0, 0.8, 0.6), periodic=(True, False, True), jitter=0.1, seed=3)
    s = Lobatto(m, 3, riemann, scheme=scheme, precision=precision)
    s.SetSmartBoundary(2, cases.SOD_LEFT)
    if scheme == "dgsem":
        s.SetInviscidWall(3)  # FR: group 3 stays without a boundary condition
    x = meshlib.node_coordinates(m, 3).reshape(-1, 3)
    n = s.column_size
    lib = capi.load()
    for call in range(2):
        u = torch.from_numpy(cases.smooth_ic(x + 0.05 * call).ravel()).cuda()
        s.set_solution_device(u.data_ptr(), n)
        ref = torch.empty(n, dtype=torch.float64, device="cuda")
        s.residual_device(ref.data_ptr(), n)
        out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        code = lib.mcfd_residual_device_noalloc(s.handle, C.c_void_p(u.data_ptr()),
                                                C.c_void_p(out.data_ptr()), n)
        capi.check(code, s.handle)
        torch.cuda.synchronize()
        assert torch.cuda.current_device() == 0
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all()
        err = _rel_l2(got, want)
        assert err <= RTOL[precision], (call, err)
    s.close()


def test_noalloc_rejects_meshes_beyond_the_static_capacity(gpu):
    import torch
    # 24^3 periodic, p = 3: 41,472 faces x 16 points = 663,552 > 419,430
    m = meshlib.box((24, 24, 24), periodic=(True, True, True))
    s = Lobatto(m, 3, "rusanov")
    n = s.column_size
    u = torch.zeros(n, dtype=torch.float64, device="cuda")
    r = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib = capi.load()
    code = lib.mcfd_residual_device_noalloc(s.handle, C.c_void_p(u.data_ptr()), C.c_void_p(r.data_ptr()), n)
    assert code == capi.ERR_ARGUMENT
    assert b"static capacity" in lib.mcfd_last_error(s.handle)
    s.close()
