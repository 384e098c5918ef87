"""The face kernels' regrouped Riemann fluxes (HLLC's star flux of the
selected side, Roe's upwind form, Rusanov's summed side fluxes) equal the
reference-ordered primitive forms of the same header to 1e-12 row-scaled, on
the host: tests/cpp/flux_forms_host.cu compiled by nvcc as host code, no GPU.
The device instances of the same templates are compared with the oracle by
tests/test_gpu_probe.py."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_regrouped_fluxes_equal_the_primitive_forms(tmp_path):
    from pvcriemannsolvers_gb300 import build
    try:
        nvcc = build.nvcc()
    except RuntimeError as e:
        pytest.skip(str(e))
    exe = tmp_path / "flux_forms_host"
    cmd = [nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}",
           str(ROOT / "tests/cpp/flux_forms_host.cu"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
