"""The reference-side C++ binding (include/mcfd_system.hpp): a System with
the reference's four virtuals, driven by an SSP-RK3 loop that makes the
reference's call sequence, agrees with the fused device update."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def build_dropin(tmp_path):
    from pvcriemannsolvers_gb300 import build, capi
    build.build()
    exe = tmp_path / "dropin_rk3"
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/dropin_rk3.cpp"),
           "-o", str(exe), f"-L{capi.LIB_PATH.parent}", "-lmcfd", f"-Wl,-rpath,{capi.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_dropin_compiles(tmp_path):
    assert build_dropin(tmp_path).exists()


@pytest.mark.gpu
def test_dropin_runs(gpu, tmp_path):
    exe = build_dropin(tmp_path)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(res.stdout, res.stderr)
    assert res.returncode == 0, res.stdout + res.stderr
