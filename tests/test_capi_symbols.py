"""The C-ABI library loads on a CPU-only host and exports every entry point
that include/*.h declares (no compute calls: they need a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(mcfd_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("mcfd_create", "mcfd_destroy", "mcfd_set_solution", "mcfd_get_solution",
                     "mcfd_residual", "mcfd_time_step", "mcfd_rk_step", "mcfd_advance",
                     "mcfd_set_bc", "mcfd_set_time", "mcfd_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(mcfd_lib):
    from pvcriemannsolvers_gb300 import capi
    lib = ctypes.CDLL(str(capi.LIB_PATH))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers every declared entry point
    assert set(declared_symbols()) <= set(capi.SIGNATURES)


def test_abi_version_and_create_errors_without_gpu(mcfd_lib):
    """Calls that touch no device memory: version, argument validation."""
    assert mcfd_lib.mcfd_abi_version() == 2
    h = ctypes.c_void_p()
    assert mcfd_lib.mcfd_create(None, None, ctypes.byref(h)) == 1  # MCFD_ERR_ARGUMENT
    assert b"null" in mcfd_lib.mcfd_last_error(None)
