"""The C ABI library loads and exports every symbol include/flowmc.h declares
(CPU only: no compute call is made)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    out = set()
    for h in (ROOT / "include").glob("*.h"):
        out |= set(re.findall(r"^FMC_API\s+[\w\s\*]+?\b(fmc_\w+)\s*\(", h.read_text(), flags=re.M))
    return out


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "fmc_local_steps" in syms and "fmc_last_error" in syms


def test_library_exports_every_declared_symbol():
    from flowmc_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        pytest.skip("libflowmc.so not built")
    h = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in sorted(declared_symbols()) if not hasattr(h, s)]
    assert not missing, missing


def test_python_binding_covers_declared_symbols():
    import flowmc_gb300.api  # noqa: F401  (registers every entry point)
    from flowmc_gb300 import _lib
    assert declared_symbols() <= set(_lib.EXPORTED)


def test_version_without_gpu():
    from flowmc_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        pytest.skip("libflowmc.so not built")
    assert _lib.lib().fmc_version() == 3
