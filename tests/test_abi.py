"""The C-ABI library loads and exports every entry point include/nbpg.h declares (no GPU calls)."""
import os

import pytest


def test_library_exports_header_symbols():
    from nbpg_gb300 import _lib, build_ext
    if not os.path.exists(_lib.LIB_PATH):
        build_ext.build()
    L = _lib.lib()
    names = _lib.exported_symbols()
    assert "nbpg_search" in names and "nbpg_gt" in names and "nbpg_build" in names
    for n in names:
        assert hasattr(L, n), n
    assert L.nbpg_version().startswith(b"nbpg_gb300")


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    from nbpg_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(_lib.NbpgError):
        _lib.lib()
