"""The C ABI library loads and exports every entry point include/*.h declares.

No compute calls: this runs on machines without a GPU.
"""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:gbpoly_status|const char\*)\s+(gbpoly_\w+)\s*\(", text, flags=re.M))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "gbpoly_gemm_f32" in names and "gbpoly_init" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    import gbpoly

    if not gbpoly.LIB_PATH.exists():
        pytest.skip("libgbpoly.so not built (run __graft_entry__.build())")
    lib = gbpoly.load_library()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    import gbpoly

    assert set(gbpoly.SIGNATURES) == declared_symbols()


def test_last_error_is_empty_string_initially():
    import gbpoly

    if not gbpoly.LIB_PATH.exists():
        pytest.skip("libgbpoly.so not built")
    lib = gbpoly.load_library()
    assert isinstance(lib.gbpoly_last_error(), bytes)
