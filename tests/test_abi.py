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


def test_workspace_query_is_host_logic():
    # gbpoly_workspace_query needs no context or device: the split panels of
    # the tensor-core forms, and the K-split partials of small FP32 grids
    import ctypes as ct

    import gbpoly
    from gbpoly import Precision

    if not gbpoly.LIB_PATH.exists():
        pytest.skip("libgbpoly.so not built")
    lib = gbpoly.load_library()

    def query(prec, M, N, K, same=0):
        out = ct.c_size_t()
        assert lib.gbpoly_workspace_query(int(prec), M, N, K, same, ct.byref(out)) == 0
        return out.value

    # bf16x3: two BF16 terms of A and B, K rounded up to 64
    assert query(Precision.BF16X3, 1000, 500, 100) >= 2 * (1000 + 500) * 128 * 2
    assert query(Precision.BF16X3, 1000, 1000, 100, same=1) < query(Precision.BF16X3, 1000, 1000, 100)
    # CTA-pair shapes: the panels plus the partial sums of a K-split last round
    # (up to 64 tiles of 256 x 256 FP32)
    assert query(Precision.BF16X3, 8192, 8192, 8192) >= 2 * 2 * 8192 * 8192 * 2 + 64 * 256 * 256 * 4
    # fp32: nothing for grids that fill a device, partial products for small ones
    assert query(Precision.FP32, 8192, 8192, 8192) == 0
    small = query(Precision.FP32, 1024, 1024, 1024)
    assert small > 0 and small % (1024 * 1024 * 4) == 0
    assert query(Precision.FP32, 1024, 1024, 16) == 0  # too little K to split
    assert lib.gbpoly_workspace_query(int(Precision.FP32), -1, 4, 4, 0, ct.byref(ct.c_size_t())) != 0


def test_null_context_is_an_error_not_a_crash():
    # entry points check their context before any CUDA call: on a machine
    # without a GPU they return GBPOLY_ERR_INVALID with a message
    import ctypes as ct

    import gbpoly
    from gbpoly import Precision

    if not gbpoly.LIB_PATH.exists():
        pytest.skip("libgbpoly.so not built")
    lib = gbpoly.load_library()
    invalid = 1  # GBPOLY_ERR_INVALID
    assert lib.gbpoly_covariance_f32(None, int(Precision.BF16X3), 4, 4, None, 4, None, None, 1.0, None, 4) == invalid
    assert b"context" in lib.gbpoly_last_error()
    assert lib.gbpoly_center_columns_f32(None, 4, 4, None, 4, None, None, 1.0, None, 4) == invalid
    assert lib.gbpoly_tail_split_enable(None, 1) == invalid
    assert lib.gbpoly_profile_enable(None, 1) == invalid
