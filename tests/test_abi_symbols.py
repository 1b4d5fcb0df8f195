"""The C-ABI library loads and exports every entry point the header declares.

No compute call is made: this runs without a GPU.
"""
import ctypes
import os
import re
from pathlib import Path

from oracle import oracle
from tealeaf_opencl_gb300 import lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include",
                      "tealeaf_gb300.h")


def declared():
    text = Path(HEADER).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^[a-z][\w *]*?[\s*](\w+)\s*\(", text, flags=re.M)


def test_header_declares_reference_entry_points():
    names = set(declared())
    for sym in lib.REFERENCE_SYMBOLS:
        assert sym in names, sym


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(lib.load().__dict__.get("_name") or lib.library_path())
    names = declared()
    assert len(names) >= len(lib.REFERENCE_SYMBOLS) + len(lib.EXTRA_SYMBOLS)
    for name in names:
        assert hasattr(L, name), name


def test_binding_covers_header():
    assert sorted(declared()) == sorted(lib.REFERENCE_SYMBOLS + lib.EXTRA_SYMBOLS)


def test_reduction_rows_agree_with_oracle():
    L = lib.load()
    for x, y in [(1, 1), (10, 10), (512, 512), (500, 500), (960, 960), (2048, 2048),
                 (3840, 3840), (4096, 4096), (8192, 8192), (4096, 300), (300, 4096)]:
        assert L.tea_gb300_reduction_rows(x, y) == oracle.lib().oracle_reduction_rows(x, y)


def test_errors_are_recorded_not_fatal_without_chunk():
    """Calling an entry point before initialise_ocl_ is an error, not a crash."""
    L = lib.load()
    L.tea_gb300_finalise()
    out = ctypes.c_double(0.0)
    L.tea_leaf_cg_calc_w_kernel_ocl_(ctypes.byref(out))
    code = L.tea_gb300_last_error(None, 0)
    assert code != 0
    assert out.value != out.value  # NaN
