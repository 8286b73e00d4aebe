"""The C-ABI library loads and exports every entry point include/tristan_gpu.h
declares (no GPU needed); the host config structure matches the header."""
import ctypes
import os
import re

import pytest

from tristan_gb300 import gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tristan_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(tg_\w+)\s*\(", text, re.M)))


def test_header_lists_entry_points():
    names = declared_functions()
    assert "tg_init" in names and "tg_step" in names and len(names) >= 20
    assert set(names) == set(gpu.ENTRY_POINTS)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(gpu.LIB_PATH):
        pytest.skip("library not built")
    lib = ctypes.CDLL(gpu.LIB_PATH)
    for n in declared_functions():
        assert hasattr(lib, n), n


def test_config_struct_layout():
    # offsets the C compiler gives tg_config (x86_64 and aarch64 agree)
    c = gpu.tg_config
    assert c.x1in.offset % 8 == 0
    assert c.maxhlf.offset % 8 == 0
    assert ctypes.sizeof(c) == 216  # includes diag_every (fits the tail padding)


def test_no_cpu_fallback_without_library(tmp_path):
    with pytest.raises(RuntimeError):
        gpu._lib = None
        gpu.load_library(str(tmp_path / "missing.so"))
