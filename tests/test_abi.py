"""The C ABI library builds, loads and exports every symbol the header declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

from visacd_gb300 import _native, build

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "visacd_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\**\s+\**([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_lists_expected_entry_points():
    names = declared_functions()
    assert "visacd_visibility" in names and "classify_and_rate_planes" in names
    assert set(names) == set(_native.EXPORTED)


def test_library_exports_every_declared_symbol():
    lib_path = build.build_gpu()
    lib = ctypes.CDLL(str(lib_path))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version_and_error_string_without_gpu():
    lib = _native.lib()
    assert lib.visacd_abi_version() == 1
    assert isinstance(lib.visacd_last_error(), bytes)
