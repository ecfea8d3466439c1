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


def test_header_is_plain_c_and_links(tmp_path):
    """include/visacd_gpu.h compiles as C99 (no C++ or torch types in the
    signatures) and a C program links against the library by those names."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest
        pytest.skip("gcc not found")
    lib_path = build.build_gpu()
    src = tmp_path / "abi_check.c"
    src.write_text(
        '#include "visacd_gpu.h"\n'
        "#include <stdio.h>\n"
        "int main(void) {\n"
        "  visacd_vis_stats st;\n"
        "  (void)st;\n"
        '  printf("%d %d\\n", visacd_abi_version(), visacd_vis_variant_count());\n'
        "  return visacd_abi_version() == 1 ? 0 : 1;\n"
        "}\n")
    exe = tmp_path / "abi_check"
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
                        str(lib_path), f"-Wl,-rpath,{lib_path.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split()[0] == "1"
