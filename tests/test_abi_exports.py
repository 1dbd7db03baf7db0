"""The C-ABI library loads and exports every function include/amx.h declares (no GPU needed)."""
import ctypes
import os
import re

from astronomix_gb300 import _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "amx.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(amx_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "amx_plan_create" in names and "amx_run" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(amx_lib):
    lib = ctypes.CDLL(_native.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(amx_lib):
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_version_string(amx_lib):
    assert amx_lib.amx_version().startswith(b"amx ")


def test_struct_layout_matches_c_compiler(tmp_path):
    """ctypes mirrors of the structs have the C compiler's size and field offsets."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    checks = []
    for struct, cls in (("amx_config", _native.amx_config), ("amx_params", _native.amx_params),
                        ("amx_run_info", _native.amx_run_info)):
        checks.append('printf("%s %%zu\\n", sizeof(%s));' % (struct, struct))
        for fname, _ in cls._fields_:
            checks.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (struct, fname, struct, fname))
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "amx.h"\nint main(void){%s return 0;}\n'
                   % "".join(checks))
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for struct, cls in (("amx_config", _native.amx_config), ("amx_params", _native.amx_params),
                        ("amx_run_info", _native.amx_run_info)):
        assert int(out[struct]) == ctypes.sizeof(cls), struct
        for fname, _ in cls._fields_:
            assert int(out["%s.%s" % (struct, fname)]) == getattr(cls, fname).offset, (struct, fname)
