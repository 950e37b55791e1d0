"""The C-ABI library builds, loads and exports every symbol of include/gbmie.h
(CPU only: no compute calls)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gbmie.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbmie_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding_table():
    from geosmie_gb300 import _native
    assert set(_declared()) == set(_native.SIGNATURES)


def test_library_exports_all_symbols():
    from geosmie_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in _declared() if not hasattr(lib, s)]
    assert not missing, missing


def test_status_strings_without_gpu():
    from geosmie_gb300 import build
    lib = ctypes.CDLL(build.build())
    lib.gbmie_status_string.restype = ctypes.c_char_p
    assert lib.gbmie_status_string(0) == b"ok"
    assert b"invalid" in lib.gbmie_status_string(1)


def test_header_is_plain_c(tmp_path):
    """include/gbmie.h compiles as strict C99 and as C++17 (what a cgo, JNI
    or ctypes binding includes), with no warnings."""
    import shutil
    import subprocess
    import pytest
    src = tmp_path / "use_header.c"
    src.write_text('#include "gbmie.h"\nint main(void) { return 0; }\n')
    inc = os.path.join(ROOT, "include")
    for cc, flags in (("gcc", ["-std=c99", "-pedantic"]), ("g++", ["-std=c++17", "-x", "c++"])):
        if shutil.which(cc) is None:
            pytest.skip("%s not found" % cc)
        r = subprocess.run([cc] + flags + ["-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc, str(src)],
                           capture_output=True, text=True)
        assert r.returncode == 0, (cc, r.stderr)
