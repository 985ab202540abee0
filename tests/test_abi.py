"""The C ABI library loads without a GPU and exports every function include/pf2.h declares."""
import ctypes
import os
import re
import subprocess

import pytest

import gpupfem2_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pf2.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pf2_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    lib = g.lib()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version():
    assert g.lib().pf2_abi_version() == 1


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_compiles_standalone(lang, tmp_path):
    src = os.path.join(tmp_path, "t." + ("c" if lang == "c" else "cpp"))
    with open(src, "w") as f:
        f.write('#include "pf2.h"\nint main(void){ pf2_params p; (void)p; return 0; }\n')
    cc = "gcc" if lang == "c" else "g++"
    r = subprocess.run([cc, "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_status_strings_without_gpu():
    lib = g.lib()
    lib.pf2_status_string.restype = ctypes.c_char_p
    assert lib.pf2_status_string(1) == b"solver did not converge"
