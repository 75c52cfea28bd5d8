"""The C ABI: header/ctypes layout agreement and the exported symbol set (no GPU)."""
import os
import re
import subprocess

import pytest

from kiyosi_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kgpu.h")


def _declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(kgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_exactly_the_ctypes_symbols():
    assert sorted(abi.EXPORTED_SYMBOLS) == _declared_functions()


def test_struct_layouts_match_header(tmp_path):
    names = list(abi.STRUCT_SIZES)
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "kgpu.h"\nint main(void){\n' +
                   "".join(f'printf("{n} %zu\\n", sizeof({n}));\n' for n in names) +
                   "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    sizes = {line.split()[0]: int(line.split()[1]) for line in out.splitlines()}
    assert sizes == abi.STRUCT_SIZES


def test_library_exports_every_declared_symbol():
    from kiyosi_gb300 import build
    lib = build.LIB
    if not os.path.exists(lib):
        build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (kgpu_[a-z0-9_]+)", out))
    assert set(_declared_functions()) <= exported


def test_library_loads_and_reports_abi_version():
    from kiyosi_gb300 import _native
    lib = _native.library()
    assert lib.kgpu_abi_version() == 1
