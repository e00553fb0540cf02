"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/orbit_gb300.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "orbit_gb300.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char\*)\s+(orbit_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from orbit_gb300 import build
    path = build.build_library()
    return ctypes.CDLL(path)


def test_header_has_entry_points():
    names = declared()
    assert "orbit_sc2p5d_track" in names and "orbit_program_run" in names
    assert len(names) >= 40


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from orbit_gb300 import _native
    assert sorted(_native.exported_symbols()) == declared()


def test_built_for_sm_103a_only():
    from orbit_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_cpu_fallback_in_product():
    """The product package never imports the oracle."""
    pkg = os.path.join(ROOT, "py-orbit_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
