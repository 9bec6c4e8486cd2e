"""The C-ABI library loads and exports every entry point the header declares (no
compute calls: this runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT
from kmos_gb300 import build, engine


def declared_functions():
    text = open(os.path.join(ROOT, "include", "kmc_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kmc_\w+)\s*\(", text)))


def test_library_builds_and_exports_header():
    lib = ctypes.CDLL(build.build())
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_functions()) == set(engine.SIGNATURES)


def test_version_string():
    assert b"sm_103a" in engine.load().kmc_version()
