"""The C-ABI library builds, loads without a GPU, and exports every function the
public headers declare (no compute call is made here)."""
import ctypes as C
import os
import re

import pytest

from simulation_project_gb300 import build, lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h") or h == "mps_types.h":
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, re.M):
            name = m.group(1)
            if name in ("if", "defined", "extern"):
                continue
            names.append(name)
    return sorted(set(names))


@pytest.fixture(scope="module")
def so():
    path = build.build()
    return C.CDLL(path)


def test_every_declared_function_is_exported(so):
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_binding_signatures_cover_exports(so):
    for name in lib.exported_symbols():
        assert hasattr(so, name), name


def test_library_is_built_for_sm103a():
    path = build.build()
    blob = open(path, "rb").read()
    assert b"sm_103a" in blob
