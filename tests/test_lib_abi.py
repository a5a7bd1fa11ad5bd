"""The C-ABI library loads on a host without a GPU and exports every declared symbol."""
import os
import re

from redux_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "rdxg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"^\s*(?:int|int32_t|int64_t|const char\*)\s+(rdxg_\w+)\s*\(", src, flags=re.M))
    return names


def test_header_declares_the_python_table():
    assert declared_functions() == set(_lib.EXPORTED)


def test_library_exports_every_symbol():
    L = _lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.rdxg_version() >= 100
