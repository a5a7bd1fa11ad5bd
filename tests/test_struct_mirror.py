"""The ctypes mirrors of the C ABI's structs (redux_gb300/_lib.py) match include/rdxg.h field by
field: the same names, order and types, so that every field reaches the library where the
header puts it (CPU only)."""
import ctypes as C
import os
import re

import pytest

from redux_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "rdxg_geometry": _lib.Geometry,
    "rdxg_static": _lib.Static,
    "rdxg_solve_params": _lib.SolveParams,
    "rdxg_patch_report": _lib.PatchReport,
    "rdxg_patch_shape": _lib.PatchShape,
    "rdxg_launch_shape": _lib.LaunchShape,
    "rdxg_mode_params": _lib.ModeParams,
}

SCALARS = {"int32_t": C.c_int32, "int64_t": C.c_int64, "double": C.c_double}


def header_structs():
    src = open(os.path.join(ROOT, "include", "rdxg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.fullmatch(r"(?:const\s+)?(\w+)\s*(\*?)\s*(\w+)", decl)
            assert m, (name, decl)
            base, ptr, field = m.groups()
            fields.append((field, C.c_void_p if ptr else SCALARS[base]))
        out[name] = fields
    return out


def test_every_header_struct_has_a_mirror():
    assert set(header_structs()) == set(MIRRORS)


@pytest.mark.parametrize("name", sorted(MIRRORS))
def test_mirror_matches_the_header(name):
    want = header_structs()[name]
    got = [(f, t) for f, t in MIRRORS[name]._fields_]
    assert [f for f, _ in got] == [f for f, _ in want]
    for (f, t), (_, tw) in zip(got, want):
        assert t is tw, (name, f, t, tw)
