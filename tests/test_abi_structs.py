"""The ctypes mirrors of the C ABI's structs (graphbrew_gb300/__init__.py)
declare the same fields, in the same order and with the same types, as
include/gbgpu.h."""
import ctypes as C
import os
import re

import graphbrew_gb300 as gb

HEADER = os.path.join(os.path.dirname(__file__), "..", "include", "gbgpu.h")
CTYPES = {"double": C.c_double, "int32_t": C.c_int32, "int64_t": C.c_int64}


def _header_fields(name):
    text = open(HEADER).read()
    end = re.search(r"\}\s*" + name + ";", text)
    assert end, name
    start = text.rindex("typedef struct {", 0, end.start()) + len("typedef struct {")
    body = re.sub(r"/\*.*?\*/|//[^\n]*", "", text[start:end.start()], flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, field = decl.split()
        fields.append((field, typ))
    return fields


def test_stats_struct_matches_header():
    want = _header_fields("gbgpu_stats")
    got = gb.GbgpuStats._fields_
    assert [f for f, _ in got] == [f for f, _ in want]
    for (f, t), (_, ct) in zip(want, got):
        assert CTYPES[t] is ct, f
