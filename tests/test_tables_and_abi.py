"""Case tables, the C-ABI library's exports and host-side helpers (CPU only)."""
import ctypes
import os
import re

import numpy as np
import pytest

from binarymeshfitting_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLES = os.path.join(ROOT, "binarymeshfitting_gb300", "csrc", "bmf_case_tables.h")
REF_SRC = os.environ.get("BMF_REFERENCE_SRC") or os.path.normpath(
    os.path.join(ROOT, "..", "reference", "BinaryMeshFitting"))

CORNERS = [(0, 4), (1, 5), (2, 6), (3, 7), (0, 2), (1, 3), (4, 6), (5, 7), (0, 1), (2, 3), (4, 5), (6, 7)]


def _table(name):
    s = open(TABLES).read()
    i = s.index("#define " + name)
    body = s[i:s.index("}", i)]
    return [int(v, 16) for v in re.findall(r"0x([0-9a-f]{16})ULL", body)]


def crossing(mask, e):
    a, b = CORNERS[e]
    return ((mask >> a) & 1) != ((mask >> b) & 1)


def test_triangle_table_uses_only_crossing_edges():
    tri = _table("BMF_TRI_CASES_INIT")
    assert len(tri) == 256
    for m, w in enumerate(tri):
        nt = w >> 60
        edges = [(w >> (4 * i)) & 0xF for i in range(3 * nt)]
        assert all(crossing(m, e) for e in edges), m
        assert (nt == 0) == (m in (0, 255))


def test_group_table_partitions_crossing_edges():
    groups = _table("BMF_GROUP_CASES_INIT")
    for m, w in enumerate(groups):
        ng = (w >> 48) & 0xF
        for e in range(12):
            g = (w >> (4 * e)) & 0xF
            assert (g != 0xF) == crossing(m, e), (m, e)
            assert g == 0xF or g < ng
        assert (ng == 0) == (m in (0, 255))


def test_edge_use_table_matches_triangles():
    tri, uses = _table("BMF_TRI_CASES_INIT"), _table("BMF_EDGE_USES_INIT")
    for m in range(256):
        cnt = [0] * 12
        for i in range(3 * (tri[m] >> 60)):
            cnt[(tri[m] >> (4 * i)) & 0xF] += 1
        assert all(((uses[m] >> (4 * e)) & 0xF) == cnt[e] for e in range(12))


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")
def test_tables_match_reference_headers():
    """Decoded tables equal the reference's MCTable.h tri_table / edge_map and Tables.hpp EdgeTable."""
    mc = open(os.path.join(REF_SRC, "MCTable.h")).read()
    em = [int(v, 16) for v in re.findall(r"0x([0-9A-Fa-f]+)", mc[mc.index("edge_map"):mc.index("tri_table")])]
    for m in range(256):
        assert em[m] == sum(1 << e for e in range(12) if crossing(m, e))
    from binarymeshfitting_gb300.csrc import gen_case_tables as g
    rows = g._rows(mc, "tri_table")[:256]
    assert [g.pack_tri(r) for r in rows] == _table("BMF_TRI_CASES_INIT")
    tb = open(os.path.join(REF_SRC, "Tables.hpp")).read()
    assert [g.pack_groups(r) for r in g._rows(tb, "EdgeTable")] == _table("BMF_GROUP_CASES_INIT")


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    header = open(os.path.join(ROOT, "include", "bmf.h")).read()
    declared = sorted(set(re.findall(r"^\s*BMF_API\s+(?:bmf_status|const char\*|int64_t)\s+(bmf_\w+)\(", header, re.M)))
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) <= set(_lib.SIGNATURES), "ctypes binding misses a declared symbol"
