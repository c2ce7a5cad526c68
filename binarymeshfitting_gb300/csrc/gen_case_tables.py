"""Regenerates bmf_case_tables.h from the reference's case tables.

Bit-exact triangle order (Mode R) needs the very same per-case triangle lists
as the reference (BinaryMeshFitting/MCTable.h:25-282, ``MarchingCubes::tri_table``),
and the DMC vertex groups (Mode Q) come from BinaryMeshFitting/Tables.hpp:96-354
(``Tables::EdgeTable``).  This script parses those two tables as data and writes
them in this project's own packed encoding:

* ``kBmfTriCases[mask]``: bits 4*i..4*i+3 hold the i-th edge id of the case's
  triangle list (i < 15), bits 60..63 the number of triangles (0..5).
* ``kBmfGroupCases[mask]``: bits 4*e..4*e+3 hold the vertex group of grid edge
  e (0..11) in this case, 0xF when the edge is not crossed; bits 48..51 hold
  the number of groups.  Groups are numbered in the table's listing order.
* ``kBmfEdgeUses[mask]`` (derived): bits 4*e..4*e+3 count how often edge e
  occurs in the case's triangle list, i.e. the reference's per-cell
  contribution to ``DualVertex::init_valence`` (DMCChunk.cpp:573).

Each table is also emitted as an initializer macro (``BMF_TRI_CASES_INIT`` ...)
so CUDA ``__constant__`` arrays can be statically initialised from it.

Run it where the reference sources are present:
    python binarymeshfitting_gb300/csrc/gen_case_tables.py <path to BinaryMeshFitting>
"""
import os
import re
import sys


def _rows(text, name):
    start = text.index(name)
    body = text[text.index("{", start) + 1:]
    rows = re.findall(r"\{([^{}]*)\}", body[: body.index("};")])
    return [[int(v) for v in r.replace("\n", " ").split(",") if v.strip()] for r in rows]


def pack_tri(row):
    edges = []
    for v in row:
        if v == -1:
            break
        edges.append(v)
    assert len(edges) % 3 == 0 and len(edges) <= 15
    word = 0
    for i, e in enumerate(edges):
        word |= (e & 0xF) << (4 * i)
    return word | ((len(edges) // 3) << 60)


def pack_groups(row):
    group_of = [0xF] * 12
    g = 0
    n_groups = 0
    for v in row:
        if v == -2:
            break
        if v == -1:
            g += 1
            continue
        assert group_of[v] == 0xF
        group_of[v] = g
        n_groups = g + 1
    word = 0
    for e in range(12):
        word |= group_of[e] << (4 * e)
    return word | (n_groups << 48)


def edge_uses(tri_word):
    counts = [0] * 12
    for i in range(3 * (tri_word >> 60)):
        counts[(tri_word >> (4 * i)) & 0xF] += 1
    assert max(counts) < 16
    word = 0
    for e in range(12):
        word |= counts[e] << (4 * e)
    return word


def main(src):
    mc = open(os.path.join(src, "MCTable.h")).read()
    tb = open(os.path.join(src, "Tables.hpp")).read()
    tri = _rows(mc, "tri_table")
    groups = _rows(tb, "EdgeTable")
    assert len(tri) >= 256 and len(groups) == 256
    tri = tri[:256]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bmf_case_tables.h")
    with open(out, "w") as f:
        f.write("// Generated by gen_case_tables.py from the reference's MCTable.h (tri_table)\n")
        f.write("// and Tables.hpp (EdgeTable); encoding described in that script.\n")
        f.write("// Cell case = 8-bit corner mask, bit (4*dx + 2*dy + dz) set when corner\n")
        f.write("// (x+dx, y+dy, z+dz) is inside.  Edge ids: 0-3 x-edges at (dy,dz) =\n")
        f.write("// (0,0),(0,1),(1,0),(1,1); 4-7 y-edges at (dx,dz); 8-11 z-edges at (dx,dy).\n")
        f.write("#pragma once\n#include <stdint.h>\n\n")
        tri_words = [pack_tri(r) for r in tri]
        for name, macro, words in (("kBmfTriCases", "BMF_TRI_CASES_INIT", tri_words),
                                   ("kBmfGroupCases", "BMF_GROUP_CASES_INIT", [pack_groups(r) for r in groups]),
                                   ("kBmfEdgeUses", "BMF_EDGE_USES_INIT", [edge_uses(w) for w in tri_words])):
            f.write("#define %s { \\\n" % macro)
            for i in range(0, 256, 4):
                f.write("  " + ", ".join("0x%016xULL" % w for w in words[i:i + 4]) + ", \\\n")
            f.write("}\n")
            f.write("static const uint64_t %s[256] = %s;\n\n" % (name, macro))
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "BinaryMeshFitting")
