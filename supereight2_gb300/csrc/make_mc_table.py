"""Writes mc_case_table.inc: the marching-cubes case table of supereight2
(include/se/map/algorithms/edge_tables.hpp, triTable) in this library's encoding. It is a
constant table of the standard algorithm, kept identical to the reference's so that meshes match
face for face. Not run by the build; regenerate with

    python supereight2_gb300/csrc/make_mc_table.py path/to/supereight2
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read_table(src):
    txt = open(os.path.join(src, "include/se/map/algorithms/edge_tables.hpp")).read()
    body = txt[txt.index("triTable[256][16]"):]
    body = body[body.index("{") + 1:]
    rows = re.findall(r"\{([-\d,\s]+)\}", body)[:256]
    table = [[int(v) for v in r.split(",") if v.strip()] for r in rows]
    assert len(table) == 256 and all(len(r) == 16 for r in table)
    return table


def encode(row):
    edges = [e for e in row if e >= 0]
    assert len(edges) % 3 == 0 and len(edges) <= 15 and all(0 <= e < 12 for e in edges)
    word = (len(edges) // 3) << 60
    for i, e in enumerate(edges):
        word |= e << (4 * i)
    return word


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_mc_table.py <supereight2 source tree>")
    words = [encode(r) for r in read_table(sys.argv[1])]
    lines = ["// Generated by make_mc_table.py: the marching-cubes case table of supereight2",
             "// (include/se/map/algorithms/edge_tables.hpp, triTable), one word per case: the number of",
             "// faces in bits 60..63 and the cube edges of the faces in the table's order, 4 bits each",
             "// (face f, vertex v at bits 12 f + 4 v). Edges and corners as meshing::edge_to_corners.",
             "static const unsigned long long kMcCaseWords[256] = {"]
    for i in range(0, 256, 4):
        lines.append("    " + ", ".join(f"0x{w:016x}ull" for w in words[i:i + 4]) + ",")
    lines.append("};")
    with open(os.path.join(HERE, "mc_case_table.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
