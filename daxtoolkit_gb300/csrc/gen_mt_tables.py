"""Regenerate ``mt_tables.h``, the packed marching-tetrahedra case table.

The triangle table must match the one the Dax worklet reads
(``dax/worklet/internal/MarchingTetrahedraTable.h:28-53``: ``NumFaces[16]``
and ``TriTable[16][8]``) entry for entry, because triangle order and edge
choice are part of the bit-exact output contract.  This script parses that
header and re-encodes each case as one 32-bit word:

  bits  0..23  six 4-bit edge ids (vertex n of the case in bits 4n..4n+3,
               0xF where unused)
  bits 28..31  number of triangles (0..2)

Usage: python gen_mt_tables.py <path-to-MarchingTetrahedraTable.h> [out.h]
"""
import re
import sys


def parse(path):
    text = open(path).read()
    nf_src = re.search(r"NumFaces\[16\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    tri_src = re.search(r"TriTable\[16\]\[8\]\s*=\s*\{(.*)\};", text, re.S).group(1)
    num_faces = [int(v) for v in re.findall(r"\d+", nf_src)]
    rows = re.findall(r"\{([^{}]*)\}", tri_src)
    tri = [[int(v) for v in re.findall(r"\d+", r)] for r in rows]
    assert len(num_faces) == 16 and len(tri) == 16
    assert all(len(r) == 8 for r in tri)
    return num_faces, tri


def pack(num_faces, tri):
    words = []
    for case in range(16):
        edges = [e for e in tri[case] if e != 255]
        assert len(edges) == 3 * num_faces[case], case
        assert all(0 <= e < 6 for e in edges)
        w = 0
        for n in range(6):
            nib = edges[n] if n < len(edges) else 0xF
            w |= nib << (4 * n)
        w |= num_faces[case] << 28
        words.append(w)
    return words


def emit(words, out):
    lines = [
        "// Generated by gen_mt_tables.py from the Dax marching-tetrahedra case table",
        "// (dax/worklet/internal/MarchingTetrahedraTable.h:28-53). Do not edit.",
        "// Word layout: bits 4n..4n+3 = edge of output vertex n (0xF unused),",
        "// bits 28..31 = triangle count of the case.",
        "#pragma once",
        "#include <stdint.h>",
        "#define DAX_GB300_MT_CASE_WORDS { \\",
    ]
    for i in range(0, 16, 4):
        chunk = ", ".join("0x%08xu" % w for w in words[i:i + 4])
        lines.append("  " + chunk + ("," if i + 4 < 16 else "") + " \\")
    lines.append("}")
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else __file__.replace("gen_mt_tables.py", "mt_tables.h")
    nf, tri = parse(src)
    emit(pack(nf, tri), out)
    print("wrote", out, "sum(NumFaces) =", sum(nf))
