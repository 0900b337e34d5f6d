"""Regenerate ``mc_tables.h``, the packed marching-cubes case table.

The triangle table must match the one the Dax worklet reads
(``dax/worklet/internal/MarchingCubesTable.h:28-306``: ``NumFaces[256]`` and
``TriTable[256][16]``) entry for entry, because triangle order and edge choice
are part of the bit-exact output contract.  This script parses that header and
re-encodes each case as one 64-bit word so a GPU thread fetches a whole case
with a single constant-cache load:

  bits  0..59  fifteen 4-bit edge ids (vertex n of the case in bits 4n..4n+3,
               0xF where unused)
  bits 60..63  number of triangles (0..5)

Usage: python gen_mc_tables.py <path-to-MarchingCubesTable.h> [out.h]
"""
import re
import sys


def parse(path):
    text = open(path).read()
    nf_src = re.search(r"NumFaces\[256\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    tri_src = re.search(r"TriTable\[256\]\[16\]\s*=\s*\{(.*)\};", text, re.S).group(1)
    num_faces = [int(v) for v in re.findall(r"\d+", nf_src)]
    rows = re.findall(r"\{([^{}]*)\}", tri_src)
    tri = [[int(v) for v in re.findall(r"\d+", r)] for r in rows]
    assert len(num_faces) == 256 and len(tri) == 256
    assert all(len(r) == 16 for r in tri)
    return num_faces, tri


def pack(num_faces, tri):
    words = []
    for case in range(256):
        edges = [e for e in tri[case] if e != 255]
        assert len(edges) == 3 * num_faces[case], case
        assert all(0 <= e < 12 for e in edges)
        w = 0
        for n in range(15):
            nib = edges[n] if n < len(edges) else 0xF
            w |= nib << (4 * n)
        w |= num_faces[case] << 60
        words.append(w)
    return words


def emit(words, out):
    lines = [
        "// Generated by gen_mc_tables.py from the Dax marching-cubes case table",
        "// (dax/worklet/internal/MarchingCubesTable.h:28-306). Do not edit.",
        "// Word layout: bits 4n..4n+3 = edge of output vertex n (0xF unused),",
        "// bits 60..63 = triangle count of the case.",
        "#pragma once",
        "#include <stdint.h>",
        "#define DAX_GB300_MC_CASE_WORDS { \\",
    ]
    for i in range(0, 256, 4):
        chunk = ", ".join("0x%016xULL" % w for w in words[i:i + 4])
        lines.append("  " + chunk + ("," if i + 4 < 256 else "") + " \\")
    lines.append("}")
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else __file__.replace("gen_mc_tables.py", "mc_tables.h")
    nf, tri = parse(src)
    emit(pack(nf, tri), out)
    print("wrote", out, "sum(NumFaces) =", sum(nf))
