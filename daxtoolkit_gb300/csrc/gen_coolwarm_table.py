"""Regenerate ``coolwarm_table.h``, the cool-warm colour map of the Mandelbulb
surface colouring.

``ColorsAndNorms`` (``Benchmarks/Mandlebulb/Worklets.h:177-209``) colours
every output point with entry ``(int)(257 * s)`` of the 257-entry RGB table in
``Benchmarks/Mandlebulb/CoolWarmColorMap.h:53-311``; the colours are part of
the output, so the table must match entry for entry.  This script parses that
header and writes the table as one flat byte list (r, g, b per entry).

Usage: python gen_coolwarm_table.py <path-to-CoolWarmColorMap.h> [out.h]
"""
import re
import sys


def parse(path):
    text = open(path).read()
    body = re.search(r"coolWarmTable\[NUM_COLORS\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    rows = re.findall(r"ColorType\(\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*\)", body)
    table = [tuple(int(v) for v in r) for r in rows]
    assert len(table) == 257 and all(0 <= v <= 255 for r in table for v in r)
    return table


def emit(table, out):
    lines = [
        "// Generated by gen_coolwarm_table.py from the Mandelbulb benchmark's cool-warm",
        "// colour map (Benchmarks/Mandlebulb/CoolWarmColorMap.h:53-311). Do not edit.",
        "// 257 entries of r, g, b.",
        "#pragma once",
        "#define DAX_GB300_COOLWARM_ENTRIES 257",
        "#define DAX_GB300_COOLWARM_RGB { \\",
    ]
    flat = [v for r in table for v in r]
    for i in range(0, len(flat), 24):
        chunk = ", ".join("%d" % v for v in flat[i:i + 24])
        lines.append("  " + chunk + ("," if i + 24 < len(flat) else "") + " \\")
    lines.append("}")
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else __file__.replace("gen_coolwarm_table.py",
                                                                 "coolwarm_table.h")
    emit(parse(src), out)
    print("wrote", out)
