"""Build recipe of the device-adapter tag's C++ test program (test
infrastructure).

tests/tag/test_tag.cpp includes the DaxToolkit's own control headers
(ArrayHandle, ArrayManagerExecution, Timer, the error classes) and
include/dax_gb300_tag.h, and links libdax_gb300.so.  Where the reference
tree is present it is compiled from there (with oracle/build.py's Boost
stand-ins and configured headers), and a preprocessed copy with the
reference and repository headers expanded is written next to the binary;
where the tree is absent (the GPU host) that copy is compiled instead.  All
outputs go to the git-ignored tests/tag/_build/.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
BIN = os.path.join(OUT, "test_tag")
PP = os.path.join(OUT, "test_tag_pp.cpp")
SRC = os.path.join(HERE, "test_tag.cpp")


def _link_args():
    from daxtoolkit_gb300 import build as gb
    lib = gb.build()
    return ["-L", os.path.dirname(lib), "-ldax_gb300", "-Wl,-rpath," + os.path.dirname(lib)]


def build(force=False):
    """Returns the test program's path, or None if neither the reference tree
    nor an exported source is available."""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import oracle.build as ob
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "host_arch")
    link = _link_args()
    include = os.path.join(ROOT, "include")
    deps = [SRC, os.path.join(include, "dax_gb300_tag.h"), os.path.join(include, "dax_gb300.h")]
    fresh = (os.path.exists(BIN) and os.path.exists(stamp) and
             open(stamp).read().strip() == platform.machine())
    if ob.reference_available():
        if not force and fresh and all(os.path.getmtime(d) <= os.path.getmtime(BIN) for d in deps):
            return BIN
        gen = os.path.join(ob.REF_OUT, "gen")
        ob._configure_headers(gen)
        subprocess.check_call(["g++"] + ob.REF_DEFS + ["-O1", "-I", os.path.join(ob.HERE, "ref_shim"),
                                                       "-I", gen, "-I", ob.REFERENCE_DIR, "-I",
                                                       include, SRC, "-o", BIN] + link)
        ob._export_portable_source(gen, [], (), PP, SRC, (include,))
    elif os.path.exists(PP):
        if not force and fresh and os.path.getmtime(PP) <= os.path.getmtime(BIN):
            return BIN
        subprocess.check_call(["g++", "-std=c++11", "-w", "-O1", "-x", "c++", PP, "-o", BIN] + link)
    else:
        return None
    open(stamp, "w").write(platform.machine())
    return BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
