"""Build recipes for the CPU oracle (test infrastructure only).

Two libraries come out of this:

* ``oracle/build/liboracle.so`` -- the plain-C restatement in ``dax_oracle.c``.
* ``oracle/_ref/libdaxref.so`` -- ``ref_driver.cpp`` compiled against the
  DaxToolkit's own headers (worklets, uniform topology and its point
  coordinates, Lerp), and ``oracle/_ref/libdaxref64.so``, the same driver
  with the reference's ``DAX_USE_DOUBLE_PRECISION`` option (the FP64 twin),
  with
  the five std-based Boost stand-ins in ``ref_shim/`` and the three generated
  headers (``Configure.h`` and the ``VectorOperations.h`` instances) that the
  reference's CMake would normally produce.

The reference tree is read in place (``DAX_REFERENCE_DIR``, else a
``reference`` directory beside the repository); nothing from it is copied into the repository.  Where the
tree is absent the reference library is simply not built and callers fall back
to the C restatement.  Everything compiles with ``-ffp-contract=off`` so that
float expressions round exactly as written (no fused multiply-add), which is
what the reference's Serial adapter does on x86-64.
"""
import os
import re
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")
REF_SO = os.path.join(REF_OUT, "libdaxref.so")


def _reference_dir():
    """The DaxToolkit source tree: ``DAX_REFERENCE_DIR`` when set, else a
    ``reference`` directory beside this repository's root."""
    env = os.environ.get("DAX_REFERENCE_DIR")
    if env:
        return env
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


REFERENCE_DIR = _reference_dir()

CFLAGS = ["-O2", "-ffp-contract=off", "-fPIC", "-shared"]


def _same_arch():
    """False when the build directory holds objects of another host arch."""
    import platform
    stamp = os.path.join(BUILD, "host_arch")
    arch = platform.machine()
    os.makedirs(BUILD, exist_ok=True)
    ok = os.path.exists(stamp) and open(stamp).read().strip() == arch
    open(stamp, "w").write(arch)
    return ok


def _newer(target, sources):
    if not os.path.exists(target) or not _same_arch():
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "dax_oracle.c")
    tables = [os.path.join(HERE, "..", "daxtoolkit_gb300", "csrc", t)
              for t in ("mc_tables.h", "mt_tables.h", "coolwarm_table.h")]
    if force or not _newer(ORACLE_SO, [src] + tables):
        subprocess.check_call(["gcc", "-std=c99"] + CFLAGS + [src, "-o", ORACLE_SO, "-lm"])
    return ORACLE_SO


VTK_BIN = os.path.join(BUILD, "vtk_ostream")


def build_vtk_ostream(force=False):
    """The std::ostream VTK writer (vtk_ostream.cpp), the byte-format pin of
    the library's legacy-VTK writer."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "vtk_ostream.cpp")
    if force or not _newer(VTK_BIN, [src]):
        subprocess.check_call(["g++", "-std=c++11", "-O1", src, "-o", VTK_BIN])
    return VTK_BIN


def _configure_headers(gen):
    """Produce what the reference's CMake would configure (CMakeLists.txt:73,
    dax/CMakeLists.txt:37-46, dax/exec/CMakeLists.txt:38-50,
    dax/cont/CMakeLists.txt:56-68): float Scalar, 32-bit Id."""
    os.makedirs(os.path.join(gen, "dax", "internal"), exist_ok=True)
    os.makedirs(os.path.join(gen, "dax", "exec"), exist_ok=True)
    os.makedirs(os.path.join(gen, "dax", "cont"), exist_ok=True)
    cfg = open(os.path.join(REFERENCE_DIR, "dax", "internal", "Configure.h.in")).read()
    cfg = re.sub(r"^#cmakedefine (\w+)", r"/* #undef \1 */", cfg, flags=re.M)
    for k, v in {"DAX_SIZE_FLOAT": "4", "DAX_SIZE_DOUBLE": "8", "DAX_SIZE_INT": "4",
                 "DAX_SIZE_LONG": "8", "DAX_SIZE_LONG_LONG": "8"}.items():
        cfg = cfg.replace("@%s@" % k, v)
    open(os.path.join(gen, "dax", "internal", "Configure.h"), "w").write(cfg)
    tmpl = open(os.path.join(REFERENCE_DIR, "dax", "internal", "VectorOperations.h.in")).read()
    for ns, name, start, end, export, sub in [
        ("dax", "dax", "namespace dax {", "}", "DAX_EXEC_CONT_EXPORT", "dax"),
        ("dax::exec", "dax_exec", "namespace dax { namespace exec {", "} }", "DAX_EXEC_EXPORT",
         "dax/exec"),
        ("dax::cont", "dax_cont", "namespace dax { namespace cont {", "} }", "DAX_CONT_EXPORT",
         "dax/cont"),
    ]:
        text = (tmpl.replace("@DAX_VECTOR_OPERATIONS_NAMESPACE_NAME@", name)
                .replace("@DAX_VECTOR_OPERATIONS_NAMESPACE_START@", start)
                .replace("@DAX_VECTOR_OPERATIONS_NAMESPACE_END@", end)
                .replace("@DAX_VECTOR_OPERATIONS_EXPORT@", export)
                .replace("@DAX_VECTOR_OPERATIONS_NAMESPACE@", ns))
        open(os.path.join(gen, sub, "VectorOperations.h"), "w").write(text)


def _openmp_ok():
    probe = os.path.join(BUILD, "omp_probe.c")
    os.makedirs(BUILD, exist_ok=True)
    open(probe, "w").write("#include <omp.h>\nint main(void){return omp_get_max_threads()<1;}\n")
    r = subprocess.run(["gcc", "-fopenmp", probe, "-o", probe + ".bin"],
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return r.returncode == 0


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_DIR, "dax", "worklet", "MarchingCubes.h"))


REF_PP = os.path.join(REF_OUT, "ref_driver_pp.cpp")
REF_DEFS = ["-std=c++11", "-w", "-DDAX_USE_VARIADIC_TEMPLATE=1",
            "-DDAX_DEVICE_ADAPTER=DAX_DEVICE_ADAPTER_SERIAL"]
# The FP64 twin: the same driver with the reference's DAX_USE_DOUBLE_PRECISION
# option (dax::Scalar = double) and double outputs, entry points ref64_*.
REF64_SO = os.path.join(REF_OUT, "libdaxref64.so")
REF64_PP = os.path.join(REF_OUT, "ref_driver64_pp.cpp")
VARIANTS = {
    "f32": (REF_SO, REF_PP, []),
    "f64": (REF64_SO, REF64_PP, ["-DDAX_USE_DOUBLE_PRECISION", "-DDAXREF_F64"]),
}


def _system_include_dirs():
    r = subprocess.run(["g++", "-std=c++11", "-x", "c++", "-E", "-v", os.devnull, "-o", os.devnull],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    dirs, on = [], False
    for line in r.stdout.splitlines():
        if line.startswith("#include <...> search starts here"):
            on = True
        elif line.startswith("End of search list"):
            on = False
        elif on:
            dirs.append(os.path.normpath(line.strip()))
    return sorted(dirs, key=len, reverse=True)


def _export_portable_source(gen, omp, defs=(), out_pp=REF_PP, src=None, includes=()):
    """Write oracle/_ref/ref_driver_pp.cpp: ref_driver.cpp with the reference
    headers expanded by the preprocessor and every system header left as an
    #include line, so that the same reference-built driver can be compiled on
    a host without the reference tree (e.g. an aarch64 GPU host).  The file is
    a build output: it lives in the git-ignored oracle/_ref/ only."""
    src = src or os.path.join(HERE, "ref_driver.cpp")
    inc = [x for d in includes for x in ("-I", d)]
    r = subprocess.run(["g++"] + REF_DEFS + list(defs) + omp +
                       ["-E", "-I", os.path.join(HERE, "ref_shim"), "-I", gen, "-I",
                        REFERENCE_DIR] + inc + [src],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, check=True)
    sysdirs = _system_include_dirs()
    marker = re.compile(r'^# (\d+) "([^"]*)"((?: \d)*)$')
    out = ["// Generated by oracle/build.py from %s; not part of the repository."
           % os.path.basename(src),
           "#include <omp.h>" if omp else ""]
    # Stack of (is_system) for the files being read; only markers with flag 1
    # (enter) or 2 (return) change it -- a marker without flags inside a
    # macro expansion (e.g. NULL from <stddef.h>) only moves line numbers.
    stack = [False]
    for line in r.stdout.splitlines():
        m = marker.match(line)
        if m:
            path, flags = m.group(2), m.group(3).split()
            is_sys = "3" in flags
            if "1" in flags:
                if is_sys and not stack[-1]:  # user code includes a system header
                    p = os.path.normpath(path)
                    rel = next((os.path.relpath(p, d) for d in sysdirs
                                if p.startswith(d + os.sep)), None)
                    if rel is None:
                        raise RuntimeError("cannot spell system header " + path)
                    out.append("#include <%s>" % rel)
                stack.append(is_sys or stack[-1])
            elif "2" in flags and len(stack) > 1:
                stack.pop()
            continue
        if not stack[-1]:
            out.append(line)
    open(out_pp, "w").write("\n".join(out) + "\n")


def build_ref(force=False, variant="f32"):
    """Compile the reference-side driver (variant "f32", or "f64" for the
    FP64 twin); returns the .so path or None.

    With the reference tree present: configure, export the portable
    preprocessed source, compile.  Without it: compile the exported source if
    an earlier export travelled here; otherwise None."""
    so, pp, defs = VARIANTS[variant]
    omp = ["-fopenmp"] if _openmp_ok() else []
    import platform
    stamp = os.path.join(REF_OUT, "host_arch_" + variant)
    if not reference_available():
        if os.path.exists(pp):
            fresh = (os.path.exists(so) and os.path.exists(stamp) and
                     open(stamp).read().strip() == platform.machine() and
                     os.path.getmtime(so) >= os.path.getmtime(pp))
            if force or not fresh:
                subprocess.check_call(["g++", "-std=c++11", "-w"] + CFLAGS + omp +
                                      ["-x", "c++", pp, "-o", so])
                open(stamp, "w").write(platform.machine())
            return so
        return None
    src = os.path.join(HERE, "ref_driver.cpp")
    fresh = (os.path.exists(stamp) and open(stamp).read().strip() == platform.machine())
    if not force and fresh and _newer(so, [src]) and os.path.exists(pp):
        return so
    gen = os.path.join(REF_OUT, "gen")
    os.makedirs(REF_OUT, exist_ok=True)
    _configure_headers(gen)
    cmd = (["g++"] + REF_DEFS + defs + CFLAGS + omp +
           ["-I", os.path.join(HERE, "ref_shim"), "-I", gen, "-I", REFERENCE_DIR, src,
            "-o", so])
    subprocess.check_call(cmd)
    _export_portable_source(gen, omp, defs, pp)
    open(stamp, "w").write(platform.machine())
    return so


def clean():
    for d in (BUILD, REF_OUT):
        if os.path.isdir(d):
            shutil.rmtree(d)


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref(force=True, variant="f64"))
