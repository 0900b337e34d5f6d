"""Compile the sm_103a kernels and the C ABI into an in-tree shared library.

``python -m daxtoolkit_gb300.build`` (or ``build()``) produces
``daxtoolkit_gb300/lib/libdax_gb300.so``.  Each ``.cu`` file is compiled in
parallel for exactly one target, ``-gencode arch=compute_103a,code=sm_103a``,
then linked with the CUDA runtime linked statically, so the library depends on
nothing but the driver.  No fast-math: the kernels spell out every rounding
(``__fmul_rn``/``__fadd_rn``/``__fdiv_rn``) to match the reference's float
arithmetic bit for bit.
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libdax_gb300.so")

SOURCES = ["classify.cu", "mc.cu", "pipeline.cu", "threshold.cu", "gradient.cu", "adjoint.cu", "capi.cu",
           "noalloc.cu", "memory.cu", "fused.cu", "staged.cu", "primitives.cu", "slice.cu", "mt.cu",
           "mandelbulb.cu", "fields.cu", "vtk.cu", "selftest.cu"]
HEADERS = ["common.cuh", "kernels.cuh", "mc_case.cuh", "mc_tables.h", "mt_tables.h",
           "coolwarm_table.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]


def nvcc():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(home, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    # objects and libraries built on another host architecture are stale
    stamp = os.path.join(OBJDIR, "host_arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        force = True
        open(stamp, "w").write(arch)
    include = os.path.join(HERE, "..", "include")
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(include, "dax_gb300.h")]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-I", include, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stdout.write(r.stdout)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            sys.stdout.write(r.stdout)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
