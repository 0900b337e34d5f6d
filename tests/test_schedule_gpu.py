"""The header-only parts of the device adapter, for arbitrary functors and
types: dax_gb300::Schedule (include/dax_gb300_schedule.cuh; the reference's
TestAlgorithmSchedule and TestErrorExecution, TestingDeviceAdapter.h:382-466,
:1003-1036, in tests/schedule/test_schedule.cu; TestDispatcher and the map-field / map-cell
worklets with their errors, :468-560 and :1038-1200, in
tests/schedule/test_dispatch.cu) and the generic algorithms with comparison
objects (include/dax_gb300_algorithm.cuh; tests/schedule/test_algorithm.cu).  Each program is built with nvcc against
the library and run."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROGRAMS = {"test_schedule": 8, "test_algorithm": 14, "test_dispatch": 8}  # program -> checks


def _nvcc(name, out, link=True):
    src = os.path.join(ROOT, "tests", "schedule", name + ".cu")
    lib = os.path.join(ROOT, "daxtoolkit_gb300", "lib")
    cmd = ["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), src, "-o", out]
    if link:
        cmd += ["-L", lib, "-ldax_gb300", "-Xlinker", "-rpath=" + lib]
    else:
        cmd += ["-c"]
    return subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=600)


@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_header_compiles(tmp_path, name):
    """The headers and their test programs compile for sm_103a (no GPU needed)."""
    r = _nvcc(name, str(tmp_path / (name + ".o")), link=False)
    assert r.returncode == 0, r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_header_program_on_gpu(gb300, tmp_path, name):
    exe = str(tmp_path / name)
    r = _nvcc(name, exe)
    assert r.returncode == 0, r.stdout
    run = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stdout
    assert "0 failures" in run.stdout and run.stdout.count("PASS") == PROGRAMS[name], run.stdout
