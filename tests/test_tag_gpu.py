"""The device-adapter tag through its C++ test program (tests/tag/test_tag.cpp),
which uses the DaxToolkit's own ArrayHandle, ArrayManagerExecution and Timer
on include/dax_gb300_tag.h:
* `conformance`: the restated TestingDeviceAdapter.h checks must all pass;
* `cases`: marching cubes (merged and not), threshold and CellGradient of
  the parity cases through the tag's ArrayHandles must reproduce the golden
  digests of the reference (tests/golden/golden.json) and, NaN payloads
  aside, the reference-built driver's arrays."""
import hashlib
import json
import os
import struct
import subprocess

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


@pytest.fixture(scope="module")
def program(gb300):
    from tests.tag import build
    path = build.build()
    if path is None:
        pytest.skip("neither the DaxToolkit tree nor an exported test_tag source is present")
    return path


def test_tag_conformance(program):
    r = subprocess.run([program, "conformance"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and "PASSED 0 failures" in r.stdout, r.stdout


def _write_case(d, name, dims, origin, spacing, emin, f, iso, lo, hi):
    with open(os.path.join(d, name + ".in"), "wb") as out:
        out.write(struct.pack("<6f", *origin, *spacing))
        out.write(struct.pack("<6i", *emin, *[emin[a] + dims[a] - 1 for a in range(3)]))
        out.write(struct.pack("<3f", iso, lo, hi))
        out.write(struct.pack("<q", f.size))
        out.write(np.ascontiguousarray(f, np.float32).tobytes())


def _bits(a):
    a = np.ascontiguousarray(a)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def _check(path, key, ref, dtype, checked):
    got = np.fromfile(path, dtype=dtype)
    ref = np.ascontiguousarray(ref)
    assert got.size == ref.size, key
    if dtype == np.float32:
        assert np.array_equal(_bits(got), _bits(ref.ravel())), key
    else:
        assert np.array_equal(got, ref.ravel()), key
    g = GOLDEN.get(key)
    if g is not None and not (dtype == np.float32 and np.isnan(ref).any()):
        assert hashlib.sha256(got.tobytes()).hexdigest() == g["sha256"], key
        checked.append(key)


def test_tag_cases_against_golden(program, oracle_best, tmp_path):
    import oracle
    items = []
    for name, dims, origin, spacing, emin, f, iso in cases.mc_cases():
        items.append(("mc", name, dims, origin, spacing, emin, f, iso, 0.0, 0.0))
    for name, dims, origin, spacing, emin, f, lo, hi in cases.threshold_cases():
        items.append(("thr", name, dims, origin, spacing, emin, f, 0.0, lo, hi))
    for name, dims, origin, spacing, emin, f in cases.gradient_cases():
        items.append(("grad", name, dims, origin, spacing, emin, f, 0.0, 0.0, 0.0))
    names = []
    for n, (kind, name, dims, origin, spacing, emin, f, iso, lo, hi) in enumerate(items):
        tag = "%s_%d" % (kind, n)
        names.append(tag)
        _write_case(str(tmp_path), tag, dims, origin, spacing, emin, f, iso, lo, hi)
    open(os.path.join(str(tmp_path), "cases.txt"), "w").write("\n".join(names) + "\n")
    r = subprocess.run([program, "cases", str(tmp_path)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    checked = []
    for tag, (kind, name, dims, origin, spacing, emin, f, iso, lo, hi) in zip(names, items):
        p = os.path.join(str(tmp_path), tag)
        og = oracle.make_grid(dims, origin, spacing, emin)
        if kind == "mc":
            count, _ = oracle_best.mc_count(og, f, iso)
            for merge in (0, 1):
                ref = oracle_best.mc_generate(og, f, iso, count, bool(merge))
                _check(p + ".mc%d.conn.bin" % merge, "mc/%s/m%d/conn" % (name, merge), ref["conn"],
                       np.int32, checked)
                _check(p + ".mc%d.verts.bin" % merge, "mc/%s/m%d/verts" % (name, merge),
                       ref["verts"], np.float32, checked)
        elif kind == "thr":
            ref = oracle_best.threshold_generate(og, f, oracle_best.threshold_count(og, f, lo, hi))
            for k, dt in (("conn", np.int32), ("coords", np.float32), ("field", np.float32)):
                _check(p + ".thr.%s.bin" % k, "thr/%s/%s" % (name, k), ref[k], dt, checked)
        else:
            _check(p + ".grad.bin", "grad/%s" % name, oracle_best.cell_gradient(og, f), np.float32,
                   checked)
    # most outputs are pinned by the golden digests as well
    assert len(checked) >= 20, checked
