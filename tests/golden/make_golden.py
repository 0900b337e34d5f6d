"""Regenerate the golden fixtures in this directory from the reference-built
oracle (the DaxToolkit's own worklet functors compiled from its source tree,
oracle/ref_driver.cpp).  Run where the reference tree is available:

    python tests/golden/make_golden.py

Small outputs are stored whole; larger ones as SHA-256 of their bytes plus
their sizes.  tests/test_golden_cpu.py checks the C oracle against them, so
the oracle stays pinned on machines without the reference tree.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from tests import cases  # noqa: E402

SMALL = 20000  # bytes; arrays up to this size are stored whole


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def put(store, arrays, key, a):
    a = np.ascontiguousarray(a)
    store[key] = {"shape": list(a.shape), "dtype": str(a.dtype), "sha256": digest(a)}
    if a.nbytes <= SMALL:
        arrays[key] = a


def main():
    R = oracle.Oracle("reference")
    meta, arrays = {}, {}
    for name, dims, origin, spacing, emin, f, iso in cases.mc_cases():
        g = oracle.make_grid(dims, origin, spacing, emin)
        count, cs = R.mc_count(g, f, iso)
        put(meta, arrays, "mc/%s/count" % name, count)
        put(meta, arrays, "mc/%s/cases" % name, cs)
        for merge in (0, 1):
            out = R.mc_generate(g, f, iso, count, bool(merge))
            for k in ("verts", "conn", "rec_a", "rec_b", "rec_w"):
                put(meta, arrays, "mc/%s/m%d/%s" % (name, merge, k), out[k])
    for name, dims, origin, spacing, emin, f, lo, hi in cases.threshold_cases():
        g = oracle.make_grid(dims, origin, spacing, emin)
        count = R.threshold_count(g, f, lo, hi)
        out = R.threshold_generate(g, f, count)
        put(meta, arrays, "thr/%s/count" % name, count)
        for k in ("conn", "coords", "field"):
            put(meta, arrays, "thr/%s/%s" % (name, k), out[k])
    for name, dims, origin, spacing, emin, po, pn in cases.slice_cases():
        g = oracle.make_grid(dims, origin, spacing, emin)
        count = R.slice_count(g, po, pn)
        put(meta, arrays, "slice/%s/count" % name, count)
        for merge in (0, 1):
            out = R.slice_generate(g, po, pn, count, bool(merge))
            for k in ("verts", "conn", "rec_a", "rec_b", "rec_w"):
                put(meta, arrays, "slice/%s/m%d/%s" % (name, merge, k), out[k])
    for name, pts, conn, f, iso in cases.mt_cases():
        count = R.mt_count(conn, f, iso)
        put(meta, arrays, "mt/%s/count" % name, count)
        for merge in (0, 1):
            out = R.mt_generate(pts, conn, f, iso, count, bool(merge))
            for k in ("verts", "conn", "rec_a", "rec_b", "rec_w"):
                put(meta, arrays, "mt/%s/m%d/%s" % (name, merge, k), out[k])
    for name, dims, origin, spacing, emin, f in cases.gradient_cases():
        g = oracle.make_grid(dims, origin, spacing, emin)
        put(meta, arrays, "grad/%s" % name, R.cell_gradient(g, f))
    json.dump(meta, open(os.path.join(HERE, "golden.json"), "w"), indent=0, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"),
                        **{k.replace("/", "__"): v for k, v in arrays.items()})
    print("wrote %d digests, %d whole arrays" % (len(meta), len(arrays)))


if __name__ == "__main__":
    main()
