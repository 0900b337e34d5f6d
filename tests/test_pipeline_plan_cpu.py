"""Slab plan of dax_gb300_mc_pipeline, checked on the host for many grid
shapes and slab counts: before any pass of slab s reads a bit, a word offset
or an active-word entry, the passes it is ordered after must have written it.

What the kernels read (csrc/mc.cu):
* count of row word (r, m): the bit rows r, r + 1, r + ny, r + ny + 1, five
  words from word (r nx + 32 m) >> 5 each;
* emit of active row word (r, m): the bit rows up to r + 2 ny + 1 (owner rows
  of the cells' far corners and the next word's owner points), two words
  past 32 (m + 1); the offsets of row words up to (r + ny + 1, m + 1); the
  offsets at the slab's end word for its capacity check.
Order: classification of slabs 0..s, then count + scan of slab s, then the
emit of slab s."""
import ctypes

import pytest

from daxtoolkit_gb300 import build, capi

TILE = 4096
NS = 17


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.lib()


def _plan(lib, dims, slabs):
    g = capi.UniformGridDesc()
    for a in range(3):
        g.spacing[a] = 1.0
        g.extent_max[a] = dims[a] - 1
    out = (ctypes.c_int64 * (1 + 3 * NS))()
    capi.call("dax_gb300_mc_pipeline_plan", ctypes.byref(g), slabs, out)
    S = out[0]
    W = list(out[1:1 + S + 1])
    E = list(out[1 + NS:1 + NS + S + 1])
    K = list(out[1 + 2 * NS:1 + 2 * NS + S + 1])
    return S, W, E, K


SHAPES = [(2, 2, 2), (3, 2, 2), (33, 5, 4), (64, 64, 64), (37, 29, 23), (100, 3, 500),
          (512, 512, 512), (257, 129, 65), (31, 400, 9), (1, 1, 1), (8192, 2, 3),
          (600, 600, 40), (96, 80, 70), (129, 65, 1000), (5, 7, 20000), (1290, 1290, 1290)]


@pytest.mark.parametrize("dims", SHAPES, ids=lambda d: "x".join(map(str, d)))
@pytest.mark.parametrize("slabs", [1, 2, 3, 8, 16])
def test_plan_orders_every_read_after_its_write(lib, dims, slabs):
    nx, ny, nz = dims
    wr = (nx + 31) // 32
    rowwords = ny * nz * wr
    P = nx * ny * nz
    chunks = (P + 127) // 128
    S, W, E, K = _plan(lib, dims, slabs)
    assert 1 <= S <= max(1, slabs)
    # count/scan ranges: tile-aligned, increasing, covering every row word
    assert W[0] == 0 and W[S] == rowwords
    assert all(W[s] < W[s + 1] for s in range(S)) or rowwords == 0
    assert all(W[s] % TILE == 0 for s in range(S))
    # emit ranges: increasing, covering every row word, each at or before
    # its count range's start
    assert E[0] == 0 and E[S] == rowwords
    assert all(E[s] < E[s + 1] for s in range(S)) or rowwords == 0
    assert all(0 <= E[s] <= W[s] for s in range(S))
    # classification ranges: increasing, covering every chunk
    assert K[0] == 0 and K[S] == chunks
    assert all(K[s] <= K[s + 1] for s in range(S))
    for s in range(S):
        classified = K[s + 1] * 128 if K[s + 1] < chunks else None  # None: everything
        # count of slab s: last row of the slab, plus one plane and one row
        if W[s + 1] > W[s]:
            r = (W[s + 1] - 1) // wr
            max_bit = ((r + ny + 1) * nx + 32 * (wr - 1)) // 32 * 32 + 5 * 32
            assert classified is None or max_bit < classified, (s, max_bit, classified)
        # emit of slab s
        if E[s + 1] > E[s]:
            r = (E[s + 1] - 1) // wr
            max_bit = (r + 2 * ny + 1) * nx + 32 * wr + 2 * 32
            assert classified is None or max_bit < classified, (s, max_bit, classified)
            # offsets read: owner words up to (r + ny + 1) rows ahead, one word
            # on; the capacity check at E[s+1]; all scanned by slabs <= s
            last_word = (E[s + 1] - 1) + wr * (ny + 1) + 1
            if s + 1 < S:
                assert last_word < W[s + 1] and E[s + 1] < W[s + 1], s


def test_plan_uses_the_requested_slabs_at_512(lib):
    S, W, E, K = _plan(lib, (512, 512, 512), 8)
    assert S == 8
    assert W[1] == 128 * TILE  # 1024 tiles, 128 per slab
    assert E[1] == W[1] - (16 * 513 + 2)


def test_plan_of_default_setting(lib):
    capi.call("dax_gb300_set_pipeline_slabs", 0)
    assert _plan(lib, (512, 512, 512), 0)[0] == 1
    capi.call("dax_gb300_set_pipeline_slabs", 8)
    assert _plan(lib, (512, 512, 512), 0)[0] == 8
    capi.call("dax_gb300_set_pipeline_slabs", 0)
    with pytest.raises(capi.ErrorControlBadValue):
        capi.call("dax_gb300_set_pipeline_slabs", 17)
