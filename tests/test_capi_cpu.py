"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/dax_gb300.h declares; host-side argument validation (no GPU work)."""
import ctypes

import pytest

from daxtoolkit_gb300 import build, capi


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.lib()


def test_header_symbols_exported(lib):
    names = capi.header_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in capi.SIGNATURES, n


def test_abi_version(lib):
    assert lib.dax_gb300_abi_version() == 1


def _desc(emin, emax):
    g = capi.UniformGridDesc()
    for a in range(3):
        g.spacing[a] = 1.0
        g.extent_min[a] = emin[a]
        g.extent_max[a] = emax[a]
    return g


def test_scratch_sizes_grow_with_grid(lib):
    small = lib.dax_gb300_mc_scratch_bytes(ctypes.byref(_desc((0, 0, 0), (15, 15, 15))))
    big = lib.dax_gb300_mc_scratch_bytes(ctypes.byref(_desc((0, 0, 0), (63, 63, 63))))
    thr = lib.dax_gb300_threshold_scratch_bytes(ctypes.byref(_desc((0, 0, 0), (63, 63, 63))))
    assert 0 < small < big and thr > small
    # bits (P/8) + two int64 row offsets per row dominate
    assert big >= 64 ** 3 // 8 + 2 * 8 * 64 * 64


@pytest.mark.parametrize("n", [1, 4095, 8192, 8193, 16384, 16385, 1_000_003, 2 ** 31 - 1])
def test_primitive_scratch_covers_single_pass(lib, n):
    """The single-pass scan and compaction write a 64-byte control head and a
    state per 64 KB tile of the staged array: 16 bytes for 64-bit sums (int64
    scans: 8192 elements a tile), 8 bytes for 32-bit ones (int32 scans and the
    compaction's counts: 16384 4-byte or 8192 8-byte elements a tile).  The
    public scratch sizes must cover the largest of these for every n."""
    def tiles(per):
        return (n + per - 1) // per
    assert lib.dax_gb300_scan_scratch_bytes(n) >= 64 + 16 * tiles(8192)
    assert lib.dax_gb300_scan_scratch_bytes(n) >= 64 + 8 * tiles(16384)
    assert lib.dax_gb300_compact_scratch_bytes(n, 0) >= 64 + 8 * tiles(16384)
    assert lib.dax_gb300_compact_scratch_bytes(n, 4) >= 64 + 8 * tiles(16384)
    assert lib.dax_gb300_compact_scratch_bytes(n, 8) >= 64 + 8 * tiles(8192)


def test_bad_extent_rejected(lib):
    g = _desc((0, 0, 0), (-1, 3, 3))
    assert lib.dax_gb300_mc_scratch_bytes(ctypes.byref(g)) == 0
    st = lib.dax_gb300_mc_count(ctypes.byref(g), None, 0.0, None, 0, None)
    assert st == capi.ERROR_BAD_VALUE
    assert b"extent" in lib.dax_gb300_last_error()


def test_too_many_points_rejected(lib):
    g = _desc((0, 0, 0), (2047, 2047, 1023))  # 2^32 points > int32 ids
    st = lib.dax_gb300_mc_count(ctypes.byref(g), None, 0.0, None, 0, None)
    assert st == capi.ERROR_UNSUPPORTED


def test_null_field_rejected(lib):
    g = _desc((0, 0, 0), (7, 7, 7))
    st = lib.dax_gb300_cell_gradient(ctypes.byref(g), None, None, None)
    assert st == capi.ERROR_BAD_VALUE
    with pytest.raises(capi.ErrorControlBadValue):
        capi.check(st)
