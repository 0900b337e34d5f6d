"""The device adapter's generic primitives against the reference's own tests.

The first half restates dax/cont/testing/TestingDeviceAdapter.h (ARRAY_SIZE
500, OFFSET 1000, :54-55) case by case -- scans of OFFSET-filled arrays
(:940-1001), StreamCompact with and without a stencil (:564-619), Sort /
Unique / LowerBounds / UpperBounds on i % 50 data and on its eight-value
known-answer array (:621-717), Sort with SortLess / SortGreater (:719-768),
SortByKey with dax::Vector3 values and keys (:770-838).  The second half
compares against numpy on large random inputs of every element type, with
edge cases (empty, one element, ragged tile ends, all-equal keys, reversed
input).  Integer results are exact; float scans are compared with a relative
tolerance of 1e-5 of the running magnitude (summation order differs).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ARRAY_SIZE = 500
OFFSET = 1000


@pytest.fixture(scope="module")
def A(gb300):
    return gb300.Algorithm


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# ---- TestingDeviceAdapter.h ----------------------------------------------------
def test_scan_inclusive_reference(A):
    arr = torch.full((ARRAY_SIZE,), OFFSET, dtype=torch.int32, device="cuda")
    total, out = A.ScanInclusive(arr, arr)
    assert total == OFFSET * ARRAY_SIZE
    pos = np.arange(1, ARRAY_SIZE + 1)
    assert np.array_equal(np.cumsum(out.cpu().numpy()), pos * (pos + 1) // 2 * OFFSET)


def test_scan_exclusive_reference(A):
    arr = torch.full((ARRAY_SIZE,), OFFSET, dtype=torch.int32, device="cuda")
    total, out = A.ScanExclusive(arr, arr)
    assert total == OFFSET * ARRAY_SIZE
    pos = np.arange(ARRAY_SIZE)
    assert np.array_equal(np.cumsum(out.cpu().numpy()), pos * (pos + 1) // 2 * OFFSET)


def test_stream_compact_reference(A):
    stencil = cuda((np.arange(ARRAY_SIZE) % 2).astype(np.int32))  # MarkOddNumbersKernel
    res = A.StreamCompact(stencil).cpu().numpy()
    assert len(res) == ARRAY_SIZE // 2
    assert np.array_equal(res, np.arange(ARRAY_SIZE // 2) * 2 + 1)


def test_stream_compact_with_stencil_reference(A):
    arr = cuda((OFFSET + np.arange(ARRAY_SIZE)).astype(np.int32))  # OffsetPlusIndexKernel
    stencil = cuda((np.arange(ARRAY_SIZE) % 2).astype(np.int32))
    res = A.StreamCompact(arr, stencil).cpu().numpy()
    assert len(res) == ARRAY_SIZE // 2
    assert np.array_equal(res, OFFSET + np.arange(ARRAY_SIZE // 2) * 2 + 1)


def test_ordered_unique_values_reference(A):
    data = (OFFSET + np.arange(ARRAY_SIZE) % 50).astype(np.int32)
    inp = cuda(data)
    temp = A.Copy(inp)
    A.Sort(temp)
    uniq = A.Unique(temp)
    assert uniq.numel() == 50
    lo = A.LowerBounds(uniq, inp).cpu().numpy()
    up = A.UpperBounds(uniq, inp).cpu().numpy()
    i = np.arange(ARRAY_SIZE)
    assert np.array_equal(lo, i % 50)
    assert np.all(up >= i % 50) and np.array_equal(up, i % 50 + 1)


def test_random_values_bounds_reference(A):
    random_data = np.array([500, 955, 955, 120, 320, 955, 986, 281], np.int32)
    inp = cuda(random_data)
    temp = A.Copy(inp)
    A.Sort(temp)
    uniq = A.Unique(temp)
    assert np.array_equal(A.LowerBounds(uniq, inp).cpu().numpy(), [3, 4, 4, 0, 2, 4, 5, 1])
    assert np.array_equal(A.UpperBounds(uniq, inp).cpu().numpy(), [4, 5, 5, 1, 3, 5, 6, 2])
    # values_output in place (the reference's two-argument LowerBounds)
    vals = A.Copy(inp)
    A.LowerBounds(uniq, vals, vals)
    assert np.array_equal(vals.cpu().numpy(), [3, 4, 4, 0, 2, 4, 5, 1])


def test_sort_with_comparison_object_reference(A, gb300):
    data = (OFFSET + (ARRAY_SIZE - np.arange(ARRAY_SIZE)) % 50).astype(np.int32)
    sorted_ = A.Sort(cuda(data)).cpu().numpy()
    assert np.all(sorted_[:-1] <= sorted_[1:])
    comp = A.Sort(cuda(data), gb300.SortGreater())
    assert np.array_equal(comp.cpu().numpy(), sorted_[::-1])
    less = A.Sort(comp, gb300.SortLess())
    assert np.array_equal(less.cpu().numpy(), sorted_)


def test_sort_by_key_reference(A, gb300):
    i = np.arange(ARRAY_SIZE)
    keys = cuda((ARRAY_SIZE - i).astype(np.int32))
    values = cuda(np.repeat(i.astype(np.float32)[:, None], 3, axis=1))  # dax::Vector3(i)
    A.SortByKey(keys, values)
    assert np.array_equal(keys.cpu().numpy(), i + 1)
    assert np.array_equal(values[:, 0].cpu().numpy(), ARRAY_SIZE - 1 - i)
    A.SortByKey(keys, values, gb300.SortGreater())
    assert np.array_equal(keys.cpu().numpy(), ARRAY_SIZE - i)
    assert np.array_equal(values[:, 0].cpu().numpy(), i)
    # sorting by dax::Vector3 keys (tuples compare component by component)
    A.SortByKey(values, keys)
    assert np.array_equal(values[:, 0].cpu().numpy(), i)
    assert np.array_equal(keys.cpu().numpy(), ARRAY_SIZE - i)


# ---- against numpy -------------------------------------------------------------
SIZES = [0, 1, 4095, 4096, 4097, 1_000_003]


def _rand(dtype, n, rng, lo=None, hi=None):
    if dtype == np.float32:
        return rng.standard_normal(n).astype(np.float32)
    info = np.iinfo(dtype)
    return rng.integers(info.min if lo is None else lo, (info.max if hi is None else hi),
                        n, dtype=dtype, endpoint=True)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32])
@pytest.mark.parametrize("exclusive", [False, True])
def test_scan_random(A, n, dtype, exclusive):
    rng = np.random.default_rng(n + 7)
    x = _rand(dtype, n, rng, -1000, 1000) if dtype != np.float32 else rng.random(n, np.float32)
    fn = A.ScanExclusive if exclusive else A.ScanInclusive
    total, out = fn(cuda(x))
    got = out.cpu().numpy()
    if dtype == np.float32:
        ref = np.cumsum(x.astype(np.float64))
        if exclusive:
            ref = np.concatenate([[0.0], ref[:-1]])[:n]
        scale = np.maximum(np.abs(np.cumsum(np.abs(x.astype(np.float64)))), 1.0)
        assert np.all(np.abs(got - ref) <= 1e-5 * scale)
        assert abs(total - float(np.sum(x, dtype=np.float64))) <= 1e-5 * max(1.0, float(scale[-1]) if n else 1.0)
    else:
        ref = np.cumsum(x, dtype=dtype)
        if exclusive:
            ref = np.concatenate([np.zeros(1, dtype), ref[:-1]])[:n]
        assert np.array_equal(got, ref)
        assert total == int(np.sum(x, dtype=dtype))


def test_scan_int32_wraps(A):
    x = np.full(10_000, 2 ** 30, np.int32)
    total, out = A.ScanInclusive(cuda(x))
    ref = np.cumsum(x, dtype=np.int32)  # wraps modulo 2^32
    assert np.array_equal(out.cpu().numpy(), ref)
    assert total == int(ref[-1])


# Integer scans run in one pass, each tile's prefix found by looking back
# over the tiles before it (64 KB tiles: 16384 int32 or 8192 int64 elements;
# 32 tiles a look-back step).  These sizes span thousands of tiles and many
# steps, exactly 33 tiles, and ragged ends; the scan is repeated in place and
# out of place and must give the same bits.
@pytest.mark.parametrize("n,dtype", [(50_000_001, np.int32), (12_345_679, np.int64),
                                     (16384 * 33, np.int32), (8192 * 32 + 1, np.int64)])
def test_scan_single_pass_large(A, n, dtype):
    rng = np.random.default_rng(n)
    x = _rand(dtype, n, rng)  # the type's full range: sums wrap all the time
    ref = np.cumsum(x, dtype=dtype)
    ref_ex = np.concatenate([np.zeros(1, dtype), ref[:-1]])
    d = cuda(x)
    for _ in range(2):
        total, out = A.ScanInclusive(d)
        assert np.array_equal(out.cpu().numpy(), ref)
        assert total == int(ref[-1])
    total, out = A.ScanExclusive(d)
    assert np.array_equal(out.cpu().numpy(), ref_ex)
    assert total == int(ref[-1])
    total, out = A.ScanInclusive(d, d)  # in place
    assert out.data_ptr() == d.data_ptr()
    assert np.array_equal(d.cpu().numpy(), ref)


def test_scan_single_pass_unaligned(A):
    """Arrays that do not start on a 16-byte boundary take element loads and
    stores instead of the bulk copies; results are the same."""
    n = 16384 * 5 + 77
    rng = np.random.default_rng(11)
    x = rng.integers(-2 ** 31, 2 ** 31 - 1, n + 3, dtype=np.int32, endpoint=True)
    d = cuda(x)
    src, dst = d[1:n + 1], torch.empty(n + 2, dtype=torch.int32, device="cuda")[2:]
    total, out = A.ScanInclusive(src, dst)
    ref = np.cumsum(x[1:n + 1], dtype=np.int32)
    assert np.array_equal(dst.cpu().numpy(), ref)
    assert total == int(ref[-1])


@pytest.mark.parametrize("unsigned", [np.uint32, np.uint64])
def test_scan_unsigned_through_abi(gb300, unsigned):
    """U32 / U64 through the C ABI directly (torch has no unsigned scan types
    to carry them in the wrapper): the bits of the signed scan of the same
    words, and the total in the element's width."""
    import ctypes
    from daxtoolkit_gb300 import capi
    n = 3_000_017
    rng = np.random.default_rng(5)
    x = rng.integers(0, np.iinfo(unsigned).max, n, dtype=unsigned, endpoint=True)
    ref = np.cumsum(x, dtype=unsigned)
    signed = np.int32 if unsigned == np.uint32 else np.int64
    d = cuda(x.view(signed))
    out = torch.empty_like(d)
    nb = capi.lib().dax_gb300_scan_scratch_bytes(n)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    total = np.zeros(1, unsigned)
    t = 1 if unsigned == np.uint32 else 4  # DAX_GB300_TYPE_U32 / _U64
    capi.call("dax_gb300_scan", ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(out.data_ptr()), n,
              t, 0, ctypes.c_void_p(scratch.data_ptr()), nb,
              ctypes.c_void_p(total.ctypes.data), None)
    assert np.array_equal(out.cpu().numpy().view(unsigned), ref)
    assert total[0] == ref[-1]


def _ordered_bits(k):
    """Unsigned integers with the order of k (IEEE order for floats)."""
    if k.dtype == np.float32:
        u = k.view(np.uint32)
        return np.where(u >> 31 == 1, ~u, u | np.uint32(0x80000000))
    if k.dtype == np.int32:
        return k.view(np.uint32) ^ np.uint32(0x80000000)
    if k.dtype == np.int64:
        return k.view(np.uint64) ^ np.uint64(0x8000000000000000)
    return k


def _stable_order(k, desc):
    b = _ordered_bits(k)
    return np.argsort(~b if desc else b, kind="stable")


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32, np.uint32])
@pytest.mark.parametrize("vcols", [0, 1, 3, 4])
@pytest.mark.parametrize("desc", [False, True])
def test_sort_by_key_random(A, gb300, n, dtype, vcols, desc):
    if dtype == np.uint32 and not hasattr(torch, "uint32"):
        pytest.skip("torch without uint32")
    if dtype == np.int64 and n > 100_000 and vcols not in (0, 3):
        pytest.skip("covered by the other value widths")
    rng = np.random.default_rng(1000 + n)
    # few distinct keys: many ties, so stability is exercised
    if dtype == np.float32:
        k = (rng.integers(-50, 50, n) / 4.0).astype(np.float32)
        k[k == 0] = 0.125
    elif dtype == np.uint32:
        k = rng.integers(0, 2 ** 32 - 1, n, dtype=np.uint64).astype(np.uint32)
        k[::3] = 7
    else:
        k = _rand(dtype, n, rng)
        k[::3] = -5
    v = np.arange(n * max(vcols, 1), dtype=np.int32).reshape(n, max(vcols, 1))
    keys = cuda(k)
    vals = cuda(v[:, :vcols] if vcols > 1 else v[:, 0]) if vcols else None
    A.SortByKey(keys, vals, gb300.SortGreater() if desc else None)
    order = _stable_order(k, desc)
    assert np.array_equal(keys.cpu().numpy(), k[order])
    if vcols:
        ref = v[order][:, :vcols] if vcols > 1 else v[order][:, 0]
        assert np.array_equal(vals.cpu().numpy(), ref)


def test_sort_special_inputs(A, gb300):
    for x in (np.zeros(5000, np.int32), np.arange(5000, dtype=np.int32)[::-1].copy(),
              np.arange(5000, dtype=np.int32), np.array([2 ** 31 - 1, -2 ** 31, 0, -1, 1], np.int32)):
        assert np.array_equal(A.Sort(cuda(x)).cpu().numpy(), np.sort(x))
    f = np.array([3.5, -0.0, 0.0, -7.25, np.inf, -np.inf, 1e-40, -1e-40], np.float32)
    got = A.Sort(cuda(f)).cpu().numpy()
    assert np.array_equal(got, np.sort(f))
    assert np.signbit(got[3]) and not np.signbit(got[4])  # -0 before +0


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32])
def test_unique_random(A, n, dtype):
    rng = np.random.default_rng(n + 3)
    x = np.sort(rng.integers(0, max(n // 7, 1), n)).astype(dtype)
    got = A.Unique(cuda(x)).cpu().numpy()
    assert np.array_equal(got, np.unique(x))


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("stype", [np.int32, np.float32])
@pytest.mark.parametrize("vcols", [0, 1, 3])
def test_stream_compact_random(A, n, stype, vcols):
    rng = np.random.default_rng(n + 11)
    stencil = (rng.random(n) < 0.3).astype(stype) * rng.integers(1, 5, n).astype(stype)
    if vcols == 0:
        got = A.StreamCompact(cuda(stencil)).cpu().numpy()
        assert np.array_equal(got, np.nonzero(stencil)[0].astype(np.int32))
    else:
        v = rng.standard_normal((n, vcols)).astype(np.float32)
        vv = v if vcols > 1 else v[:, 0]
        got = A.StreamCompact(cuda(vv), cuda(stencil)).cpu().numpy()
        assert np.array_equal(got, vv[stencil != 0])


# StreamCompact and Unique run in one pass: 64 KB tiles of the stencil (or
# keys), each tile's offset found by looking back over the tiles before it.
# These cases span thousands of tiles, NaN and -0.0 stencil entries, 16-byte
# values, an unaligned stencil (element loads instead of bulk copies) and
# Unique in place on 8-byte and float keys.
def test_stream_compact_single_pass_large(A):
    n = 40_000_003
    rng = np.random.default_rng(17)
    stencil = np.where(rng.random(n) < 0.3, rng.standard_normal(n), 0.0).astype(np.float32)
    stencil[rng.integers(0, n, 1000)] = np.nan   # NaN != 0: kept
    stencil[rng.integers(0, n, 1000)] = -0.0     # -0.0 == 0: dropped
    keep = stencil != 0
    got = A.StreamCompact(cuda(stencil)).cpu().numpy()
    assert np.array_equal(got, np.nonzero(keep)[0].astype(np.int32))
    v = rng.integers(-2 ** 31, 2 ** 31 - 1, (n, 4), dtype=np.int32, endpoint=True)  # 16-byte rows
    got = A.StreamCompact(cuda(v), cuda(stencil)).cpu().numpy()
    assert np.array_equal(got, v[keep])
    # an int32 stencil that starts 4 bytes past a 16-byte boundary
    si = (rng.random(n + 1) < 0.5).astype(np.int32)
    d = cuda(si)[1:]
    got = A.StreamCompact(d).cpu().numpy()
    assert np.array_equal(got, np.nonzero(si[1:])[0].astype(np.int32))


@pytest.mark.parametrize("dtype", [np.int64, np.float32, np.int32])
def test_unique_single_pass_large(A, dtype):
    n = 30_000_001
    rng = np.random.default_rng(23)
    x = np.sort(rng.integers(-5_000_000, 5_000_000, n)).astype(dtype)
    if dtype == np.float32:
        x[x == 0] = -0.0
        x[np.flatnonzero(x == 0)[::2]] = 0.0  # -0.0 and +0.0 adjacent: one run
    d = cuda(x)
    got = A.Unique(d)
    assert got.data_ptr() == d.data_ptr()  # in place
    ref = x[np.concatenate([[True], x[1:] != x[:-1]])]
    assert np.array_equal(got.cpu().numpy(), ref)


@pytest.mark.parametrize("n", [0, 1, 4097, 300_001])
@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32])
def test_bounds_random(A, n, dtype):
    rng = np.random.default_rng(n + 5)
    s = np.sort(rng.integers(-1000, 1000, n)).astype(dtype)
    q = rng.integers(-1100, 1100, 200_003).astype(dtype)
    lo = A.LowerBounds(cuda(s), cuda(q)).cpu().numpy()
    up = A.UpperBounds(cuda(s), cuda(q)).cpu().numpy()
    assert np.array_equal(lo, np.searchsorted(s, q, side="left"))
    assert np.array_equal(up, np.searchsorted(s, q, side="right"))
