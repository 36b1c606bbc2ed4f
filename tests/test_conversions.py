"""The integer FP64 -> FP32 and FP32 -> FP64 conversions of the split path (dev.cuh: narrow,
wide), restated bit for bit in numpy on uint64/uint32 patterns and checked against numpy's own
conversions (IEEE round to nearest even).  This checks the algorithm on random values and on
the cases it must get right: ties, carries out of the mantissa into the exponent, the edges of
the FP32 normal range (where the device code hands over to the hardware conversion), zeros."""
import numpy as np


def narrow_bits(x: np.ndarray):
    """(result, handled) of dev.cuh:narrow for float64 x; handled = the integer path applies."""
    b = x.view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    e = (hi >> np.uint32(20)) & np.uint32(0x7FF)
    handled = (e - np.uint32(897)) < np.uint32(254)  # unsigned wrap, as in the C code
    m = ((hi & np.uint32(0xFFFFF)) << np.uint32(3)) | (lo >> np.uint32(29))
    f = (hi & np.uint32(0x80000000)) | ((e - np.uint32(896)) << np.uint32(23)) | m
    rest = lo & np.uint32(0x1FFFFFFF)
    f = f + ((rest + (m & np.uint32(1)) + np.uint32(0x0FFFFFFF)) >> np.uint32(29))
    return f.view(np.float32), handled


def wide_bits(f: np.ndarray):
    """(result, handled) of dev.cuh:wide for float32 f."""
    u = f.view(np.uint32)
    a = u & np.uint32(0x7FFFFFFF)
    handled = (a - np.uint32(0x00800000)) < np.uint32(0x7F000000)
    hi = (u & np.uint32(0x80000000)) | ((a >> np.uint32(3)) + (np.uint32(896) << np.uint32(20)))
    lo = a << np.uint32(29)
    b = (hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)
    return b.view(np.float64), handled


def _check_narrow(x):
    r, ok = narrow_bits(x)
    with np.errstate(over="ignore", invalid="ignore"):  # out-of-range values are excluded below
        ref = x.astype(np.float32)
    assert ok.any()
    np.testing.assert_array_equal(r[ok].view(np.uint32), ref[ok].view(np.uint32))
    # what the integer path leaves to the hardware: zero, FP32-subnormal results, overflow, NaN
    small = np.abs(x[~ok]) < 2.0 ** -126
    big = ~np.isfinite(x[~ok]) | (np.abs(x[~ok]) >= 2.0 ** 128)
    assert np.all(small | big)


def test_narrow_random_values():
    rng = np.random.default_rng(3)
    x = rng.standard_normal(1_000_000) * np.exp(rng.uniform(-80, 80, 1_000_000))
    _check_narrow(x)
    bits = rng.integers(0, 2 ** 63, 1_000_000, dtype=np.uint64) | (rng.integers(0, 2, 1_000_000, dtype=np.uint64) << 63)
    y = bits.view(np.float64)
    _check_narrow(y[np.isfinite(y)])


def test_narrow_ties_carries_and_range_edges():
    one = np.float64(1.0)
    ulp32 = 2.0 ** -23
    cases = [one + k * ulp32 / 2 for k in range(-4, 5)]                  # exact ties to even
    cases += [np.nextafter(one + ulp32 / 2, 2), np.nextafter(one + ulp32 / 2, 0)]
    cases += [np.nextafter(2.0, 0.0), np.nextafter(np.float64(np.float32(3.4e38)), 0)]  # carry into exponent
    cases += [2.0 ** -126, np.nextafter(2.0 ** -126, 1), np.nextafter(2.0 ** -126, 0), 2.0 ** 127]
    cases += [float(np.finfo(np.float32).max), np.nextafter(float(np.finfo(np.float32).max), np.inf)]
    x = np.array(cases + [-c for c in cases], dtype=np.float64)
    _check_narrow(x)
    r, ok = narrow_bits(np.array([0.0, -0.0, 1e-40, np.inf, np.nan, 1e39]))
    assert not ok.any()  # all handed to the hardware conversion


def test_wide_is_exact():
    rng = np.random.default_rng(4)
    f = rng.integers(0, 2 ** 32, 1_000_000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    r, ok = wide_bits(f)
    with np.errstate(invalid="ignore"):  # NaN patterns, excluded below
        ref = f.astype(np.float64)
    np.testing.assert_array_equal(r[ok].view(np.uint64), ref[ok].view(np.uint64))
    a = np.abs(f[~ok])
    assert np.all((a < np.float32(2.0 ** -126)) | ~np.isfinite(a))
