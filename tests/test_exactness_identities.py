"""CPU checks of the arithmetic identities the exact kernels rely on (no GPU needed).

- The shortlist pick sums (a - b)^2 over rows of 32 categorical codes 0..3 held as two bit
  planes: with u = a1 - b1, v = a0 - b0, (a - b)^2 = 4u^2 + 4uv + v^2, u^2 = a1 ^ b1,
  v^2 = a0 ^ b0 and, where both are nonzero, uv = +1 exactly when a1 == a0. Per row:
  popc(x0) + 4 (popc(x1) + popc(y)) - 8 popc(y & (a1 ^ a0)), x = (a ^ b) & mask, y = x1 & x0.
- Per-position passes compare FP32 map values with Float64 bounds in FP32, through the
  directed roundings of the bound: (double)d < x <=> d < round_up(x), (double)d <= x <=>
  d <= round_down(x).
"""
import numpy as np


def _popc(v):
    return bin(int(v)).count("1")


def _row_ssd_planes(a, b, m):
    """The kernel's row formula on 32 codes a, b (0..3) under the boolean mask m."""
    bits = lambda arr: sum(int(x) << i for i, x in enumerate(arr))
    a0, a1 = bits(a & 1), bits(a >> 1)
    b0, b1 = bits(b & 1), bits(b >> 1)
    mk = bits(m.astype(np.int64))
    x1, x0 = (a1 ^ b1) & mk, (a0 ^ b0) & mk
    y = x1 & x0
    return _popc(x0) + 4 * (_popc(x1) + _popc(y)) - 8 * _popc(y & (a1 ^ a0))


def test_plane_row_sum_equals_direct_sum():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        a = rng.integers(0, 4, 32)
        b = rng.integers(0, 4, 32)
        m = rng.random(32) < rng.random()
        direct = int((((a - b) ** 2) * m).sum())
        assert _row_ssd_planes(a, b, m) == direct


def test_plane_row_sum_every_code_pair():
    for x in range(4):
        for y in range(4):
            a = np.full(32, x)
            b = np.full(32, y)
            assert _row_ssd_planes(a, b, np.ones(32, bool)) == 32 * (x - y) ** 2


def _round_up(x):
    f = np.float32(x)
    return f if float(f) >= x else np.nextafter(f, np.float32(np.inf))


def _round_down(x):
    f = np.float32(x)
    return f if float(f) <= x else np.nextafter(f, np.float32(-np.inf))


def test_float_comparisons_against_double_bounds():
    rng = np.random.default_rng(1)
    for _ in range(20000):
        x = float(rng.standard_normal() * 10.0 ** int(rng.integers(-6, 6)))
        # floats near x, and x itself when it is a float
        d = np.float32(x) if rng.random() < 0.3 else np.nextafter(
            np.float32(x), np.float32(np.inf if rng.random() < 0.5 else -np.inf))
        assert (float(d) < x) == bool(d < _round_up(x))
        assert (float(d) <= x) == bool(d <= _round_down(x))
        assert (float(d) > x) == bool(d > _round_down(x))
