"""The arguments behind two same-bits rewrites in the device code, checked on
the host with IEEE doubles (numpy), lane by lane:

* the warp reduce-scatter (mph_device.cuh: warp_sum_scatter, warp_reduce_scatter)
  adds the same pairs as the xor butterfly `v += shfl_xor(v, o)`,
  o = 16 ... 1, so each lane's result has the butterfly's bits for the
  component it holds (FP64 addition commutes);
* the range and radius tests on bit patterns (sep_exact, r2_within,
  r2_pos_below) decide as the FP64 compares they replace, for every value a
  squared distance or a shifted separation can take, NaN included.
"""
import numpy as np


def _butterfly(v):
    """v: (trials, 32 lanes, N) -> every lane's sums after the xor butterfly"""
    for o in (16, 8, 4, 2, 1):
        v = v + v[:, np.arange(32) ^ o, :]
    return v


def _reduce_scatter(v):
    """warp_reduce_scatter<N>: lanes with bit o set keep the upper half of
    their values, the others the lower half, each adding the partner's copy
    of the half it keeps; then plain butterfly steps.  Returns each lane's sum
    and the index of the value it holds (lane >> (5 - log2 N))."""
    n = v.shape[2]
    L = n.bit_length() - 1
    lanes = np.arange(32)
    for s in range(L):
        o = 16 >> s
        h = (n >> s) // 2
        up = (lanes & o) != 0
        keep = np.where(up[None, :, None], v[:, :, h:2 * h], v[:, :, :h])
        send = np.where(up[None, :, None], v[:, :, :h], v[:, :, h:2 * h])
        v = keep + send[:, lanes ^ o, :]
    a = v[:, :, 0]
    o = 16 >> L
    while o > 0:
        a = a + a[:, lanes ^ o]
        o >>= 1
    return a, lanes >> (5 - L)


def _warp_sum_scatter3(v):
    """warp_sum_scatter<3>: lanes 0-15 keep components 0 and 1, 16-31
    component 2 twice; then lanes 0-7 component 0, 8-15 component 1, 16-31
    component 2."""
    lanes = np.arange(32)
    hi = (lanes & 16) != 0
    a0 = np.where(hi, v[:, :, 2], v[:, :, 0]) + np.where(hi, v[:, :, 0], v[:, :, 2])[:, lanes ^ 16]
    a1 = np.where(hi, v[:, :, 2], v[:, :, 1]) + np.where(hi, v[:, :, 1], v[:, :, 2])[:, lanes ^ 16]
    b8 = (lanes & 8) != 0
    a = np.where(b8, a1, a0) + np.where(b8, a0, a1)[:, lanes ^ 8]
    for o in (4, 2, 1):
        a = a + a[:, lanes ^ o]
    return a, np.minimum(lanes >> 3, 2)


def _lane_values(rng, trials, n):
    mag = 10.0 ** rng.uniform(-9, 9, size=(trials, 32, n))
    v = rng.uniform(-1, 1, size=(trials, 32, n)) * mag
    v[rng.random((trials, 32, n)) < 0.2] = 0.0   # rows with fewer slots than lanes
    return v


def test_reduce_scatter_has_the_butterfly_bits():
    rng = np.random.default_rng(7)
    for n in (2, 4, 8, 16, 32):
        v = _lane_values(rng, 400, n)
        ref = _butterfly(v)
        got, idx = _reduce_scatter(v)
        want = ref[:, np.arange(32), idx]
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), n


def test_three_component_scatter_has_the_butterfly_bits():
    rng = np.random.default_rng(8)
    v = _lane_values(rng, 2000, 3)
    ref = _butterfly(v)
    got, idx = _warp_sum_scatter3(v)
    want = ref[:, np.arange(32), idx]
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    # the wall kernel's nine sums padded to sixteen values
    v9 = np.concatenate([_lane_values(rng, 400, 9), np.zeros((400, 32, 7))], axis=2)
    got, idx = _reduce_scatter(v9)
    want = _butterfly(v9)[:, np.arange(32), idx]
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def _bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def _special():
    return np.array([0.0, 5e-324, 1e-310, 2.2250738585072014e-308, 1.0, 1e300,
                     np.inf, np.nan, -np.nan], dtype=np.float64)


def test_radius_tests_on_bit_patterns():
    rng = np.random.default_rng(9)
    r2 = np.abs(rng.uniform(0, 2, 300000)) * 10.0 ** rng.uniform(-8, 3, 300000)
    R2 = rng.uniform(1e-6, 10, 300000)
    r2[::97] = R2[::97]                        # on the radius
    r2 = np.concatenate([r2, np.repeat(_special(), 50)])
    R2 = np.concatenate([R2, np.tile(rng.uniform(1e-6, 10, 50), len(_special()))])
    with np.errstate(invalid="ignore"):
        within = R2 - r2 >= 0                  # the reference's forms
        pos_below = (r2 != 0) & (R2 - r2 > 0)
    b, B = _bits(r2), _bits(R2)
    assert np.array_equal(within, (b >= 0) & (b <= B))          # r2_within
    assert np.array_equal(pos_below, (b > 0) & (b < B))         # r2_pos_below


def test_minimum_image_range_test_on_bit_patterns():
    rng = np.random.default_rng(10)
    t = rng.uniform(-3, 3, 300000) * 10.0 ** rng.uniform(-3, 3, 300000)
    t = np.concatenate([t, _special(), -_special()[1:7]])
    wsafe = rng.uniform(0.1, 100, t.size)
    wsafe[:1000] = np.abs(t[:1000])            # on the bound
    with np.errstate(invalid="ignore"):
        fast = (t >= 0.0) & (t < wsafe)
    tb = _bits(t)
    assert np.array_equal(fast, (tb >= 0) & (tb < _bits(wsafe)))
