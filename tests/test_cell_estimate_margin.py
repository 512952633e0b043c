"""CPU check of the build's FP32 cell shortcut (octree_gb300/csrc/otg_build.cu: cell_estimate_margin,
entity_key): where the FP32 estimate of a coordinate clears the rounding margin, its truncation must
be the reference's cell. The estimate is restated here in numpy FP32 arithmetic (round to nearest,
no fused multiply-add, as the kernels are compiled) and compared with the oracle's location keys on
coordinates on cell boundaries, a few ulps either side, at distances around the margin, and at
random, for spaces near and far from the origin."""
import numpy as np
import pytest

from _oracle_lib import KIND_POINTS, oracle


def approx_f(x):
    """FP64 -> FP32 by truncating the mantissa to 23 bits (the kernels' approx_f)."""
    b = np.ascontiguousarray(x, np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    ex = ((hi >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64) - 1023 + 127
    bits = (hi & np.uint32(0x80000000)) | (np.clip(ex, 0, 255).astype(np.uint32) << np.uint32(23))
    bits |= ((hi & np.uint32(0xFFFFF)) << np.uint32(3)) | (lo >> np.uint32(29))
    f = bits.view(np.float32).copy()
    f[ex <= 0] = 0.0
    big = ex >= 255
    f[big] = np.where((hi[big] >> np.uint32(31)) != 0, np.float32(-3.0e38), np.float32(3.0e38))
    return f


def compact1by2(v):
    v = v & np.uint64(0x9249249249249249)
    for sh, m in ((2, 0x30C30C30C30C30C3), (4, 0xF00F00F00F00F00F), (8, 0x00FF0000FF0000FF), (16, 0xFFFF00000000FFFF), (32, 0x1FFFFF)):
        v = (v ^ (v >> np.uint64(sh))) & np.uint64(m)
    return v


def estimate_cells(pts, lo, hi, depth, margin_scale=1.0):
    """(fast, cell) per coordinate: whether the estimate clears its margin (scaled by margin_scale),
    and trunc(estimate)."""
    cells = 1 << depth
    f32 = pts.dtype == np.float32
    if f32:  # FP32 trees below depth 16 rasterise in FP32: rast = float(2^D) / (max - min)
        size = (hi - lo).astype(np.float32)
        rast = np.where(size == 0, np.float32(1), np.float32(cells) / np.where(size == 0, np.float32(1), size)).astype(np.float32)
        rast_d = rast.astype(np.float64)
        ax = pts.astype(np.float32)
    else:
        size = (hi - lo).astype(np.float64)
        rast_d = np.where(size == 0, 1.0, cells / np.where(size == 0, 1.0, size))
        rast = rast_d.astype(np.float32)
        ax = approx_f(pts)
    min_f = lo.astype(np.float32)
    est = ((ax - min_f).astype(np.float32) * rast).astype(np.float32)
    M = np.maximum(np.abs(lo.astype(np.float64)), np.abs(hi.astype(np.float64)))
    m = (rast_d * M * 2.0**-22 + cells * 2.0**-22 + 2.0**-20) * margin_scale
    m32 = m.astype(np.float32)
    m32 = np.where(m32.astype(np.float64) < m, np.nextafter(m32, np.float32(np.inf)), m32)  # rounded up
    m32 = np.where(m < 0.25, m32, np.float32(2.0))
    inside = (est > m32) & (est < np.float32(cells) - m32)
    g = np.where(inside, np.trunc(np.where(inside, est, 0)), 0).astype(np.int64)
    frac = (est - g.astype(np.float32)).astype(np.float32)
    fast = inside & (frac > m32) & (frac < np.float32(1) - m32)
    return fast, g


SIZE = 1000.123456789  # a space whose cell boundaries and factor are not short binary fractions
LOW = 0.3712345


def _space(offset):
    return offset + LOW, offset + LOW + SIZE


def _points(rng, depth, offset, dtype, n=40_000):
    cells = 1 << depth
    lo, hi = _space(offset)
    width = SIZE / cells
    j = rng.integers(0, cells + 1, (n, 3)).astype(np.float64)
    x = lo + j * width
    k = rng.integers(-4, 5, x.shape)
    for step in range(4):
        x = np.where(k > step, np.nextafter(x, np.inf), np.where(k < -step, np.nextafter(x, -np.inf), x))
    margin = (SIZE + abs(offset)) * (cells / SIZE) * 2.0**-22 + cells * 2.0**-22
    near = lo + (j + rng.choice([-2.0, -1.0, -0.5, 0.5, 1.0, 2.0], j.shape) * margin) * width
    band = lo + (j + (rng.random(j.shape) * 2.0 - 1.0) * 2.0 * margin) * width  # full-mantissa values
    pts = np.concatenate([x, near, band, lo + rng.random((n, 3)) * SIZE])  # the random points come last
    return np.clip(pts, lo, hi).astype(dtype)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("depth", [8, 10, 12, 15])
@pytest.mark.parametrize("offset", [0.0, 819.0, -5000.0, 1e6])
def test_estimate_cells_match_the_oracle(dtype, depth, offset):
    rng = np.random.default_rng(depth * 7 + int(abs(offset)) % 1000)
    pts = _points(rng, depth, offset, dtype)
    for box in (None, np.array([_space(offset)[0]] * 3 + [_space(offset)[1]] * 3, dtype)):
        lo = pts.min(0) if box is None else box[:3]
        hi = pts.max(0) if box is None else box[3:]
        fast, g = estimate_cells(pts, lo, hi, depth)
        keys = oracle().create(pts, KIND_POINTS, depth, box, 16).location_keys()
        loc = keys >> np.uint64(5)
        ref = np.stack([compact1by2(loc >> np.uint64(s)).astype(np.int64) for s in range(3)], 1)
        valid = (keys != 0)[:, None]
        bad = fast & ~(valid & (ref == g))
        assert not bad.any(), f"{int(bad.sum())} estimated cells differ from the reference's, e.g. {pts[np.argwhere(bad)[0][0]]}"
        if offset == 0.0 and depth <= 12:
            # the shortcut decides nearly every random coordinate near the origin
            assert fast[-40_000:].mean() > 0.99
        if offset == 1e6 and dtype == np.float64 and depth >= 12:
            assert not fast.any()  # a margin of 1/4 or more switches the shortcut off


def test_the_boundary_inputs_need_the_margin():
    """Without its margin the estimate gets cells wrong on these inputs: the check above has teeth."""
    rng = np.random.default_rng(5)
    pts = _points(rng, 10, 819.0, np.float64)
    fast, g = estimate_cells(pts, pts.min(0), pts.max(0), 10, margin_scale=0.0)
    keys = oracle().create(pts, KIND_POINTS, 10, None, 16).location_keys()
    loc = keys >> np.uint64(5)
    ref = np.stack([compact1by2(loc >> np.uint64(s)).astype(np.int64) for s in range(3)], 1)
    assert (fast & (ref != g)).any()
