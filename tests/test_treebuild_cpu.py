"""CPU checks of the arithmetic facts the device tree build (meshlib_gb300/csrc/treebuild.cu) relies on.

The median select starts below the leading key bytes that the node box already fixes: every leaf's
key word is orderedBits(mn + mx) along the split dimension, and because float32 rounding is
monotone, mn + mx lies between (min mn) + (min mn) and (max mx) + (max mx).  These tests restate
the key map and the prefix arithmetic in numpy and check them on boxes with mixed signs, signed
zeros, ties and wide exponent ranges.
"""
import numpy as np


def ordered_bits(x: np.ndarray) -> np.ndarray:
    """treebuild.cu orderedBits: -0 becomes +0, then float32 maps monotonically onto uint32."""
    x = np.where(x == 0, np.float32(0), x).astype(np.float32)
    b = x.view(np.uint32)
    return np.where(b & np.uint32(0x80000000), ~b, b | np.uint32(0x80000000)).astype(np.uint32)


def common_prefix(lo: np.uint32, hi: np.uint32):
    """treebuild.cu segNodes: leading bytes shared by both ends and the prefix word they give."""
    x = int(lo) ^ int(hi)
    nb = 4 if x == 0 else (32 - x.bit_length()) // 8
    if nb == 4:
        return nb, int(lo)
    mask = 0 if nb == 0 else (~(0xFFFFFFFF >> (8 * nb))) & 0xFFFFFFFF
    return nb, int(lo) & mask


def _boxes(rng, n, centre, spread, ties):
    v = (centre + spread * rng.standard_normal((n, 3, 3))).astype(np.float32)
    if ties:  # shared vertices: many equal box ends, as on a real mesh
        v = np.round(v / spread * 4) * spread / 4
        v = v.astype(np.float32)
    mn, mx = v.min(axis=1), v.max(axis=1)
    return mn.astype(np.float32), mx.astype(np.float32)


def test_ordered_bits_is_monotone_and_merges_signed_zeros():
    vals = np.array([-np.inf, -3.5, -1e-30, -0.0, 0.0, 1e-38, 1e-30, 2.0, np.inf], np.float32)
    k = ordered_bits(vals)
    assert np.all(np.diff(k.astype(np.int64)) >= 0)
    assert k[3] == k[4]
    assert np.all(np.diff(k[4:].astype(np.int64)) > 0) and np.all(np.diff(k[:4].astype(np.int64)) > 0)


def test_centre_keys_lie_between_doubled_box_ends():
    rng = np.random.default_rng(7)
    cases = [(0.0, 1.0, False), (0.5, 0.01, False), (-3.0, 1e-3, True), (1e4, 1.0, True), (0.0, 1e-20, False),
             (0.0, 1.0, True)]
    for centre, spread, ties in cases:
        for _ in range(20):
            mn, mx = _boxes(rng, 2000, centre, spread, ties)
            for d in range(3):
                c = (mn[:, d] + mx[:, d]).astype(np.float32)  # makeLeaves: e.c[d] = e.mn[d] + e.mx[d]
                bmn, bmx = mn[:, d].min(), mx[:, d].max()
                lo = ordered_bits(np.array([bmn + bmn], np.float32))[0]
                hi = ordered_bits(np.array([bmx + bmx], np.float32))[0]
                keys = ordered_bits(c)
                assert keys.min() >= lo and keys.max() <= hi
                nb, prefix = common_prefix(lo, hi)
                if nb:
                    shift = 32 - 8 * nb
                    assert np.all((keys.astype(np.uint64) >> shift) == (prefix >> shift))


def test_prefix_of_identical_coordinates_is_the_whole_word():
    # a flat mesh: every centre has the same coordinate along the split dimension
    mn = np.zeros(100, np.float32)
    mx = np.zeros(100, np.float32)
    lo = ordered_bits(np.array([mn.min() * 2], np.float32))[0]
    hi = ordered_bits(np.array([mx.max() * 2], np.float32))[0]
    nb, prefix = common_prefix(lo, hi)
    assert nb == 4 and prefix == int(ordered_bits(np.zeros(1, np.float32))[0])
