"""The traversal kernels take a ray's inverse direction as the correctly
rounded float reciprocal (one rounding) where the reference rounds the
double quotient 1.0 / double(x) to float (two roundings).  The two agree
for every float x by the double-rounding theorem (a 53-bit intermediate is
at least 2 * 24 + 2 bits).  This checks the claim exhaustively over the
significands of three exponent ranges and over random bit patterns,
subnormals and the overflow edge included; numpy's float32 division rounds
to nearest as IEEE 754 asks.
"""
import numpy as np


def _agree(x):
    x = x[np.isfinite(x) & (x != 0)]
    with np.errstate(over="ignore"):  # reciprocals of tiny subnormals overflow to inf in both
        one = (np.float32(1) / x).view(np.uint32)
        two = (1.0 / x.astype(np.float64)).astype(np.float32).view(np.uint32)
    bad = np.nonzero(one != two)[0]
    assert bad.size == 0, f"{bad.size} mismatches, first x = {x[bad[0]]!r}"
    return x.size


def test_every_significand_of_three_binades():
    sig = np.arange(1 << 23, dtype=np.uint32)
    n = 0
    for exp in (127, 100, 1):  # [1, 2), [2^-27, 2^-26), the smallest normal binade
        n += _agree(((np.uint32(exp) << np.uint32(23)) | sig).view(np.float32))
    assert n == 3 << 23


def test_random_bit_patterns_subnormals_and_edges():
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 1 << 32, size=4_000_000, dtype=np.uint64).astype(np.uint32)
    sub = rng.integers(1, 1 << 23, size=1_000_000, dtype=np.uint64).astype(np.uint32)
    edges = np.array([0x00000001, 0x007FFFFF, 0x00800000, 0x00200000, 0x00200001, 0x001FFFFF,
                      0x3F800000, 0x3F800001, 0x7F7FFFFF, 0x3F7FFFFF], dtype=np.uint32)
    for b in (bits, sub, edges, edges | np.uint32(0x80000000)):
        _agree(b.view(np.float32))
