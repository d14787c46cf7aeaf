"""Seeded procedural scene: the height field and spheres in numpy.

The device generator (csrc/hd_scene.cu) voxelises the same integer function;
this host copy serves workload generation (surface points for edit centres,
camera framing).  Solid voxels: {y <= height(x, z)} united with 64 spheres.

height(x, z) = E/2 + floor(E * total / (31 * 16384)) where
total = sum over 5 octaves o of (value_noise_o(x, z) >> o) in Q16, each
octave a lattice of period E/4 >> o with values hashed from (seed, o, i, j)
and smoothstep-weighted bilinear interpolation.  All integer arithmetic.
"""
import numpy as np

_M64 = (1 << 64) - 1
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + _GOLD
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _lattice(seed, octave, i, j):
    k = (np.uint64(octave) << np.uint64(58)) ^ (i.astype(np.uint64) << np.uint64(29)) ^ j.astype(np.uint64)
    k = _mix64(np.uint64(seed) ^ _mix64(k))
    return (k >> np.uint64(47)).astype(np.int64) - 65536


def _smooth(t):
    return (t * t * (3 * 65536 - 2 * t)) >> 32


def height(seed, depth, x, z):
    """Vectorised height of columns (x, z) (arrays of equal shape)."""
    x = np.asarray(x, dtype=np.int64)
    z = np.asarray(z, dtype=np.int64)
    total = np.zeros(np.broadcast(x, z).shape, np.int64)
    for o in range(5):
        lp = depth - 2 - o
        i, j = x >> lp, z >> lp
        fx, fz = x & ((1 << lp) - 1), z & ((1 << lp) - 1)
        sx = _smooth((fx << 16) >> lp)
        sz = _smooth((fz << 16) >> lp)
        v00, v10 = _lattice(seed, o, i, j), _lattice(seed, o, i + 1, j)
        v01, v11 = _lattice(seed, o, i, j + 1), _lattice(seed, o, i + 1, j + 1)
        a = v00 + (((v10 - v00) * sx) >> 16)
        b = v01 + (((v11 - v01) * sx) >> 16)
        n = a + (((b - a) * sz) >> 16)
        total += n >> o
    e = 1 << depth
    return (e >> 1) + np.floor_divide(total * e, 31 * 16384)


def spheres(seed, depth):
    """64 x (cx, cy, cz, r) int64."""
    state = (seed ^ 0x5EED5EED12345678) & _M64
    mask = (1 << depth) - 1
    out = np.zeros((64, 4), np.int64)
    for s in range(64):
        vals = []
        for _ in range(4):
            state = (state + 0x9E3779B97F4A7C15) & _M64
            vals.append(int(_mix64(np.uint64(state))))
        out[s] = (vals[0] & mask, vals[1] & mask, vals[2] & mask, 8 + vals[3] % 57)
    return out


def solid(seed, depth, x, y, z):
    x, y, z = (np.asarray(v, dtype=np.int64) for v in (x, y, z))
    res = y <= height(seed, depth, x, z)
    for cx, cy, cz, r in spheres(seed, depth):
        res |= (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= r * r
    return res


def surface_points(seed, depth, n, rng):
    """n surface voxels of the height field: (x, height(x, z), z)."""
    e = 1 << depth
    x = rng.integers(0, e, n)
    z = rng.integers(0, e, n)
    y = np.minimum(height(seed, depth, x, z), e - 1)
    return np.stack([x, y, z], axis=1)
