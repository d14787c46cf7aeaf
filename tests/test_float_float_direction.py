"""The traversal kernels normalise a camera ray's double vector v without
double arithmetic (dir_from_vec in hd_trace.cu): v split into float pairs,
|v|^2 summed exactly with its remainders, an rsqrtf seed refined once in
float and once in float-float, each component formed as P + L, and the
float nearest to P + L kept only when P + L lies more than 2^-40 |P + L|
from a float rounding midpoint (otherwise the exact double path runs).

This restates that computation in numpy, operation for operation (float32
arithmetic rounds to nearest; fused multiply-adds are formed exactly from
float64 products and a two-sum), with rsqrtf seeds up to 4 ulps off, and
checks the two claims the kernels rely on: P + L lies within 2^-43 of the
exact v / |v| (80-bit long double), and every accepted component equals the
reference's float((1.0 / sqrt(dot)) * v) with every double operation
rounded on its own.  (The reference's fused form differs from that double
by a few double ulps, far inside the 2^-40 margin; the GPU tests compare
both arithmetic modes on whole frames.)
"""
import numpy as np
import pytest

F = np.float32


def _round_f32_of_sum(s, err):
    """float32 nearest to s + err (s a double, |err| <= ulp(s) / 2)."""
    r = s.astype(F)
    rd = r.astype(np.float64)
    hi = np.nextafter(r, F(np.inf)).astype(np.float64)
    lo = np.nextafter(r, F(-np.inf)).astype(np.float64)
    up = (s == (rd + hi) / 2) & (err > 0) & (rd < s)
    dn = (s == (rd + lo) / 2) & (err < 0) & (rd > s)
    r = np.where(up, np.nextafter(r, F(np.inf)), r)
    r = np.where(dn, np.nextafter(r, F(-np.inf)), r)
    return r


def fma32(a, b, c):
    p = a.astype(np.float64) * b.astype(np.float64)
    cc = c.astype(np.float64)
    s = p + cc
    bb = s - p
    err = (p - (s - bb)) + (cc - bb)
    return _round_f32_of_sum(s, err)


def split_f64(v):
    b = v.view(np.uint64)
    sign = ((b >> np.uint64(32)) & np.uint64(0x80000000)).astype(np.uint32)
    mag = b & np.uint64(0x7FFFFFFFFFFFFFFF)
    e = (mag >> np.uint64(52)).astype(np.int64) - 1023
    ok = (mag == 0) | ((e >= -40) & (e < 40))
    ee = np.clip(e, -40, 39)
    hi_bits = sign | ((ee + 127).astype(np.uint32) << np.uint32(23)) | ((mag >> np.uint64(29)).astype(np.uint32) & np.uint32(0x7FFFFF))
    hi = np.where(mag == 0, sign.view(F), hi_bits.view(F))
    scale = (sign | ((ee - 52 + 127).astype(np.uint32) << np.uint32(23))).view(F)
    rem = (mag & np.uint64((1 << 29) - 1)).astype(F)  # exact int -> float rounding (numpy rounds to nearest)
    lo = np.where(mag == 0, F(0), rem * scale)
    return hi, lo, ok


def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def round_pair(P, L):
    R = P + L
    r = L - (R - P)
    rb = R.view(np.uint32)
    ex = (rb >> np.uint32(23)) & np.uint32(0xFF)
    ok = (ex >= 64) & (ex <= 190)
    exc = np.clip(ex, 64, 190)
    half_up = ((exc - 24) << np.uint32(23)).view(F)
    half_dn = np.where((rb & np.uint32(0x7FFFFF)) != 0, half_up, ((exc - 25) << np.uint32(23)).view(F))
    margin = ((exc - 39) << np.uint32(23)).view(F)
    s = np.where((rb >> np.uint32(31)) != 0, -r, r)
    ok &= ((half_up - s) > margin) & ((half_dn + s) > margin)
    return R, ok


def dir_from_vec(v, seed_ulps, rng):
    """(d [n, 3] float32, P + L as float64 pairs [n, 3, 2], accepted [n])."""
    h, l, ok = zip(*(split_f64(v[:, a]) for a in range(3)))
    ok = ok[0] & ok[1] & ok[2]
    with np.errstate(all="ignore"):
        p = [h[a] * h[a] for a in range(3)]
        e = (fma32(h[0], h[0], -p[0]) + fma32(h[1], h[1], -p[1])) + fma32(h[2], h[2], -p[2])
        c = ((h[0] + h[0]) * l[0] + (h[1] + h[1]) * l[1]) + (h[2] + h[2]) * l[2]
        s1, t1 = two_sum(p[0], p[1])
        S, t2 = two_sum(s1, p[2])
        Slo = ((t1 + t2) + e) + c
        ok &= S >= F(2.0 ** -80)
        x0 = S + Slo
        q0 = (1.0 / np.sqrt(x0.astype(np.float64))).astype(F)
        k = rng.integers(-seed_ulps, seed_ulps + 1, size=q0.size)
        for step in range(seed_ulps):
            q0 = np.where(k > step, np.nextafter(q0, F(np.inf)), q0)
            q0 = np.where(-k > step, np.nextafter(q0, F(0)), q0)
        xq = x0 * q0
        r0 = fma32(q0 * fma32(-xq, q0, np.full_like(q0, 1)), np.full_like(q0, 0.5), q0)
        A = S * r0
        Al = fma32(S, r0, -A)
        hh = fma32(-A, r0, np.full_like(r0, 1)) - fma32(Al, r0, (Slo * r0) * r0)
        corr = (r0 * hh) * F(0.5)
        d = np.zeros((v.shape[0], 3), F)
        pl = np.zeros((v.shape[0], 3, 2))
        for a in range(3):
            P = r0 * h[a]
            Pl = fma32(r0, h[a], -P)
            L = Pl + (r0 * l[a] + (corr * h[a] + corr * l[a]))
            R, ok_a = round_pair(P, L)
            zero = h[a] == 0
            d[:, a] = np.where(zero, h[a], R)
            ok &= ok_a | zero
            pl[:, a, 0], pl[:, a, 1] = np.where(zero, 0, P), np.where(zero, 0, L)
    return d, pl, ok


def _vectors(rng, n):
    kinds = rng.integers(0, 4, size=n)
    u = rng.random((n, 3)) * 2 - 1
    scale = np.ldexp(1.0, rng.integers(-20, 20, size=(n, 3)))
    pos = 16384.0 * rng.random((n, 3))
    canc = (pos + u) - pos  # a screen point minus a camera position far from the origin
    axis = np.column_stack([np.ones(n), u[:, 1] * 1e-3, u[:, 2] * 1e-3])
    v = np.where(kinds[:, None] == 0, u, np.where(kinds[:, None] == 1, u * scale, np.where(kinds[:, None] == 2, canc, axis)))
    zero = rng.random(n) < 1 / 64
    v[zero, rng.integers(0, 3, size=int(zero.sum()))] = 0.0
    return v


@pytest.mark.parametrize("seed_ulps", [2, 4])
def test_float_float_direction_matches_reference_rounding(seed_ulps):
    rng = np.random.default_rng(11 + seed_ulps)
    v = _vectors(rng, 1_000_000)
    d, pl, ok = dir_from_vec(v, seed_ulps, rng)
    assert ok.mean() > 0.999
    # the error bound of P + L against the exact direction
    ld = v.astype(np.longdouble)
    exact = ld / np.sqrt((ld * ld).sum(axis=1, keepdims=True))
    approx = pl[:, :, 0].astype(np.longdouble) + pl[:, :, 1].astype(np.longdouble)
    nz = (v != 0) & ok[:, None]
    rel = np.abs(approx[nz] - exact[nz]) / np.abs(exact[nz])
    assert float(rel.max()) < 2.0 ** -43
    # accepted components are the reference's floats (double operations rounded one by one)
    dot0 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    ref0 = ((1.0 / np.sqrt(dot0))[:, None] * v).astype(F)
    assert np.array_equal(d[ok].view(np.uint32), ref0[ok].view(np.uint32))
