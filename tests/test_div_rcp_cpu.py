"""The float blend modes divide by one correctly rounded reciprocal per
denominator with two Newton-Raphson correction steps (pixie_gb300/csrc/
pxg_device.cuh div_rcp): y = RN(1/d), q0 = RN(n*y), q1 = RN(q0 + RN(n - q0*d)*y),
r1 = n - q1*d (exact), result RN(q1 + r1*y).  Checked here against the
correctly rounded float32 quotient RN(n/d) on the operands those divisions
see -- every output alpha of the composite (d = as + ab*(1-as) for all 65536
byte pairs) against random numerators, and random clipColor-like operands --
and checked that r1 is exact (the hypothesis of Markstein's theorem, which
makes the last step correctly rounded).

Every float32 step is emulated exactly in float64: a product of two float32
values is exact; a fused multiply-add n - q*d is exact in float64 (q*d is
within a few ulps of n), so converting it to float32 rounds it once; 1/d and
n/d rounded to float64 are never float32 midpoints unless exactly (a float32
midpoint has 25 significant bits, and |M/N - a/2^25| is 0 or at least 2^-49
for 24-bit integers M, N), so rounding them to float64 first changes nothing;
and q + r*y is rounded by choosing, among q's float32 neighbours, the one
nearest to it, with differences that are exact in float64."""
import numpy as np

F32 = np.float32


def rn_sum(q, t):
    """RN32(q + t) for float32 q and float64 t with |t| at most a few ulps of q,
    ties to even."""
    q64 = q.astype(np.float64)
    cands = [q]
    lo = hi = q
    for _ in range(3):
        lo = np.nextafter(lo, F32(-np.inf))
        hi = np.nextafter(hi, F32(np.inf))
        cands = [lo] + cands + [hi]
    best = None
    best_err = None
    for c in cands:
        err = np.abs((c.astype(np.float64) - q64) - t)  # exact: all terms are a few ulps of q
        if best is None:
            best, best_err = c.copy(), err
            continue
        even = (c.view(np.uint32) & 1) == 0
        take = (err < best_err) | ((err == best_err) & even)
        best = np.where(take, c, best)
        best_err = np.where(take, err, best_err)
    return best


def div_rcp(n, d):
    n64, d64 = n.astype(np.float64), d.astype(np.float64)
    y = (1.0 / d64).astype(F32)                           # RN32(1/d)
    y64 = y.astype(np.float64)
    q0 = (n64 * y64).astype(F32)                          # RN32(n*y): the product is exact in float64
    r0 = (n64 - q0.astype(np.float64) * d64).astype(F32)  # fma(-q0, d, n), rounded once
    q1 = rn_sum(q0, r0.astype(np.float64) * y64)          # fma(r0, y, q0)
    r1x = n64 - q1.astype(np.float64) * d64
    r1 = r1x.astype(F32)                                  # fma(-q1, d, n)
    assert np.all(r1.astype(np.float64) == r1x), "the second remainder must be exact"
    return rn_sum(q1, r1.astype(np.float64) * y64)        # fma(r1, y, q1)


def check(n, d):
    got = div_rcp(n, d)
    want = (n.astype(np.float64) / d.astype(np.float64)).astype(F32)  # RN32(n/d)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, f"n={n[bad[:3]]!r} d={d[bad[:3]]!r}: {got[bad[:3]]!r} != {want[bad[:3]]!r}"


def test_composite_alpha_denominators():
    u = (np.arange(256, dtype=F32) / F32(255)).astype(F32)  # v / 255.0f
    a_s, a_b = np.meshgrid(u, u, indexing="ij")
    ao = (a_s + a_b * (F32(1) - a_s)).astype(F32).ravel()
    ao = ao[ao > 0]
    rng = np.random.default_rng(7)
    for _ in range(16):
        n = (rng.random(ao.size, dtype=np.float32) * ao * F32(1.01)).astype(F32)
        check(n, ao)


def test_clip_color_like_operands():
    rng = np.random.default_rng(11)
    for _ in range(20):
        d = rng.uniform(1e-6, 2.0, 1 << 20).astype(F32)
        n = (rng.uniform(-2.0, 2.0, 1 << 20) * rng.uniform(0.0, 1.0, 1 << 20)).astype(F32)
        check(n, d)
