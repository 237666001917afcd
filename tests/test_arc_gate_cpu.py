"""The gate for flattening arcs on the GPU.

pixie's addArc (src/pixie/paths.nim:764-884) calls the C library's float32
sin/cos at every step, and the step decisions depend on the exact floats.  A
GPU arc path would need its own sin/cos giving the C library's result for
every angle the stepping visits.  The best an in-house function can be is
correctly rounded; this test measures how often the C library's sinf/cosf
differ from the correctly rounded values on angles of the arc stepping's
range (theta + delta * t, |a| <= 3 pi).  On glibc 2.39 the rate is about
1.4 %, so no in-house sin/cos can pass the zero-disagreement gate and arcs
stay flattened on the host with the C library's sinf/cosf (host_geom.cpp),
as the reference does.
"""
import numpy as np

from oracle import pxo


def test_libm_sincosf_against_correct_rounding():
    rng = np.random.default_rng(1234)
    x = rng.uniform(-3 * np.pi, 3 * np.pi, 1_000_000).astype(np.float32)
    s, c = pxo.libm_sincosf(x)
    xd = x.astype(np.float64)
    # float64 sin/cos rounded to float32: correctly rounded except within
    # ~2^-29 ulp of a float32 midpoint, far rarer than the rate measured here
    s_cr, c_cr = np.sin(xd).astype(np.float32), np.cos(xd).astype(np.float32)
    rate = (np.count_nonzero(s != s_cr) + np.count_nonzero(c != c_cr)) / (2 * x.size)
    ulps = np.abs(s.view(np.int32).astype(np.int64) - s_cr.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1  # the C library is within one ulp ...
    assert rate > 0  # ... but not correctly rounded: the gate stays closed
