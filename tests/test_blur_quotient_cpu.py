"""The blur's quantisation between and after its passes, (S div 256) div 255 =
floor(S / 65280), as the kernels compute it (smallblur.cu, ringblur.cu): one
fused multiply-add rounding toward minus infinity, S * C + 1.5 * 2^23, with
C = 1/65280 rounded up to float32, whose low mantissa bits are then the
quotient.  For S < 2^24 the sum lies in [1.5 * 2^23, 2^24), where float32
steps are 1, so rounding down takes floor(S * C) exactly; this checks that
floor(S * C) = floor(S / 65280) for every S < 2^24 (S * C is exact in
float64).  The ring passes multiply S * 2^-24 by C * 2^24, the same product."""
import numpy as np


def test_constant_is_1_over_65280_rounded_up():
    c = np.float32(float.fromhex("0x1.010102p-16"))
    assert float(c) >= 1 / 65280 and float(np.nextafter(c, np.float32(0))) < 1 / 65280
    assert np.float32(257.00394) == np.float32(float(c) * 2.0 ** 24)  # the ring passes' C * 2^24


def test_floor_of_s_times_c_is_the_quotient_for_every_s():
    c = float(np.float32(float.fromhex("0x1.010102p-16")))
    step = 1 << 22
    for a in range(0, 1 << 24, step):
        s = np.arange(a, a + step, dtype=np.int64)
        got = np.floor(s.astype(np.float64) * c).astype(np.int64)
        bad = np.flatnonzero(got != s // 65280)
        assert bad.size == 0, f"S = {s[bad[:5]]}"
