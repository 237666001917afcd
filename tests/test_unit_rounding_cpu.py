"""The byte rounding of the float blend modes and gradient paints
(pixie_gb300/csrc/pxg_device.cuh unit_to_u8): round(w) half away from zero
equals floor(w + 0.5) with the sum rounded toward zero, for every float32 w in
(0, 255] -- checked exhaustively here (about 1.13e9 values), with the sum
formed exactly in float64 and rounded toward zero to float32."""
import numpy as np


def test_round_half_away_equals_floor_of_sum_toward_zero():
    lo, hi = 1, int(np.float32(255.0).view(np.uint32)) + 1
    step = 1 << 24
    for a in range(lo, hi, step):
        w = np.arange(a, min(a + step, hi), dtype=np.uint32).view(np.float32)
        s = w.astype(np.float64) + 0.5                       # exact
        f = s.astype(np.float32)                             # to nearest
        f = np.where(f.astype(np.float64) > s, np.nextafter(f, np.float32(0)), f)  # toward zero
        want = np.floor(w.astype(np.float64) + 0.5)          # half away from zero (w > 0)
        bad = np.flatnonzero(np.floor(f) != want)
        assert bad.size == 0, f"w = {w[bad[:5]]}"
