"""Kernels launched without waiting for the kernel before them (buffers
disjoint from every kernel still running, composite.cu dep_late) against the
oracle: long random sequences of draws, blurs of every kernel family, shadows
and fills over a small pool of images, enqueued in non-blocking mode so that
consecutive launches overlap, with images reused as destination, source and
blur input in every order.  A missed hazard shows as a differing byte."""
import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)
    px.blur_config(3)
    yield
    px.set_blocking(True)


MODES = list(range(20))
SCALE = [0.4, 0.0, 0.0, 0.0, 0.4, 0.0, 0.0, 0.0, 1.0]  # the 512-px paths onto the small images
RADII = [1, 2, 4, 9, 16, 33]


def run_sequence(seed, n_ops, w=256, h=192, n_img=5):
    rng = np.random.default_rng(seed)
    host = [wl.premultiplied_image(seed * 31 + k, w, h) for k in range(n_img)]
    ref = [x.copy() for x in host]
    gpu = [px.Image.from_numpy(x) for x in host]
    ops = []
    for _ in range(n_ops):
        kind = rng.choice(["draw", "draw", "draw", "blur", "shadow", "fill"])
        i, j = (int(v) for v in rng.choice(n_img, 2, replace=False))
        if kind == "draw":
            ops.append(("draw", i, j, int(rng.choice(MODES))))
        elif kind == "blur":
            ops.append(("blur", i, int(rng.choice(RADII))))
        elif kind == "shadow":
            ops.append(("shadow", i, j, (int(rng.integers(-9, 9)), int(rng.integers(-9, 9))),
                        int(rng.integers(0, 5)), int(rng.integers(0, 13))))
        else:
            ops.append(("fill", i, wl.plain_path(int(rng.integers(1, 1000)))))
    px.set_blocking(False)
    try:
        for op in ops:
            if op[0] == "draw":
                gpu[op[1]].draw(gpu[op[2]], (0, 0), op[3])
            elif op[0] == "blur":
                gpu[op[1]].blur(op[2])
            elif op[0] == "shadow":
                gpu[op[1]].shadow_into(gpu[op[2]], op[3], op[4], op[5], [0.1, 0.2, 0.3, 0.9])
            else:
                gpu[op[1]].fill_path(op[2], [0.9, 0.4, 0.1, 0.7], SCALE)
        px.synchronize()
    finally:
        px.set_blocking(True)
    for op in ops:
        if op[0] == "draw":
            pxo.draw(ref[op[1]], ref[op[2]], 0, 0, op[3])
        elif op[0] == "blur":
            pxo.blur(ref[op[1]], op[2])
        elif op[0] == "shadow":
            ref[op[2]][...] = pxo.shadow(ref[op[1]], op[3][0], op[3][1], op[4], op[5], [0.1, 0.2, 0.3, 0.9])
        else:
            pxo.fill_path(ref[op[1]], op[2], [0.9, 0.4, 0.1, 0.7], 1.0, 0, SCALE)
    return gpu, ref, ops


@pytest.mark.parametrize("seed", range(6))
def test_random_sequences_match_the_oracle(seed):
    gpu, ref, ops = run_sequence(seed, 80)
    for k, (g, r) in enumerate(zip(gpu, ref)):
        got = g.to_numpy()
        bad = int((got != r).any(axis=2).sum())
        assert bad == 0, f"seed {seed}: image {k} differs in {bad} px after {len(ops)} ops"


def test_independent_draws_overlap_and_chain_correctly():
    """A chain where each draw's source is the previous draw's destination
    (every launch must wait) interleaved with independent draws (which may
    not): the result is the oracle's."""
    n = 12
    host = [wl.premultiplied_image(500 + k, 512, 256) for k in range(n)]
    ref = [x.copy() for x in host]
    gpu = [px.Image.from_numpy(x) for x in host]
    px.set_blocking(False)
    try:
        for k in range(1, n):
            gpu[k].draw(gpu[k - 1], (0, 0), k % 20)           # depends on the draw before
            gpu[(k + 5) % n].draw(gpu[(k + 7) % n], (0, 0), 0)  # may overlap it
        px.synchronize()
    finally:
        px.set_blocking(True)
    for k in range(1, n):
        pxo.draw(ref[k], ref[k - 1], 0, 0, k % 20)
        pxo.draw(ref[(k + 5) % n], ref[(k + 7) % n], 0, 0, 0)
    for k in range(n):
        assert np.array_equal(gpu[k].to_numpy(), ref[k]), f"image {k}"
