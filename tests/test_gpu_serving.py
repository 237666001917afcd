"""The continuous-batching render server: every job's canvas is bit-exact
with the oracle, and the same whether the job is served alone or in a mix
of concurrently admitted jobs (different chunking, admission order and
memory pressure)."""
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


def record(items):
    sc = px.Scene()
    for it in items:
        paint = px.Paint(it["color"], 1.0, it["blend"])
        try:
            if it["kind"] == "fill":
                sc.fill_path(it["cmds"], paint, None, it["winding"])
            else:
                sc.stroke_path(it["cmds"], paint, None, it["width"], it["cap"], it["join"], it["miter"])
        except px.PixieError:
            pass  # the reference raises for this path too; a caller skips it
    return sc


def oracle_job(job):
    s = job["side"]
    ref = pxo.new_image(s, s)
    for it in job["items"]:
        try:
            if it["kind"] == "fill":
                pxo.fill_path(ref, it["cmds"], it["color"], 1.0, it["blend"], None, it["winding"])
            else:
                pxo.stroke_path(ref, it["cmds"], it["color"], 1.0, it["blend"], None, it["width"],
                                it["cap"], it["join"], it["miter"])
        except pxo.OracleError:
            pass
    if job["blur"]:
        pxo.blur(ref, job["blur"])
    return ref


def serve(jobs, scenes, budget, per_job, per_step, order=None):
    sv = px.Server(budget, per_job, per_step)
    ids = {}
    for k in (order if order is not None else range(len(jobs))):
        ids[sv.submit(scenes[k], jobs[k]["side"], jobs[k]["side"], jobs[k]["blur"])] = k
    out = {}
    guard = 0
    while sv.pending() > 0:
        sv.step()
        for jid in sv.poll():
            out[ids[jid]] = sv.take(jid)[0]
        guard += 1
        assert guard < 100000
    for jid in sv.poll():
        out[ids[jid]] = sv.take(jid)[0]
    return out, sv.stats()


def small_jobs(n, seed=3):
    return [wl.serving_job(seed * 1000 + i, min_side=64, max_side=320, min_paths=5, max_paths=120,
                           blur_share=0.4) for i in range(n)]


def test_served_jobs_match_oracle():
    jobs = small_jobs(10)
    assert any(j["blur"] for j in jobs) and any(not j["blur"] for j in jobs)
    scenes = [record(j["items"]) for j in jobs]
    out, st = serve(jobs, scenes, 1 << 30, 16, 64)
    assert st["peak_admitted"] > 1  # jobs really ran side by side
    for k, j in enumerate(jobs):
        ref = oracle_job(j)
        d = np.abs(out[k].astype(np.int32) - ref.astype(np.int32))
        assert int(d.max()) == 0, f"job {k}: max|delta|={int(d.max())} differing px={int((d.max(axis=2) > 0).sum())}"


def test_alone_equals_in_mix():
    jobs = small_jobs(16, seed=5)
    scenes = [record(j["items"]) for j in jobs]
    alone = {}
    for k in range(len(jobs)):
        o, _ = serve([jobs[k]], [scenes[k]], 1 << 30, 1 << 20, 1 << 20)
        alone[k] = o[0]
    # the mix: small chunks, reversed arrival order, a budget that admits
    # only a few canvases at a time
    mix, st = serve(jobs, scenes, 3 * 320 * 320 * 8, 7, 40, order=list(reversed(range(len(jobs)))))
    assert st["peak_admitted"] >= 2
    assert st["peak_bytes"] <= 3 * 320 * 320 * 8
    for k in range(len(jobs)):
        assert np.array_equal(alone[k], mix[k]), f"job {k} differs alone vs in the mix"


def test_budget_rejects_oversized_job_and_errors_surface():
    sv = px.Server(1000, 8, 8)
    with pytest.raises(px.PixieError, match="budget"):
        sv.submit(px.Scene(), 64, 64)
    sv = px.Server(1 << 28, 8, 8)
    sc = px.Scene()
    sc.fill_path(np.zeros(0, np.float32), [1, 0, 0, 1])  # raises "Path int overflow detected" when drawn
    jid = sv.submit(sc, 32, 32)
    while sv.pending():
        sv.step()
    assert sv.poll() == [jid]
    with pytest.raises(px.PixieError, match="Path int overflow detected"):
        sv.take(jid)
