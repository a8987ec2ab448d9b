"""The continuous-batching request server.

Requests are submitted while others run; each result must equal the same
request run alone, bit for bit (same arithmetic, same stochastic-rounding
bits), requests must join the batch while others are in flight, and bad
requests must be refused at submission.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REQS = [  # edge, tau, u0, steps, precision name
    (48, 0.004, 0.05, 600, "f32"),      # still running when the others arrive
    (16, 0.004, 0.05, 37, "f32"),
    (24, 0.02, 0.06, 25, "f16dev"),
    (32, 0.0007, 0.04, 60, "f32"),
    (16, 0.01, 0.07, 9, "f16dev"),
    (8, 0.1, 0.03, 50, "f32"),
    (20, 0.003, 0.05, 44, "f16dev"),
    (12, 0.05, 0.05, 0, "f32"),
    (28, 0.002, 0.08, 31, "f32"),
]


def prec(imex, name):
    return {"f32": imex.IMEX_F32, "f16dev": imex.IMEX_F16DEV}[name]


def alone(imex, r):
    edge, tau, u0, steps, pname = r
    with imex.LBM(edge, edge, edge, tau, 1.0, u0, precision=prec(imex, pname)) as lat:
        lat.Initialize()
        lat.step(steps)
        return lat.Conserved()


def test_results_equal_alone_and_requests_overlap(imex):
    with imex.Server(budget_bytes=2e9, max_active=4, steps_per_tick=7) as srv:
        for i, r in enumerate(REQS):
            edge, tau, u0, steps, pname = r
            srv.submit(edge, edge, edge, tau, u0, steps, prec(imex, pname), tag=i)
            time.sleep(0.002)
        got = {}
        t0 = time.time()
        while len(got) < len(REQS) and time.time() - t0 < 120:
            for res in srv.poll():
                got[res["tag"]] = res
            time.sleep(0.01)
        st = srv.stats()
    assert len(got) == len(REQS) and st["failed"] == 0
    for i, r in enumerate(REQS):
        res = got[i]
        assert res["status"] == 0, res
        assert res["steps"] == r[3]
        assert res["t_submit"] <= res["t_admit"] <= res["t_done"]
        assert res["conserved"] == alone(imex, r), i
    # continuous batching: requests were admitted while the first one ran,
    # and finished before it
    first = got[0]
    joined = [i for i in got if i and first["t_admit"] < got[i]["t_admit"] < first["t_done"]]
    assert joined and any(got[i]["t_done"] < first["t_done"] for i in joined)
    assert st["completed"] == len(REQS) and st["cell_updates"] > 0


def test_budget_and_slots_queue_requests(imex):
    """With one slot, requests run one after another in arrival order."""
    with imex.Server(budget_bytes=1e9, max_active=1, steps_per_tick=5) as srv:
        for i in range(3):
            srv.submit(16, 16, 16, 0.01, 0.05, 12, imex.IMEX_F32, tag=i)
        got = []
        t0 = time.time()
        while len(got) < 3 and time.time() - t0 < 60:
            got += srv.poll()
            time.sleep(0.01)
    got.sort(key=lambda r: r["tag"])
    assert [r["status"] for r in got] == [0, 0, 0]
    for a, b in zip(got, got[1:]):
        assert b["t_admit"] >= a["t_done"] - 1e-6


def test_bad_requests_refused(imex):
    with imex.Server(budget_bytes=1e8, max_active=2, steps_per_tick=5) as srv:
        with pytest.raises(imex.ImexError):
            srv.submit(8, 8, 8, 0.01, 0.05, 5, imex.IMEX_F64)      # float64 is not batched
        with pytest.raises(imex.ImexError):
            srv.submit(256, 256, 256, 0.01, 0.05, 5, imex.IMEX_F32)  # larger than the budget
        with pytest.raises(imex.ImexError):
            srv.submit(0, 8, 8, 0.01, 0.05, 5, imex.IMEX_F32)


def test_diverging_request_reports_nonfinite(imex):
    """A solve that blows up (BGK at tau near 0 on a coarse grid at Mach 0.3)
    still runs its steps and returns its diagnostics with IMEX_ERR_NONFINITE;
    the server and the other requests carry on."""
    with imex.Server(budget_bytes=1e9, max_active=4, steps_per_tick=10) as srv:
        srv.submit(16, 16, 16, 1e-5, 0.3, 400, imex.IMEX_F32, tag=1)
        srv.submit(16, 16, 16, 0.01, 0.05, 30, imex.IMEX_F32, tag=2)
        got = {}
        t0 = time.time()
        while len(got) < 2 and time.time() - t0 < 60:
            for r in srv.poll():
                got[r["tag"]] = r
            time.sleep(0.01)
        assert srv.stats()["failed"] == 0
    assert got[1]["status"] == imex.IMEX_ERR_NONFINITE
    assert not np.all(np.isfinite(got[1]["conserved"]))
    assert got[1]["steps"] == 400
    assert got[2]["status"] == 0


def test_pause_and_resume_across_requests(imex, tmp_path):
    """A solve saved at step 30 and resumed by a later request to step 70
    ends where a single 70-step solve ends, bit for bit (stochastic
    rounding included: the saved step count seeds the random bits)."""
    ck = str(tmp_path / "req.ckpt")
    for pname in ("f32", "f16dev"):
        p = prec(imex, pname)
        with imex.Server(budget_bytes=1e9, max_active=4, steps_per_tick=8) as srv:
            srv.submit(20, 16, 24, 0.003, 0.06, 30, p, tag=1, save_path=ck)
            first = _wait(srv, 1)
            srv.submit(20, 16, 24, 0.003, 0.06, 70, p, tag=2, resume_path=ck)
            srv.submit(20, 16, 24, 0.003, 0.06, 70, p, tag=3)
            rest = _wait(srv, 2)
        assert first[1]["status"] == 0 and first[1]["steps"] == 30
        assert rest[2]["status"] == 0 and rest[2]["steps"] == 70
        assert rest[2]["conserved"] == rest[3]["conserved"]
        with imex.LBM(20, 16, 24, 0.003, 1.0, 0.06, precision=p) as lat:
            lat.checkpoint_load(ck)
            assert lat.steps_done() == 30


def test_resume_from_missing_file_fails_that_request(imex, tmp_path):
    with imex.Server(budget_bytes=1e9, max_active=2, steps_per_tick=5) as srv:
        srv.submit(8, 8, 8, 0.01, 0.05, 10, imex.IMEX_F32, tag=1, resume_path=str(tmp_path / "nope"))
        srv.submit(8, 8, 8, 0.01, 0.05, 10, imex.IMEX_F32, tag=2)
        got = _wait(srv, 2)
        assert srv.stats()["failed"] == 0
    assert got[1]["status"] == imex.IMEX_ERR_IO
    assert got[2]["status"] == 0


def _wait(srv, n, timeout=60):
    got = {}
    t0 = time.time()
    while len(got) < n and time.time() - t0 < timeout:
        for r in srv.poll():
            got[r["tag"]] = r
        time.sleep(0.01)
    assert len(got) == n
    return got


def test_least_work_policy_admits_small_requests_first(imex):
    with imex.Server(budget_bytes=2e9, max_active=1, steps_per_tick=10) as srv:
        srv.set_policy(imex.IMEX_POLICY_LEAST_WORK)
        srv.submit(96, 96, 96, 0.004, 0.05, 3000, imex.IMEX_F32, tag=1)  # running while the others queue
        time.sleep(0.02)
        srv.submit(32, 32, 32, 0.004, 0.05, 200, imex.IMEX_F32, tag=2)   # more work
        srv.submit(16, 16, 16, 0.004, 0.05, 20, imex.IMEX_F32, tag=3)    # least work, arrives last
        got = _wait(srv, 3)
    assert all(r["status"] == 0 for r in got.values())
    assert got[3]["t_admit"] < got[2]["t_admit"]
    with pytest.raises(imex.ImexError):
        imex.Server(budget_bytes=1e8, max_active=1, steps_per_tick=5).set_policy(7)


def test_results_survive_retunes_as_the_batch_grows_and_shrinks(imex):
    """Large float16 requests joining a running float32 / float16 pair
    multiply the batch's cells, so the server re-tunes its launch shapes
    (and again when they leave); a re-tune times the row kernel switched
    off, which outgrows the segment kernel's group table.  The tick's
    captured graph must follow, and every result equal the request alone."""
    reqs = [(16, 0.004, 0.05, 300, "f32"), (32, 0.02, 0.06, 300, "f16dev"),
            (96, 0.01, 0.07, 40, "f16dev"), (80, 0.003, 0.05, 35, "f16dev"), (24, 0.002, 0.08, 30, "f32")]
    with imex.Server(budget_bytes=4e9, max_active=8, steps_per_tick=5) as srv:
        got = {}
        for i, r in enumerate(reqs):
            edge, tau, u0, steps, pname = r
            srv.submit(edge, edge, edge, tau, u0, steps, prec(imex, pname), tag=i)
            if i == 1:  # let the first two run (tuned, graph captured) before the large ones arrive
                t0 = time.time()
                while srv.stats()["ticks"] < 3 and time.time() - t0 < 60:
                    time.sleep(0.005)
        t0 = time.time()
        while len(got) < len(reqs) and time.time() - t0 < 120:
            for res in srv.poll():
                got[res["tag"]] = res
            time.sleep(0.01)
        st = srv.stats()
    assert len(got) == len(reqs) and st["failed"] == 0
    for i, r in enumerate(reqs):
        assert got[i]["status"] == 0, got[i]
        assert got[i]["conserved"] == alone(imex, r), i
