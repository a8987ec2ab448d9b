"""The synthetic workloads of the batched and served measurements match
their stated configurations (host logic only, no GPU).

Batched: 64 cubic lattices, edges uniform over {32, 48, 64, 96, 128}, Re
uniform in [100, 3200] cast to int, u0 uniform in [0.02, 0.08], phase
offsets in [0, 2 pi)^3, seeded.  Served: Poisson arrivals at 50/s for 60 s,
edges {32, 64, 96, 128, 192, 256} with weights (.3, .25, .2, .12, .08, .05),
Re log-uniform in [100, 5000], u0 uniform in [0.02, 0.08], steps uniform in
[200, 5000], float32 or float16 deviations 50/50."""
import math

import numpy as np


def test_served_trace(imex):
    from imexlbm_gb300 import serve
    reqs = serve.trace()
    n = len(reqs)
    assert abs(n - 3000) < 5 * math.sqrt(3000)
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) >= 0) and t[0] >= 0 and t[-1] < 60.0
    edges = np.array([r["edge"] for r in reqs])
    for e, w in zip(serve.EDGES, serve.WEIGHTS):
        assert abs(np.mean(edges == e) - w) < 0.03, (e, np.mean(edges == e))
    re = np.array([r["Re"] for r in reqs])
    assert re.min() >= 100 and re.max() <= 5000
    assert abs(math.log(np.median(re)) - 0.5 * math.log(100 * 5000)) < 0.15   # log-uniform
    u0 = np.array([r["u0"] for r in reqs])
    assert u0.min() >= 0.02 and u0.max() <= 0.08
    steps = np.array([r["steps"] for r in reqs])
    assert steps.min() >= 200 and steps.max() <= 5000
    f32 = np.mean([r["precision"] == "f32" for r in reqs])
    assert 0.45 < f32 < 0.55
    assert serve.trace() == reqs                  # seeded: the same trace every run


def test_batched_workload(imex):
    from imexlbm_gb300 import batched
    w = batched.workload(64)
    assert len(w) == 64 and w == batched.workload(64)
    assert {x["edge"] for x in w} <= set(batched.EDGES)
    assert all(100 <= x["Re"] <= 3200 and isinstance(x["Re"], int) for x in w)
    assert all(0.02 <= x["u0"] <= 0.08 for x in w)
    assert all(0.0 <= p < 2 * math.pi for x in w for p in x["phase"])
    assert all(x["precision"] == "f32" for x in w)
    mixed = batched.workload(64, precision="mixed")
    assert {x["precision"] for x in mixed} == {"f32", "f16dev"}


def test_tau_follows_the_deck(imex):
    """tau = u0 sx / Re / cs2 / 2 / 3.1415926 with Re an int (src/System.cpp:22-28)."""
    from imexlbm_gb300 import serve
    for edge, re, u0 in [(32, 147, 0.058), (256, 1600, 0.05), (96, 4999, 0.02)]:
        want = u0 * edge / re / (1.0 / 3.0) / 2.0 / 3.1415926
        assert abs(serve.tau_of(edge, re, u0) - want) <= 1e-15 * want
