"""Continuous batching: requests submitted while others are on the GPU are
admitted between restart cycles, overlap on the device, and each result is
the same as the same solve run alone (bit-identical: a system's reductions
use only its own parts)."""
import time

import numpy as np
import pytest

from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


def test_served_results_equal_solo(fg):
    probs = [G.transport_problem(n, angle_deg=a, k=k) for n, a, k in
             [(65, 30.0, 1e-6), (17, 200.0, 1e-3), (33, 95.0, 1e-8), (129, 315.0, 1e-5), (9, 10.0, 1e-2),
              (48, 140.0, 1e-7)]]
    # alone
    solo = []
    for p in probs:
        s = fg.transport_system(p)
        s.transport_prepare(p)
        st = fg.solve_resident([s], precision=fg.FG_PREC_MIXED)[0]
        solo.append((s.solution(), st))
    # served, staggered arrivals
    systems = [fg.transport_system(p) for p in probs]
    sv = fg.Server(precision=fg.FG_PREC_MIXED)
    for i, (s, p) in enumerate(zip(systems, probs)):
        sv.submit(s, p, i)
        time.sleep(0.003 * (i % 3))
    sv.wait(len(probs), timeout=120)
    res = {r["tag"]: r for r in sv.poll()}
    sv.close()
    assert sorted(res) == list(range(len(probs)))
    overlapped = 0
    for i, s in enumerate(systems):
        X0, st0 = solo[i]
        assert res[i]["converged"] == 1 and res[i]["status"] == 0
        assert res[i]["iterations"] == st0["iterations"]
        assert res[i]["true_rel_residual"] <= 1e-10
        assert np.array_equal(s.solution(), X0)
        assert res[i]["t_submit"] <= res[i]["t_admit"] <= res[i]["t_done"]
        others = [r for j, r in res.items() if j != i]
        overlapped += any(r["t_admit"] < res[i]["t_done"] and res[i]["t_admit"] < r["t_done"] for r in others)
    assert overlapped >= 2


def test_server_admission_respects_budget(fg):
    probs = [G.transport_problem(33, angle_deg=30.0 * i, k=1e-4) for i in range(4)]
    systems = [fg.transport_system(p) for p in probs]
    sv = fg.Server(precision=fg.FG_PREC_MIXED, max_active=1)
    for i, (s, p) in enumerate(zip(systems, probs)):
        sv.submit(s, p, i)
    sv.wait(4, timeout=120)
    res = sorted(sv.poll(), key=lambda r: r["t_admit"])
    sv.close()
    assert len(res) == 4
    for a, b in zip(res, res[1:]):
        assert b["t_admit"] >= a["t_done"]      # one at a time
