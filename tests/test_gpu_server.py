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


def test_served_mixed_transport_and_euler(fg):
    """Euler time loops served beside transport solves: each Euler result
    equals the same loop run alone through fg_euler_predictor (the loop is
    deterministic), transport results are unchanged, and Euler loops overlap
    with the transport batch in time."""
    tprobs = [G.transport_problem(n, angle_deg=a, k=1e-5) for n, a in [(129, 30.0), (65, 200.0), (97, 300.0)]]
    eprobs = [G.obliquo_problem(n) for n in (33, 17)]
    topts = [fg.time_opts(0, 2, 1e-3, 0, 4 * p.dt, 1e-6, max_steps=4) for p in eprobs]
    solo_u = []
    for p, to in zip(eprobs, topts):
        s = fg.euler_system(p)
        u, a, st = s.euler_predictor(p, to, kmax=30, lmax=10000, tol=1e-10, precision=fg.FG_PREC_MIXED)
        solo_u.append((u, st))
    solo_t = []
    for p in tprobs:
        s = fg.transport_system(p)
        s.transport_prepare(p)
        solo_t.append(fg.solve_resident([s], precision=fg.FG_PREC_MIXED)[0])
    tsys = [fg.transport_system(p) for p in tprobs]
    esys = [fg.euler_system(p) for p in eprobs]
    sv = fg.Server(precision=fg.FG_PREC_MIXED)
    sv.submit_euler(esys[0], eprobs[0], topts[0], 100)
    for i, (s, p) in enumerate(zip(tsys, tprobs)):
        sv.submit(s, p, i)
    sv.submit_euler(esys[1], eprobs[1], topts[1], 101)
    sv.wait(5, timeout=120)
    res = {r["tag"]: r for r in sv.poll()}
    sv.close()
    assert sorted(res) == [0, 1, 2, 100, 101]
    for k, (u0, st0) in zip((100, 101), solo_u):
        assert np.array_equal(res[k]["u"], u0)
        assert res[k]["iterations"] == st0["gmres_iterations"]
        assert res[k]["cycles"] == st0["corrections"]
        assert res[k]["true_rel_residual"] <= 1e-10
    for i in range(3):
        assert res[i]["iterations"] == solo_t[i]["iterations"]
    e0 = res[100]
    assert any(res[i]["t_admit"] < e0["t_done"] and e0["t_admit"] < res[i]["t_done"] for i in range(3))


def test_server_euler_rejects_transport_system(fg):
    p = G.transport_problem(9)
    s = fg.transport_system(p)
    sv = fg.Server()
    with pytest.raises(fg.FemGpuError):
        sv.submit_euler(s, G.obliquo_problem(9), fg.time_opts(0, 1, 1e-3, 0, 1.0, 1e-6, max_steps=1), 7)
    sv.close()


def test_server_budget_admits_one_at_a_time_from_idle(fg):
    """A byte budget smaller than one request: four requests submitted to an
    idle server are admitted one at a time (a request larger than the budget
    still runs, alone), transport and Euler alike."""
    probs = [G.transport_problem(33, angle_deg=40.0 * i, k=1e-4) for i in range(4)]
    systems = [fg.transport_system(p) for p in probs]
    ep = G.obliquo_problem(17)
    es = fg.euler_system(ep)
    to = fg.time_opts(0, 2, 1e-3, 0, 2 * ep.dt, 1e-6, max_steps=2)
    sv = fg.Server(precision=fg.FG_PREC_MIXED, hbm_budget_bytes=1)
    for i, (s, p) in enumerate(zip(systems, probs)):
        sv.submit(s, p, i)
    sv.submit_euler(es, ep, to, 10)
    sv.wait(5, timeout=120)
    res = sorted(sv.poll(), key=lambda r: r["t_admit"])
    sv.close()
    assert len(res) == 5 and all(r["converged"] == 1 for r in res)
    for a, b in zip(res, res[1:]):
        assert b["t_admit"] >= a["t_done"]      # never two admitted at once


def test_served_euler_loops_share_cycles(fg):
    """Several Euler loops submitted together run at the same time (their
    correction solves share the Euler batch) and each ends in exactly the
    state of its solo fg_euler_predictor run."""
    eprobs = [G.obliquo_problem(n) for n in (17, 25, 33, 21)]
    topts = [fg.time_opts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6, max_steps=3) for p in eprobs]
    solo = []
    for p, to in zip(eprobs, topts):
        s = fg.euler_system(p)
        u, a, st = s.euler_predictor(p, to, kmax=30, lmax=10000, tol=1e-10, precision=fg.FG_PREC_MIXED)
        solo.append((u, st))
    esys = [fg.euler_system(p) for p in eprobs]
    sv = fg.Server(precision=fg.FG_PREC_MIXED)
    for i, (s, p, to) in enumerate(zip(esys, eprobs, topts)):
        sv.submit_euler(s, p, to, i)
    sv.wait(len(eprobs), timeout=120)
    res = {r["tag"]: r for r in sv.poll()}
    sv.close()
    assert sorted(res) == list(range(len(eprobs)))
    for i, (u0, st0) in enumerate(solo):
        assert np.array_equal(res[i]["u"], u0)
        assert res[i]["iterations"] == st0["gmres_iterations"]
        assert res[i]["cycles"] == st0["corrections"]
    overlaps = sum(res[i]["t_admit"] < res[j]["t_done"] and res[j]["t_admit"] < res[i]["t_done"]
                   for i in res for j in res if i < j)
    assert overlaps >= 3


def test_host_buffer_requests_equal_solo(fg):
    """fg_server_submit_host: blocks and right-hand side from host buffers
    (the C ABI of fg_set_blocks + fg_precond_setup(Diag) + fg_solve, served);
    the solution lands in the caller's host array before the result is
    polled and equals the device-assembled solve run alone, bit for bit."""
    probs = [G.transport_problem(n, angle_deg=a, k=k) for n, a, k in
             [(33, 30.0, 1e-6), (17, 200.0, 1e-3), (65, 95.0, 1e-8), (25, 315.0, 1e-5)]]
    solo, bufs = [], []
    for p in probs:
        s = fg.transport_system(p)
        F = s.transport_assemble(p)
        A = s.get_blocks()
        s.transport_prepare(p)
        st = fg.solve_resident([s], precision=fg.FG_PREC_MIXED)[0]
        solo.append((s.solution(), st))
        bufs.append((A, F))
    systems = [fg.transport_system(p) for p in probs]
    Xs = [np.full(p.mesh.neq + 1, np.nan) for p in probs]
    sv = fg.Server(precision=fg.FG_PREC_MIXED)
    for i, (s, (A, F)) in enumerate(zip(systems, bufs)):
        sv.submit_host(s, A, F, Xs[i], i)
    sv.wait(len(probs), timeout=120)
    res = {r["tag"]: r for r in sv.poll()}
    sv.close()
    assert sorted(res) == list(range(len(probs)))
    for i in range(len(probs)):
        X0, st0 = solo[i]
        assert res[i]["converged"] == 1 and res[i]["status"] == 0
        assert res[i]["iterations"] == st0["iterations"]
        assert res[i]["true_rel_residual"] <= 1e-10
        assert np.array_equal(Xs[i][:-1], X0[:-1])
