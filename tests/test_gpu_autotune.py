"""The autotuner (fg_autotune): candidate launch shapes timed on the batch
itself, the fastest kept per (block size, precision, batch-size class).

* the choice is one of the candidates and is returned again, unchanged and
  marked as cached, for the same key (deterministic for a given cache);
* batches solved afterwards (which use the cached choice) converge to the
  same solutions as with the built-in rule;
* fg_tune_clear forgets it;
* a choice installed with fg_tune_set is used as given: with the 3x3
  matvec pinned to the bulk-copy pipeline or to the register kernel (same
  sums in the same order) the batch solves to the same bits.
"""
import numpy as np
import pytest

from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


def _batch(fg, count=6):
    probs = [G.transport_problem(n, angle_deg=30.0 + 40 * i, k=1e-5) for i, n in enumerate(range(65, 65 + 24 * count, 24))]
    systems = [fg.transport_system(p) for p in probs]
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    return probs, systems


def test_autotune_choice_is_cached_and_deterministic(fg):
    probs, systems = _batch(fg)
    fg.tune_clear()
    with pytest.raises(fg.FemGpuError) as e:
        fg.tune_lookup(systems)
    assert e.value.code == fg.FG_ERR_STATE
    c = fg.autotune(systems)
    # 8 part sizes x {bulk-copy, register} 3x3 matvec
    assert c["from_cache"] == 0 and c["candidates"] == 16
    assert c["part_dofs"] in (256, 512, 1024, 2048, 4096, 8192, 12288, 16384) and c["mv3_pipeline"] in (0, 1)
    assert c["ms_per_cycle"] > 0
    for again in (fg.tune_lookup(systems), fg.autotune(systems)):
        assert again["from_cache"] == 1
        assert (again["part_dofs"], again["mv3_pipeline"], again["ms_per_cycle"]) == \
               (c["part_dofs"], c["mv3_pipeline"], c["ms_per_cycle"])
    fg.tune_clear()
    with pytest.raises(fg.FemGpuError):
        fg.tune_lookup(systems)


def test_tuned_batches_solve_to_the_same_solutions(fg):
    probs, systems = _batch(fg)
    fg.tune_clear()
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    st0 = fg.solve_resident(systems, tol=1e-10, precision=fg.FG_PREC_MIXED)
    x0 = [s.solution() for s in systems]
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    fg.autotune(systems)
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    st1 = fg.solve_resident(systems, tol=1e-10, precision=fg.FG_PREC_MIXED)
    fg.tune_clear()
    for a, b, s, x in zip(st0, st1, systems, x0):
        assert a["converged"] == b["converged"] == 1 and b["true_rel_residual"] <= 1e-10
        assert np.linalg.norm(s.solution() - x) <= 1e-8 * np.linalg.norm(x)


@pytest.mark.parametrize("part_dofs", [1024, 16384])
def test_pinned_matvec_kernels_give_the_same_bits(fg, part_dofs):
    probs, systems = _batch(fg)
    sols, stats = [], []
    try:
        for mv in (1, 0):
            fg.tune_clear()
            fg.tune_set(systems, part_dofs, mv3_pipeline=mv)
            c = fg.tune_lookup(systems)
            assert (c["part_dofs"], c["mv3_pipeline"]) == (part_dofs, mv)
            for s, p in zip(systems, probs):
                s.transport_prepare(p)
            stats.append(fg.solve_resident(systems, tol=1e-10, precision=fg.FG_PREC_MIXED))
            sols.append([s.solution() for s in systems])
    finally:
        fg.tune_clear()
    for a, b, xa, xb in zip(stats[0], stats[1], sols[0], sols[1]):
        assert a["converged"] == b["converged"] == 1 and a["true_rel_residual"] <= 1e-10
        assert a["iterations"] == b["iterations"]
        assert np.array_equal(xa, xb)


def test_tune_set_rejects_bad_choices(fg):
    probs, systems = _batch(fg, count=2)
    for bad in (dict(part_dofs=100), dict(part_dofs=20000), dict(part_dofs=1001),
                dict(part_dofs=1024, mv3_pipeline=2), dict(part_dofs=1024, mv3_pipeline=-1)):
        with pytest.raises(fg.FemGpuError) as e:
            fg.tune_set(systems, **bad)
        assert e.value.code == fg.FG_ERR_ARG
