"""The autotuner (fg_autotune): candidate launch shapes timed on the batch
itself, the fastest kept per (block size, precision, batch-size class).

* the choice is one of the candidates and is returned again, unchanged and
  marked as cached, for the same key (deterministic for a given cache);
* batches solved afterwards (which use the cached choice) converge to the
  same solutions as with the built-in rule;
* fg_tune_clear forgets it.
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
