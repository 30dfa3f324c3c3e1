"""The autotuner's greedy search (host logic, CPU) and, on the GPU, that the
tuned engine steps the same trajectory as the default one."""
from __future__ import annotations

import numpy as np
import pytest


def test_greedy_search_keeps_the_best_of_each_stage():
    from gpudem_gb300 import autotune
    stages = [[{"a": 1}, {"a": 2}, {"a": 3}], [{"b": 1}, {"b": 2}]]
    cost = {(1, None): 5.0, (2, None): 3.0, (3, None): 4.0, (2, 1): 2.5, (2, 2): 3.5}
    seen = []

    def measure(s):
        seen.append(dict(s))
        return cost[(s["a"], s.get("b"))]

    t = autotune.search(stages, measure)
    assert t.settings == {"a": 2, "b": 1}
    assert t.ms_per_step == 2.5
    assert seen[3:] == [{"a": 2, "b": 1}, {"a": 2, "b": 2}]   # stage 2 starts from stage 1's best
    assert len(t.trials) == 5


def test_candidates_keep_the_cell_at_least_the_list_cutoff():
    from gpudem_gb300 import autotune, scenes
    sc = scenes.config1_box_drop()
    rmax = float(sc.r.max())
    stages = autotune.candidate_stages(sc, "mixed")
    assert len(stages) == 4
    for opt in stages[1]:
        assert opt["cell_size"] >= 2 * rmax + opt["skin"] - 1e-15
    assert {o["mixed_kernel"] for o in stages[0]} == {1, 2, 3}
    assert len(autotune.candidate_stages(sc, "fp64")) == 2
    assert all(o["inner_skin"] > 0 for o in stages[2])


@pytest.mark.gpu
def test_tuned_engine_steps_the_same_trajectory():
    from gpudem_gb300 import autotune, engine, scenes
    sc = scenes.config2_tilted_box(n=5_000)
    t = autotune.autotune(sc, precision="mixed", model="hertz_mindlin", steps=16, warmup=4)
    assert t.ms_per_step > 0 and len(t.trials) == len(autotune.KERNELS) + len(autotune.SKIN_FACTORS) + len(
        autotune.INNER_FACTORS) + len(autotune.GRAPH_STEPS)
    A = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    B = engine.Engine(sc, precision="mixed", model="hertz_mindlin", **t.settings)
    A.step(300)
    B.step(300)
    xa, xb = A.export_positions(), B.export_positions()
    # kernel, skin, cell size, inner skin and graph length leave the
    # trajectory unchanged: the contacts and their order are the same
    assert np.array_equal(xa, xb)
