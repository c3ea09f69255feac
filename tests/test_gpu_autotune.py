"""The launch-shape autotuner: shapes never change results; tuning leaves no trace."""

import json

import numpy as np
import pytest

from sand_atlas_dem_gb300 import autotune
from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu


def run(tuning, steps=4):
    library, spec, case = lattice_case(side=6, viscosity=4e5, speed=0.05)
    g = build(Engine, library, spec, case)
    g.tuning = dict(tuning)
    g.initialize()
    g.advance(steps, rate=(-0.5, -0.5, -0.5))
    return g.state()


def test_launch_shapes_are_bit_identical(gpu_library):
    base = run({})
    for tuning in (dict(query_warps=4, query_blocks_per_sm=2, cull_blocks_per_sm=2, contact_blocks_per_sm=2,
                        gather_warps_per_sm=16),
                   dict(query_warps=8, query_blocks_per_sm=16, cull_blocks_per_sm=16, contact_blocks_per_sm=16,
                        gather_warps_per_sm=32)):
        other = run(tuning)
        for k, v in base.items():
            if isinstance(v, np.ndarray):
                assert v.tobytes() == other[k].tobytes(), (tuning, k)


def test_tune_restores_state_and_caches(gpu_library, tmp_path):
    library, spec, case = lattice_case(side=6, viscosity=4e5, speed=0.05)
    g = build(Engine, library, spec, case)
    g.initialize()
    g.advance(2)
    before, step = g.state(), g.step
    cache = tmp_path / "tuning.json"
    choice, table = autotune.tune(g, repeats=1, cache=cache)
    assert g.step == step
    after = g.state()
    for k, v in before.items():
        if isinstance(v, np.ndarray):
            assert v.tobytes() == after[k].tobytes(), k
    for name, value in choice.items():
        assert value in autotune.SPACE[name]
        assert set(table[name]) == {str(v) for v in autotune.SPACE[name]}
    stored = json.loads(cache.read_text())
    assert stored[autotune.signature(g)]["choice"] == choice
    # A second engine of the same workload reads the cache without timing.
    h = build(Engine, library, spec, case)
    again, _ = autotune.tune(h, cache=cache)
    assert again == choice
    # The tuned engine continues exactly like an untuned one.
    g.advance(2)
    ref = build(Engine, library, spec, case)
    ref.initialize()
    ref.advance(4)
    assert g.state()["position"].tobytes() == ref.state()["position"].tobytes()
