"""The certified distance-bound grid: every point of a cell lies at least the
cell's bound from the surface (checked against the oracle's exact query), so
skipping nodes whose bound is positive never drops a contact."""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import DISTANCE_GRID, Engine
from tests.specimens import build, lattice_case
from tests.test_oracle_pins import probe

pytestmark = pytest.mark.gpu


def test_cell_bounds_hold_at_random_points(gpu_library):
    library, spec, case = lattice_case(side=4, frequency=8)
    g = build(Engine, library, spec, case)
    o = build(OracleEngine, library, spec, case)
    shapes, cells = len(library.shapes), DISTANCE_GRID**3
    grid = g.read("distanceGrid", np.float32, (shapes, cells))
    info = g.read("distanceGridInfo", np.float32, (shapes, 4))
    rng = np.random.default_rng(5)
    positive = 0
    for s in range(shapes):
        pick = rng.integers(0, cells, 4000)
        # Favour cells near the surface, where the bound is tightest.
        near = np.flatnonzero(np.abs(grid[s]) < 0.1)
        pick[:2000] = rng.choice(near, 2000)
        ijk = np.stack([pick % DISTANCE_GRID, (pick // DISTANCE_GRID) % DISTANCE_GRID,
                        pick // DISTANCE_GRID**2], 1)
        h = float(info[s, 3])
        points = info[s, :3].astype(np.float64) + (ijk + rng.uniform(0.02, 0.98, (len(pick), 3))) * h
        phi = probe(o, s, points.astype(np.float32))[:, 3]
        bound = grid[s, pick]
        assert np.all(phi >= bound - 1e-6), (s, float((bound - phi).max()))
        assert np.all(phi[bound > 0] > 0)
        positive += int((bound > 0).sum())
    assert positive > 0
