"""Several independent periodic specimens stepped in one launch per phase.

Each specimen of a batch must evolve as it does alone: same contact keys and
forces, poses and slips within the step tolerance (the batch shares one
Verlet skin and cutoff, the largest over all grains, so its pair lists are a
superset and bin grids can differ; contact sets cannot).
"""

import numpy as np
import pytest

from sand_atlas_dem_gb300.engine import Engine
from sand_atlas_dem_gb300.spec import Experiment
from sand_atlas_dem_gb300.workloads import contact_lattice
from tests.specimens import small_library

pytestmark = pytest.mark.gpu


def specimen_cases():
    library = small_library()
    cases = [contact_lattice(library, side, spacing=sp, seed=seed, speed=0.03)
             for side, sp, seed in ((4, 0.985, 3), (5, 0.99, 8), (4, 0.98, 13))]
    return library, cases


def spec_for(n):
    return Experiment(particles=n, contact_geometry="mesh", timestep=2e-9, friction=0.5, normal_viscosity=4e5,
                      max_overlap_fraction=0.5)


def load(e, rows, name, array):
    buffer = e.read(name, np.float32, (e.n, 4))
    buffer[rows] = array
    e.buffers[name].copy_from_numpy(buffer)


def test_batch_matches_single_specimens(gpu_library):
    library, cases = specimen_cases()
    total = sum(len(c["positions"]) for c in cases)
    batch = Engine.batch(library, spec_for(total),
                         [(c["positions"], c["cell"], c["ids"], c["scales"]) for c in cases])
    starts = np.cumsum([0] + [len(c["positions"]) for c in cases])
    singles = []
    for k, c in enumerate(cases):
        rows = slice(starts[k], starts[k + 1])
        e = Engine(library, spec_for(len(c["positions"])), c["positions"], c["cell"], c["ids"], c["scales"])
        for eng, r in ((e, slice(None)), (batch, rows)):
            load(eng, r, "rotation", c["rotations"])
            v = np.zeros((len(c["positions"]), 4), np.float32)
            v[:, :3] = c["velocities"] * eng.time_unit / eng.length_unit
            load(eng, r, "velocity", v)
        singles.append(e)
    batch.initialize()
    for e in singles:
        e.initialize()
    rates = np.array([[-0.5, -0.5, -0.5], [-0.1, -0.2, -0.3], [0.0, 0.0, -1.0]])
    for _ in range(3):
        batch.advance(2, rate=rates)
        for k, e in enumerate(singles):
            e.advance(2, rate=rates[k])
    sb = batch.state()
    for k, e in enumerate(singles):
        se = e.state()
        rows = slice(starts[k], starts[k + 1])
        mine = sb["meta"][(sb["meta"][:, 0] >= starts[k]) & (sb["meta"][:, 0] < starts[k + 1])].copy()
        mine[:, :2] -= np.uint32(starts[k])
        key = lambda m: m[np.lexsort(m[:, :3].T[::-1])]  # noqa: E731
        np.testing.assert_array_equal(key(mine), key(se["meta"]))
        np.testing.assert_array_equal(sb["cell"][3 * k:3 * k + 3], se["cell"])
        for name in ("position", "velocity", "rotation", "force", "torque"):
            ref = se[name].astype(float)
            err = np.abs(sb[name][rows] - ref).max()
            assert err <= 1e-5 * max(np.abs(ref).max(), 1e-30), (k, name, err)
