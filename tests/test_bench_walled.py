"""The walled benchmark workload is a valid wall-stage case: nonperiodic, six
box planes that press the outer grains within the overlap limit, grains
inside the domain, and a timestep under the conservative bound with the
planes' stiffness included (``gpu.py:370-413``)."""

import numpy as np

import bench
from sand_atlas_dem_gb300.boundaries import BOX_NORMALS, box_extents
from sand_atlas_dem_gb300.model import HostLayout, conservative_timestep


def test_walled_workload_is_a_valid_wall_stage_case():
    w = bench.Workload("walled-10k")
    spec = w.spec
    positions, cell, ids, scales = w.specimens[0]
    assert not spec.periodic and len(spec.planes) == 6 and spec.boundary_box == list(range(6))
    assert np.array_equal([p["normal"] for p in spec.planes], BOX_NORMALS)
    assert np.all(positions > 0) and np.all(positions < cell)
    extents = box_extents(np.array([p["offset"] for p in spec.planes]), spec.boundary_box, cell)
    assert np.all(extents > 0)
    assert 0 < spec.timestep <= conservative_timestep(w.lib, spec, ids, scales)
    layout = HostLayout(w.lib, spec, positions, cell, ids, scales)
    assert layout.wall_count == 6 and layout.config(dt=spec.timestep)["wallBoxEnabled"] == 1
    # Every plane moves inward (velocity along its own normal).
    for p in spec.planes:
        assert np.dot(p["velocity"], p["normal"]) > 0
    # The planes press the outer grains by much less than the overlap limit.
    low = spec.planes[0]["offset"]
    radius = max(w.lib.shapes[int(i)].radius * s for i, s in zip(ids, scales))
    deepest = low - (positions[:, 0] - radius).min()
    assert 0 < deepest < spec.max_overlap_fraction * 2 * radius
