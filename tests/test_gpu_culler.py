"""The learned culler: gradients, training, calibration and zero misses.

* GPU gradients of the network against the float64 CPU oracle
  (``oracle/culler_ref.py``) on the same batch.
* Training lowers the loss; the calibrated margin exceeds the run-time
  prediction at every calibration point inside the shapes.
* With the culler attached, the contact key set, contact geometry and forces
  are those of the exact path (zero missed contacts), and fewer nodes go to
  the exact BVH query than without it.
"""

import numpy as np
import pytest

from oracle.culler_ref import forward_backward
from sand_atlas_dem_gb300.culler import LearnedCuller
from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu


def small_culler(engine, **kwargs):
    args = dict(points=1 << 14, steps=300, batch=1024, seed=5)
    args.update(kwargs)
    return LearnedCuller(engine, **args)


def test_gradients_match_cpu_oracle(gpu_library):
    library, spec, case = lattice_case(side=4)
    e = build(Engine, library, spec, case)
    c = small_culler(e, steps=0)
    c.training_points = c.sample(c.points, c.seed)
    grads, index = c.gradients(step=3)
    params = c.params.cpu().numpy()
    pts = c.training_points.cpu().numpy().reshape(c.shapes, c.points, 4)
    for s in range(c.shapes):
        loss, ref = forward_backward(params[s], pts[s][index[s]], c.shell, c.over)
        scale = np.abs(ref).max()
        np.testing.assert_allclose(grads[s], ref, rtol=2e-3, atol=2e-4 * scale)


def test_tensor_core_tile_matches_fp32_rows(gpu_library):
    """The tcgen05 tile (BF16 x BF16 -> FP32 in tensor memory, 128 rows a
    tile, several shapes per tile) against the same network evaluated row by
    row on CUDA cores with the same BF16 features and weights: only the
    order of the FP32 accumulation differs (tolerance 1e-5 of the output
    range)."""
    library, spec, case = lattice_case(side=4)
    e = build(Engine, library, spec, case)
    c = small_culler(e, steps=50)
    c.train()
    import ctypes as ct
    from sand_atlas_dem_gb300 import native
    native.check(c.lib.sdg_culler_round(ct.c_void_p(c.params.data_ptr()), ct.c_void_p(c.w1.data_ptr()), c.shapes,
                                        ct.c_void_p(c.stream.cuda_stream)))
    # 1000 points a shape: tiles straddle shape boundaries.
    pts = c.sample(1000, 99)
    tile = c.predict(pts).cpu().numpy()
    rows = c.evaluate(pts).cpu().numpy()
    scale = np.abs(rows).max()
    np.testing.assert_allclose(tile, rows, rtol=0, atol=1e-5 * scale)


def test_training_reduces_loss_and_margin_covers_inside(gpu_library):
    library, spec, case = lattice_case(side=4)
    e = build(Engine, library, spec, case)
    c = small_culler(e)
    losses = c.train()
    assert losses[-1][1] < 0.25 * losses[0][1]
    margins = c.calibrate()
    pts, pred = c.validation
    phi = pts[:, 3].cpu().numpy().reshape(c.shapes, -1)
    y = pred.cpu().numpy().reshape(c.shapes, -1)
    inside = phi <= 0
    assert np.all(y[inside] <= np.repeat(margins[:, None], y.shape[1], axis=1)[inside])
    # Each cell's margin covers the inside calibration points of the cell
    # and never exceeds the whole shape's.
    cells = c._cells(pts).view(c.shapes, -1).cpu().numpy()
    cell_margin = np.take_along_axis(c.cell_margins, cells, axis=1)
    assert np.all(y[inside] <= cell_margin[inside])
    assert np.all(c.cell_margins <= margins[:, None])
    assert c.cull_rate() > 0.1


@pytest.mark.parametrize("side", [4, 6])
def test_culled_step_has_zero_missed_contacts(gpu_library, side):
    library, spec, case = lattice_case(side=side, viscosity=4e5)
    # Against the reference's own filters (plane, hull): the certified
    # distance-bound grid already skips what the network could, so it is off.
    exact = build(Engine, library, spec, case, distance_grid=False)
    culled = build(Engine, library, spec, case, distance_grid=False)
    c = small_culler(culled)
    c.train()
    c.attach(culled)
    exact.initialize()
    culled.initialize()
    for _ in range(3):
        exact.advance(2, rate=(-0.5, -0.5, -0.5))
        culled.advance(2, rate=(-0.5, -0.5, -0.5))
        se, sc = exact.state(), culled.state()
        assert se["contacts"] == sc["contacts"] > 0
        np.testing.assert_array_equal(sc["meta"], se["meta"])
        for name in ("position", "velocity", "force", "torque", "slip", "normalArea"):
            assert sc[name].tobytes() == se[name].tobytes(), name
    stats = culled.read("cullerStats", np.uint32, (4,))
    assert stats[0] > 0 and stats[1] > 0
    # What the network gains: fewer exact BVH queries for the same contacts.
    work_exact, work_culled = exact.read("work", np.uint32, (64,)), culled.read("work", np.uint32, (64,))
    assert work_culled[2] == work_exact[2]          # the same conservative survivors
    assert work_culled[3] < work_culled[2]          # of which fewer go to the exact query
    print(dict(side=side, survivors=int(work_culled[2]), exact_queries=int(work_culled[3]),
               culled_share=1 - int(work_culled[3]) / int(work_culled[2])))
