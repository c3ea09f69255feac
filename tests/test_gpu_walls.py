"""Penalty planes (walls) on the GPU: plane contacts collected per (wall,
grain) in the reference CPU collector's order, the plane contact law with
friction history, the wall rows and their reduction, wall motion and the box
check, against the CPU oracle and the reference's closed-form wall checks
(``tests/test_wall_boundaries.py``, ``tests/test_wall_coulomb.py``).

Bit-exact gates at zero timestep (contact keys and order, contact records,
forces, wall rows); after timesteps the state is compared at 1e-5 relative
(CUDA and libm may round the integrator's transcendental functions
differently in the last place) with identical contact keys.
"""

import copy

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from sand_atlas_dem_gb300.model import WALL_STATE, RejectedStep
from sand_atlas_dem_gb300.shapes import ShapeLibrary, analytic_sphere
from sand_atlas_dem_gb300.spec import Experiment
from tests.specimens import box_planes, build, plane, walled_lattice

pytestmark = pytest.mark.gpu
REL = 1e-5
_CAP = []


def assert_close(a, b, what, rel=REL):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max() if a.size else 0.0
    assert err <= rel * scale, f"{what}: max error {err:.3e} vs scale {scale:.3e}"


def cap_engine(cls=Engine, capacity=4096, offset=0.00155):
    if not _CAP:
        _CAP.append(ShapeLibrary([analytic_sphere(samples=32768)]))
    spec = Experiment(periodic=False, particles=1, timestep=1e-8, max_overlap_fraction=0.1,
                      contacts_per_particle=capacity, planes=[plane(offset=offset)])
    return cls(_CAP[0], spec, [[0.002] * 3], [0.006] * 3, [0], [1])


CASES = [("mesh", False, "conservative"), ("sdf", False, "conservative"), ("mesh", True, "active-contact")]


@pytest.mark.parametrize("geometry,viscous,policy", CASES)
def test_walls_initialize_bit_exact(gpu_library, geometry, viscous, policy):
    library, spec, case, _ = walled_lattice(geometry, viscosity=4e5 if viscous else 0.0, policy=policy)
    o, g = build(OracleEngine, library, spec, case), build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    so, sg = o.state(), g.state()
    walls = so["meta"][:, 1] >= spec.particles
    assert so["contacts"] == sg["contacts"] and walls.sum() > 100 and (~walls).sum() > 100
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    for name in ("normalArea", "slip", "force", "torque"):
        assert sg[name].tobytes() == so[name].tobytes(), name
    for name in ("wallRows", "wallAccumulated", "wallPlane", "wallRemainder"):
        assert sg[name].tobytes() == so[name].tobytes(), name
    ref = o.wall_rows()
    walls = g.wall_count
    rows = g.m.read_prefix(g._reduce_walls(), 12 * walls, np.float32, shape=(walls, 3, 4))
    assert rows.tobytes() == ref.tobytes()
    row = g.diagnostics()
    for w, wall in enumerate(row["walls"]):
        assert wall["active_surface_contacts"] == int(ref[w, 0, 3].view(np.uint32))


@pytest.mark.parametrize("geometry,viscous,policy", CASES)
def test_walls_steps_match_oracle(gpu_library, geometry, viscous, policy):
    library, spec, case, velocities = walled_lattice(geometry, viscosity=4e5 if viscous else 0.0, policy=policy)
    o, g = build(OracleEngine, library, spec, case), build(Engine, library, spec, case)
    for e in (o, g):
        e.initialize()
        e.advance(3, wall_velocities=velocities)
        e.advance(4, wall_velocities=0.5 * velocities)
    so, sg = o.state(), g.state()
    assert so["contacts"] == sg["contacts"]
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    assert np.max(np.abs(so["slip"][:, :3])) > 0
    for name in ("position", "velocity", "rotation", "momentum", "force", "torque", "accumulated", "slip",
                 *WALL_STATE):
        assert_close(sg[name], so[name], name)
    ref = o.wall_rows()
    row = g.diagnostics()
    assert_close([w["work"] for w in row["walls"]], ref[:, 2, 0] * g.energy_unit, "wall work")
    assert row["wall_work"] != 0 and row["cell"] != row["domain_cell"]


def test_full_area_cap_force_reaction_moment_and_energy(gpu_library):
    """``tests/test_wall_boundaries.py:102-142`` on the GPU engine."""
    engine = cap_engine()
    engine.initialize()
    row = engine.diagnostics()
    radius, depth = 0.0005, 0.00005
    force = np.pi * 1e12 * radius * depth**2
    energy = np.pi * 1e12 * radius * depth**3 / 3
    state = engine.state()
    actual = state["force"][0, :3] * engine.force_unit
    assert abs(actual[2] / force - 1) < 0.001
    assert abs(row["elastic_energy_proxy"] / energy - 1) < 0.001
    reaction = np.array(row["walls"][0]["reaction"])
    assert np.linalg.norm(actual + reaction) < force * 1e-5
    torque = state["torque"][0, :3] * engine.energy_unit
    origin_moment = np.cross([0.002] * 3, actual) + torque
    assert np.linalg.norm(origin_moment + row["walls"][0]["reaction_moment_origin"]) < force * 0.006 * 1e-5
    assert row["walls"][0]["active_surface_contacts"] == row["active_surface_contacts"] > 0
    assert row["active_grain_pairs"] == 0
    assert row["wall_work"] == row["walls"][0]["work"] == 0


def test_moving_wall_work_balance_and_velocity_change(gpu_library):
    """``tests/test_wall_boundaries.py:198-225``: actuator work from the
    measured reactions, wall work rows and the energy balance."""
    engine = cap_engine()
    engine.initialize()
    initial = engine.diagnostics()
    energy0 = initial["elastic_energy_proxy"]
    expected_work = 0
    previous = initial
    for velocity in ([0, 0, 0.1], [0, 0, -0.1]):
        for _ in range(50):
            engine.advance(1, wall_velocities=[velocity])
            row = engine.diagnostics()
            mean_force = -0.5 * (np.array(previous["walls"][0]["reaction"]) + row["walls"][0]["reaction"])
            expected_work += np.dot(mean_force, velocity) * engine.spec.timestep
            assert abs(row["wall_work"] - expected_work) < energy0 * 1e-5
            assert abs(row["walls"][0]["work"] - row["wall_work"]) < energy0 * 1e-5
            residual = row["wall_work"] - (row["kinetic_energy"] + row["elastic_energy_proxy"] - energy0)
            assert abs(residual) < energy0 * 0.001
            assert row["cell_work"] == 0
            previous = row
    assert abs(previous["walls"][0]["offset"] - initial["walls"][0]["offset"]) < 1e-11


def test_wall_partial_slip_matches_cap_force_torque_and_return_loss(gpu_library):
    """``tests/test_wall_coulomb.py:19-71`` on the GPU engine."""
    radius, kn, kt, mu, slip, dt = 0.0005, 1e12, 5e11, 0.3, 0.000025, 1e-8
    engine = cap_engine()
    engine.initialize()
    engine.advance(1, wall_velocities=[[slip / dt, 0, 0]])
    state, row = engine.state(), engine.diagnostics()
    centre = (state["position"][0, :3].astype(float) + state["positionRemainder"][0, :3]) * engine.length_unit
    depth = radius + 0.00155 - centre[2]
    c, a = mu * kn, kt * slip
    h = min(depth, a / c)
    j0 = c * h**2 / 2 + a * (depth - h)
    j1 = c * h**3 / 3 + a * (depth**2 - h**2) / 2
    expected_force = np.array([2 * np.pi * radius * j0, 0, np.pi * kn * radius * depth**2])
    expected_torque = np.array([0, -2 * np.pi * radius * ((radius - depth) * j0 + j1), 0])
    expected_loss = 2 * np.pi * radius * c * (slip * h**2 / 2 - c * h**3 / (3 * kt))
    force = state["force"][0, :3] * engine.force_unit
    torque = state["torque"][0, :3] * engine.energy_unit
    assert np.linalg.norm(force - expected_force) < np.linalg.norm(expected_force) * 0.001
    assert np.linalg.norm(torque - expected_torque) < np.linalg.norm(expected_torque) * 0.001
    assert abs(row["friction_dissipation"] / expected_loss - 1) < 0.001
    assert 0 < row["sliding_fraction"] < 1
    assert row["wall_work"] > 0


def test_wall_friction_restart_rollback_and_restore_checks(gpu_library):
    """``tests/test_wall_boundaries.py:228-274``, ``:277-287`` and ``:387-405``."""
    engine = cap_engine()
    engine.initialize()
    engine.advance(3, wall_velocities=[[0.1, 0, 0]])
    saved = engine.state()
    assert np.max(np.abs(saved["slip"][:, :3])) > 0
    engine.advance(5)
    expected = engine.state()
    engine.restore(saved, 3)
    engine.advance(5)
    again = engine.state()
    for name in ("position", "velocity", "rotation", "momentum", "force", "torque", "accumulated", "wallPlane",
                 "wallRemainder", "wallVelocity", "wallAccumulated"):
        assert np.allclose(expected[name], again[name], rtol=2e-4, atol=3e-7), name
    # Remove and return the plane at dt = 0: history is gone.
    separated = copy.deepcopy(again)
    separated["wallPlane"][0, 3] = 0
    separated["wallRemainder"][0, 3] = 0
    engine.restore(separated, 8)
    assert engine.state()["contacts"] == 0
    returned = copy.deepcopy(engine.state())
    returned["wallPlane"] = saved["wallPlane"]
    returned["wallRemainder"] = saved["wallRemainder"]
    engine.restore(returned, 8)
    state = engine.state()
    assert state["contacts"] > 0 and not np.any(state["slip"][:, :3])
    # A penetration failure rolls back velocity, history and work.
    engine.advance(2, wall_velocities=[[0.1, 0, 0]])
    before = engine.state()
    with pytest.raises(RejectedStep, match="penetration"):
        engine.advance(3, wall_velocities=[[0, 0, 1e5]])
    after = engine.state()
    for name, value in before.items():
        assert np.array_equal(np.asarray(after[name]), np.asarray(value)), name
    assert engine.step == 10
    engine.advance(1)
    # Restore and wall velocities are checked before anything changes.
    before = engine.state()
    changed = copy.deepcopy(before)
    changed["wallPlane"][0, :3] = [0, 1, 0]
    with pytest.raises(ValueError, match="normal identity"):
        engine.restore(changed, 0)
    with np.errstate(over="ignore"):
        with pytest.raises(ValueError, match="FP32"):
            engine.advance(1, wall_velocities=[[1e300, 0, 0]])
    after = engine.state()
    for name, value in before.items():
        assert np.array_equal(np.asarray(after[name]), np.asarray(value)), name


def test_wall_contact_growth_retries_without_truncation(gpu_library):
    """``tests/test_wall_boundaries.py:290-326``."""
    results = []
    for capacity in (1, 4096):
        engine = cap_engine(capacity=capacity, offset=0.0014999)
        engine.initialize()
        engine.advance(2, wall_velocities=[[0, 0, 100]])
        results.append(engine)
    grown, baseline = results
    assert grown.capacity_retries
    assert grown.state()["contacts"] == baseline.state()["contacts"] > 16
    for name in ("position", "velocity", "force", "accumulated", "wallPlane", "wallAccumulated"):
        assert np.allclose(grown.state()[name], baseline.state()[name], rtol=2e-4, atol=3e-7), name


def test_wall_box_volume_strain_and_invalid_gap_rollback(gpu_library):
    """``tests/test_wall_boundaries.py:329-355``."""
    spec = Experiment(periodic=False, particles=1, planes=box_planes(0.0005, 0.0055), boundary_box=list(range(6)),
                      timestep=1e-8)
    engine = Engine(ShapeLibrary([analytic_sphere(samples=64)]), spec, [[0.003] * 3], [0.006] * 3, [0], [1])
    engine.initialize()
    velocities = np.zeros((6, 3))
    velocities[5, 2] = -1
    engine.advance(10, wall_velocities=velocities)
    row = engine.diagnostics()
    assert np.allclose(row["domain_cell"], [0.006] * 3, rtol=1e-7)
    assert np.allclose(row["cell"], [0.005, 0.005, 0.005 - 1e-7], rtol=1e-7)
    assert abs(row["axial_strain"] - 2e-5) < 1e-7
    before = engine.state()
    velocities[5, 2] = -1e6
    with pytest.raises(RejectedStep, match="invalid boundary box"):
        engine.advance(1, wall_velocities=velocities)
    for name, value in before.items():
        assert np.array_equal(value, engine.state()[name]), name


def test_wall_checkpoint_round_trip(gpu_library, tmp_path):
    """``sand-dem-checkpoint/4`` with the wall arrays (``simulation.py:87-136``)."""
    from sand_atlas_dem_gb300.checkpoint import load_checkpoint, resume, save_checkpoint

    library, spec, case, velocities = walled_lattice("mesh")
    g = build(Engine, library, spec, case)
    g.initialize()
    g.advance(3, wall_velocities=velocities)
    save_checkpoint(tmp_path / "walls.h5", g)
    attrs, state = load_checkpoint(tmp_path / "walls.h5")
    assert attrs["format"] == "sand-dem-checkpoint/4"
    for name in WALL_STATE:
        assert state[name].tobytes() == g.state()[name].tobytes(), name
    h = build(Engine, library, spec, case)
    resume(h, tmp_path / "walls.h5")
    for e in (g, h):
        e.advance(4)
    a, b = g.state(), h.state()
    np.testing.assert_array_equal(a["meta"], b["meta"])
    for name in ("position", "velocity", "force", "slip", *WALL_STATE):
        assert np.allclose(a[name], b[name], rtol=2e-4, atol=3e-7), name


@pytest.mark.parametrize("centre", [0.005, 5.0])
@pytest.mark.parametrize("normal", [[0, 0, 1], [0.6, 0, 0.8], [1 / 3, 2 / 3, 2 / 3]])
def test_shallow_contact_preserves_force_and_local_torque_under_translation(gpu_library, centre, normal):
    """``tests/test_wall_local_frame.py:40-91`` on the GPU engine, and its
    contact records bit for bit against the oracle."""
    from tests.test_walls import translation_case

    g = translation_case(Engine, centre, normal)
    o = translation_case(OracleEngine, centre, normal)
    for name in ("meta", "normalArea", "force", "torque"):
        assert g[name].tobytes() == o[name].tobytes(), name


def test_two_stage_wall_reduction_counts_reactions_and_moments(gpu_library):
    """``tests/test_wall_reductions.py:33-72``: two reduction passes of the
    (wall, grain) rows; the reduced rows bit for bit against the oracle."""
    from tests.test_walls import two_stage_case

    g, expected = two_stage_case(Engine)
    row = g.diagnostics()
    for w, (count, reaction, moment) in enumerate(expected):
        value = row["walls"][w]
        assert value["active_surface_contacts"] == count
        assert np.linalg.norm(value["reaction"] - reaction) < np.linalg.norm(reaction) * 1e-4
        assert np.linalg.norm(value["reaction_moment_origin"] - moment) < np.linalg.norm(reaction) * 0.04 * 1e-4
    assert sum(w["active_surface_contacts"] for w in row["walls"]) == row["active_surface_contacts"]
    o, _ = two_stage_case(OracleEngine)
    rows = g.m.read_prefix(g._reduce_walls(), 24, np.float32, shape=(2, 3, 4))
    assert rows.tobytes() == o.wall_rows().tobytes()


def test_wall_and_grain_histories_coexist_and_wall_work_reduces_over_bodies(gpu_library):
    """``tests/test_wall_reductions.py:97-151`` on the GPU engine."""
    from sand_atlas_dem_gb300.model import f4

    shape = analytic_sphere(samples=8192)
    spec = Experiment(periodic=False, particles=2, timestep=1e-8, max_overlap_fraction=0.1,
                      contacts_per_particle=4096, planes=[plane([0, 0, 1], 0.00155)])
    engine = Engine(ShapeLibrary([shape]), spec, [[0.002] * 3, [0.002995, 0.002, 0.002]], [0.006] * 3, [0, 0], [1, 1])
    engine.initialize()
    engine.buffers["velocity"].copy_from_numpy(
        f4(np.array([[0, 0.01, 0], [0, -0.01, 0]]) * engine.time_unit / engine.length_unit))
    engine.advance(3, wall_velocities=[[0.1, 0, 0.1]])
    row, state = engine.diagnostics(), engine.state()
    assert row["active_grain_pairs"] == 1
    wall_keys = state["meta"][:, 1] == 2
    assert wall_keys.any() and (~wall_keys).any()
    assert len({tuple(k[:3]) for k in state["meta"]}) == state["contacts"]
    assert np.max(np.abs(state["slip"][wall_keys, :3])) > 0
    assert np.max(np.abs(state["slip"][~wall_keys, :3])) > 0
    scale = row["elastic_energy_proxy"]
    assert abs(row["wall_work"] - row["walls"][0]["work"]) < scale * 1e-5
    total_force = state["force"][:, :3].sum(0) * engine.force_unit
    assert np.linalg.norm(total_force + row["walls"][0]["reaction"]) < np.linalg.norm(total_force) * 1e-5
    centres = (state["position"][:, :3].astype(float) + state["positionRemainder"][:, :3]) * engine.length_unit
    total_moment = np.cross(centres, state["force"][:, :3] * engine.force_unit).sum(0)
    total_moment += state["torque"][:, :3].sum(0) * engine.energy_unit
    assert np.linalg.norm(total_moment + row["walls"][0]["reaction_moment_origin"]) < np.linalg.norm(
        total_force) * 0.006 * 1e-5
