"""Closed-form and reference known-answer cases, on the CPU oracle and on the GPU.

Restates the hot-path cases of the reference CPU solver tests
(``tests/test_cpu_solver.py``) with the exact six-node cube (h = 0.1 mm,
six nodes of area h^2): frozen tolerances 2e-4 relative, 1e-9 N, 1e-13 N m.
"""

import numpy as np
import pytest

from sand_atlas_dem_gb300.model import RejectedStep
from tests.specimens import cube_pair, engine_classes, read, upload

ENGINES = engine_classes()


def physical(state, name):
    return state[name][:, :3].astype(float) + state[name + "Remainder"][:, :3].astype(float)


@pytest.mark.parametrize("geometry", ["mesh", "sdf"])
@pytest.mark.parametrize("make", ENGINES)
def test_cube_pair_force_is_exact(make, geometry):
    """``test_cpu_solver.py:176-209``: force on grain 0 is [-0.001, 0, 0] N (the
    cube's signed distance is linear near a face centre, so the trilinear
    SDF query is exact there too)."""
    e = cube_pair(make, geometry=geometry)
    e.initialize()
    force = read(e, "force", 2)[:, :3] * e.force_unit
    torque = read(e, "torque", 2)[:, :3] * e.energy_unit
    np.testing.assert_allclose(force[0], [-0.001, 0, 0], rtol=2e-4, atol=1e-9)
    np.testing.assert_allclose(force[1], [0.001, 0, 0], rtol=2e-4, atol=1e-9)
    np.testing.assert_allclose(torque[0], 0, atol=1e-13)
    e.advance(10)
    v = read(e, "velocity", 2)[:, :3]
    np.testing.assert_allclose(v.sum(axis=0), 0, atol=1e-8)


@pytest.mark.parametrize("make", ENGINES)
def test_periodic_seam_uses_minimum_image(make):
    """``test_cpu_solver.py:493-515``: a pair straddling the periodic seam."""
    e = cube_pair(make)
    positions = np.array([[0.00004995, 0.005, 0.005], [0.00995005, 0.005, 0.005]])
    p = positions / e.length_unit
    upload(e, "position", np.pad(p.astype(np.float32), ((0, 0), (0, 1))))
    upload(e, "positionRemainder", np.pad((p - p.astype(np.float32)).astype(np.float32), ((0, 0), (0, 1))))
    e.initialize()
    force = read(e, "force", 2)[:, :3] * e.force_unit
    state = e.state()
    q = physical(state, "position")
    cell = state["cell"][0, :3].astype(float)
    branch = q[1] - q[0]
    branch -= np.floor(branch / cell + 0.5) * cell
    magnitude = 1e12 * 1e-8 * (1e-4 - abs(branch[0] * e.length_unit))
    np.testing.assert_allclose(force, [[magnitude, 0, 0], [-magnitude, 0, 0]], rtol=2e-4, atol=1e-9)
    assert int(e.check_errors()[1]) == 1


@pytest.mark.parametrize("make", ENGINES)
def test_viscous_pair_force_and_galilean_invariance(make):
    """``test_cpu_solver.py:879-902``: F = 0.001 + c A v, independent of drift."""
    forces = []
    for common in (0.0, 0.7):
        e = cube_pair(make, viscosity=1e6)
        v = np.array([[0.01 + common, 0, 0], [-0.01 + common, 0, 0]]) * e.time_unit / e.length_unit
        upload(e, "velocity", np.pad(v.astype(np.float32), ((0, 0), (0, 1))))
        e.initialize()
        force = read(e, "force", 2)[:, :3] * e.force_unit
        expected = 0.001 + 1e6 * 1e-8 * 0.02
        np.testing.assert_allclose(force, [[-expected, 0, 0], [expected, 0, 0]], rtol=2e-4, atol=1e-9)
        forces.append(force)
        e.advance(3)
    np.testing.assert_allclose(forces[0], forces[1], rtol=2e-4, atol=1e-9)


@pytest.mark.parametrize("geometry", ["mesh", "sdf"])
@pytest.mark.parametrize("make", ENGINES)
def test_friction_history_restart_replays(make, geometry):
    """``test_cpu_solver.py:212-238``: slip history survives a restart."""
    e = cube_pair(make, geometry=geometry)
    v = np.array([[0, 0.01, 0], [0, -0.01, 0]]) * e.time_unit / e.length_unit
    upload(e, "velocity", np.pad(v.astype(np.float32), ((0, 0), (0, 1))))
    e.initialize()
    e.advance(7)
    state = e.state()
    assert np.linalg.norm(state["slip"][:, :3]) > 0
    e.advance(5)
    expected = e.state()
    restored = cube_pair(make, geometry=geometry)
    restored.restore(state, 7)
    restored.advance(5)
    actual = restored.state()
    for name in ("position", "velocity", "rotation", "momentum", "force", "torque", "slip", "accumulated"):
        np.testing.assert_allclose(actual[name], expected[name], rtol=2e-6, atol=1e-9)
    np.testing.assert_array_equal(actual["meta"], expected["meta"])


@pytest.mark.parametrize("make", ENGINES)
@pytest.mark.parametrize("dt", [1e-9, 2e-9])
def test_elastic_release_oscillator_and_bitwise_restart(make, dt):
    """``test_cpu_solver.py:23-97``: two-body release, free flight, replay."""
    e = cube_pair(make, separation=9.9e-5, friction=0, dt=dt)
    e.initialize()
    initial = e.state()
    positions = physical(initial, "position") * e.length_unit
    h = 1e-4
    overlap = h - (positions[1, 0] - positions[0, 0])
    stiffness = 1e12 * h * h
    mass = 2650.0 * h**3
    omega = np.sqrt(2 * stiffness / mass)
    release = np.pi / (2 * omega)
    energy0 = 0.5 * stiffness * overlap**2
    restart = None
    for sample in range(1, 21):
        target = round(sample * 1e-7 / dt)
        e.advance(target - e.step)
        state = e.state()
        time = target * dt
        if time <= release:
            shift = overlap * (1 - np.cos(omega * time)) / 2
            speed = overlap * omega * np.sin(omega * time) / 2
        else:
            speed = overlap * omega / 2
            shift = overlap / 2 + speed * (time - release)
        expected = positions.copy()
        expected[:, 0] += [-shift, shift]
        actual = physical(state, "position") * e.length_unit
        velocity = physical(state, "velocity") * e.length_unit / e.time_unit
        np.testing.assert_allclose(actual, expected, rtol=0, atol=1e-9)
        np.testing.assert_allclose(velocity[:, 0], [-speed, speed], rtol=1e-3, atol=1e-5)
        np.testing.assert_allclose(mass * velocity.sum(axis=0), 0, atol=1e-17)
        remaining = max(0, h - (actual[1, 0] - actual[0, 0]))
        energy = 0.5 * mass * np.sum(velocity**2) + 0.5 * stiffness * remaining**2
        np.testing.assert_allclose(energy, energy0, rtol=2e-3, atol=0)
        if sample == 4:
            assert state["contacts"] > 0
            restart = (target, state)
    assert state["contacts"] == 0
    replayed = cube_pair(make, separation=9.9e-5, friction=0, dt=dt)
    replayed.restore(restart[1], restart[0])
    replayed.advance(e.step - restart[0])
    replay = replayed.state()
    for name in ("position", "positionRemainder", "velocity", "velocityRemainder", "rotation", "momentum",
                 "force", "torque"):
        np.testing.assert_array_equal(replay[name], state[name])


@pytest.mark.parametrize("make", ENGINES)
@pytest.mark.parametrize("policy", ["conservative", "active-contact"])
def test_rejected_chunk_rolls_back(make, policy):
    """``test_cpu_solver.py:279-291``: a rejected chunk leaves no trace."""
    e = cube_pair(make, policy=policy)
    e.initialize()
    before = e.state()
    with pytest.raises(RejectedStep):
        e.advance(2, rate=[-1e8, 0, 0])
    after = e.state()
    assert e.step == 0
    for key, value in before.items():
        if isinstance(value, np.ndarray):
            np.testing.assert_array_equal(after[key], value)


@pytest.mark.parametrize("make", ENGINES)
def test_strain_cell_and_drag(make):
    """``test_cpu_solver.py:314-324``: the cell shrinks and drag dissipates."""
    e = cube_pair(make, separation=0.0002)
    v = np.array([[0.01, 0, 0], [-0.01, 0, 0]]) * e.time_unit / e.length_unit
    upload(e, "velocity", np.pad(v.astype(np.float32), ((0, 0), (0, 1))))
    e.initialize()
    e.advance(10, rate=[-1, 0, 0], drag=1e5)
    state = e.state()
    assert state["cell"][0, 0] * e.length_unit < 0.01
    accumulated = state["accumulated"]
    assert accumulated[:, 1].sum() > 0  # drag loss


@pytest.mark.parametrize("make", ENGINES)
def test_contact_capacity_growth_is_explicit_and_replays(make):
    """``test_cpu_solver.py:518-549``: overflow grows capacity and retries."""
    from sand_atlas_dem_gb300.shapes import ShapeLibrary, box_shape
    from sand_atlas_dem_gb300.spec import Experiment
    from sand_atlas_dem_gb300.shapes import surface_nodes

    box = box_shape([1e-3] * 3)
    v = box.vertices
    samples, areas = surface_nodes(v, box.faces, 1024, 0)
    box = box_shape([1e-3] * 3, nodes=(samples, areas))
    spec = Experiment(particles=4, timestep=1e-9, contact_geometry="mesh", contacts_per_particle=16,
                      pairs_per_particle=4, max_overlap_fraction=0.5)
    positions = [[0.005] * 3, [0.00602, 0.005, 0.005], [0.005, 0.009, 0.005], [0.00602, 0.009, 0.005]]
    e = make(ShapeLibrary([box]), spec, positions, [0.02] * 3, [0] * 4, [1] * 4)
    e.initialize()
    capacity = e.contact_capacity
    velocity = np.zeros((4, 4), np.float32)
    velocity[[1, 3], 0] = -0.00003 / spec.timestep * e.time_unit / e.length_unit
    upload(e, "velocity", velocity)
    if not hasattr(e, "capacity_retries"):
        pytest.skip("the oracle engine does not grow capacities (reference host logic)")
    e.advance(1)
    assert e.state()["contacts"] > capacity
    assert e.contact_capacity >= e.state()["contacts"] and e.capacity_retries


def _normal_probe(data, stiffness, viscosity, weight, precision="fp32"):
    """The oracle's normalResponse (normal.slang:2-11) through its
    normalProbe entry point (normal.slang:166-174): rows (depth, area, normal
    velocity, 0) -> (force, loss power, 0, 0)."""
    from oracle.engine import OracleEngine
    from sand_atlas_dem_gb300.shapes import ShapeLibrary, box_shape
    from sand_atlas_dem_gb300.spec import Experiment

    real = np.float64 if precision == "fp64" else np.float32
    e = OracleEngine(ShapeLibrary([box_shape([1e-3] * 3)]), Experiment(particles=2, contact_geometry="mesh",
                                                                       timestep=1e-9),
                     [[0.005] * 3, [0.015] * 3], [0.03] * 3, [0, 0], [1.0, 1.0], precision=precision)
    source = np.ascontiguousarray(np.asarray(data, real))
    out = np.zeros((len(source), 4), real)
    e.dispatch("normalProbe", len(source), e.config(), extra=(source, out),
               uniforms=(len(source), stiffness, viscosity, weight))
    return out


@pytest.mark.parametrize("weight", [0.5, 1.0])
@pytest.mark.parametrize("viscosity", [0.0, 3.0])
def test_normal_operator_compression_unload_clamp_inactive(weight, viscosity):
    """The reference's hand-evaluated table (tests/test_normal_viscosity.py:37-71):
    stiffness 8, area 2, depth 0.25 under compression, at rest, unloading
    unclipped and clipped, then separation and exact contact."""
    data = [[0.25, 2, v, 0] for v in (-2, 0, 0.25, 2)] + [[-0.1, 2, -2, 0], [0, 2, -2, 0]]
    expected = np.array([[4, 0], [4, 0], [4, 0], [4, 0], [0, 0], [0, 0]] if viscosity == 0
                        else [[16, 24], [4, 0], [2.5, 0.375], [0, 8], [0, 0], [0, 0]]) * weight
    actual = _normal_probe(data, 8, viscosity, weight)[:, :2]
    assert np.allclose(actual, expected, rtol=2e-6, atol=1e-7)
    assert (actual >= 0).all()


def test_compiled_normal_probe():
    """The reference's CPU normal probe case (tests/test_cpu_solver.py:685-708):
    kn 1e12, viscosity 1e6, weight 1/2."""
    values = np.array([[1e-7, 1e-8, -0.01, 0], [1e-7, 1e-8, 0.2, 0], [-1e-7, 1e-8, 0, 0]], np.float32)
    fn = np.where(values[:, 0] > 0,
                  np.maximum(0, 0.5 * 1e12 * values[:, 1] * values[:, 0] - 0.5 * 1e6 * values[:, 1] * values[:, 2]),
                  0)
    np.testing.assert_allclose(_normal_probe(values, 1e12, 1e6, 0.5)[:, 0], fn, rtol=2e-5, atol=1e-9)
