"""Penalty planes (walls): the input contract and the CPU oracle against the
reference's own closed-form wall checks (``tests/test_wall_boundaries.py``,
``tests/test_wall_coulomb.py``, ``tests/test_wall_local_frame.py``,
``tests/test_wall_reductions.py``), whose tolerances these tests keep."""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.boundaries import box_extents
from sand_atlas_dem_gb300.shapes import ShapeLibrary, analytic_sphere, box_shape, surface_nodes, with_sdf
from sand_atlas_dem_gb300.spec import Experiment
from tests.specimens import box_planes, plane

_CAP = []


def cap_shape():
    if not _CAP:
        _CAP.append(analytic_sphere(samples=32768))
    return _CAP[0]


def cap_engine(**settings):
    """One 0.5 mm sphere centred 2 mm above the origin, 0.05 mm into the plane
    z = 1.55 mm (``tests/test_wall_boundaries.py:85-99``)."""
    spec = Experiment(periodic=False, particles=1, timestep=1e-8, max_overlap_fraction=0.1,
                      contacts_per_particle=4096, planes=[plane(**settings.pop("plane", {}))], **settings)
    return OracleEngine(ShapeLibrary([cap_shape()]), spec, [[0.002] * 3], [0.006] * 3, [0], [1])


def rows_of(e):
    data, _ = e.diagnostic_rows()
    return data, e.wall_rows()


def test_wall_input_contract():
    """``tests/test_wall_boundaries.py:44-80``."""
    with pytest.raises(ValueError, match="nonperiodic"):
        Experiment(planes=[plane()])
    for change in (dict(normal=[0, 0, 2]), dict(offset=float("nan")), dict(velocity=[0, 0]),
                   dict(normal_stiffness=0), dict(tangential_stiffness=-1), dict(friction=-1), dict(extra=0)):
        value = plane()
        value.update(change)
        with pytest.raises(ValueError):
            Experiment(periodic=False, planes=[value])
    box = box_planes(0.0005, 0.0055)
    for ids in ([0] * 6, [0, 1, 2, 3, 4, 6], list(range(5)), [0, 1, 2, 3, 5, 4]):
        with pytest.raises(ValueError):
            Experiment(periodic=False, planes=box, boundary_box=ids)
    assert np.allclose(box_extents(np.array([p["offset"] for p in box]), list(range(6))), 0.005)
    with pytest.raises(ValueError, match="nonpositive"):
        Experiment(periodic=False, planes=box_planes(0.006, 0.0055), boundary_box=list(range(6)))
    with pytest.raises(ValueError, match="planes"):
        Experiment(periodic=False, stages=[dict(kind="wall", steps=2, wall_velocities=[])])
    value = Experiment(periodic=False, planes=[plane()],
                       stages=[dict(kind="wall", steps=2, wall_velocities=[[0, 0, 0.1]])])
    assert Experiment(**value.to_dict()).planes == value.planes
    assert value.checkpoint_format == "sand-dem-checkpoint/4"


def test_oracle_full_area_cap_force_reaction_moment_and_energy():
    """``tests/test_wall_boundaries.py:102-142``: penalty cap force pi kn R d^2,
    energy pi kn R d^3 / 3, the wall reaction and its moment balance the grain."""
    e = cap_engine()
    e.initialize()
    data, walls = rows_of(e)
    radius, depth = 0.0005, 0.00005
    force = np.pi * 1e12 * radius * depth**2
    energy = np.pi * 1e12 * radius * depth**3 / 3
    state = e.state()
    actual = state["force"][0, :3] * e.force_unit
    assert abs(actual[2] / force - 1) < 0.001
    assert abs(data[1, 3] * e.energy_unit / energy - 1) < 0.001
    reaction = walls[0, 0, :3] * e.force_unit
    assert np.linalg.norm(actual + reaction) < force * 1e-5
    torque = state["torque"][0, :3] * e.energy_unit
    origin_moment = np.cross([0.002] * 3, actual) + torque
    assert np.linalg.norm(origin_moment + walls[0, 1, :3] * e.energy_unit) < force * 0.006 * 1e-5
    count = int(walls[0, 0, 3].view(np.uint32))
    assert count == state["contacts"] > 0
    assert np.all(state["meta"][:, 1] == 1) and np.all(state["meta"][:, 3] == 1)
    assert data[6, 3] == 0 and walls[0, 2, 0] == 0
    # Common-node virial without a half-weight wall factor.
    nodes = cap_shape().samples + [0.002] * 3
    depths = np.maximum(0, 0.00155 - nodes[:, 2])
    nodal_force = 1e12 * cap_shape().areas * depths
    expected_stress = -np.outer([0, 0, 1], np.sum(nodal_force[:, None] * cap_shape().samples, axis=0)) / 0.006**3
    contact_stress = data[:3, :3].astype(float) * e.energy_unit / 0.006**3
    assert np.linalg.norm(contact_stress - expected_stress) < force * radius / 0.006**3 * 1e-4


def test_oracle_wall_partial_slip_matches_cap_force_torque_and_return_loss():
    """``tests/test_wall_coulomb.py:19-71``: one step of a plane sliding by
    25 um under the cap: Coulomb-limited traction integrals."""
    radius, kn, kt, mu, slip, dt = 0.0005, 1e12, 5e11, 0.3, 0.000025, 1e-8
    e = cap_engine()
    e.initialize()
    e.advance(1, wall_velocities=[[slip / dt, 0, 0]])
    state = e.state()
    data, _ = rows_of(e)
    centre = (state["position"][0, :3].astype(float) + state["positionRemainder"][0, :3]) * e.length_unit
    depth = radius + 0.00155 - centre[2]
    c, a = mu * kn, kt * slip
    h = min(depth, a / c)
    j0 = c * h**2 / 2 + a * (depth - h)
    j1 = c * h**3 / 3 + a * (depth**2 - h**2) / 2
    expected_force = np.array([2 * np.pi * radius * j0, 0, np.pi * kn * radius * depth**2])
    expected_torque = np.array([0, -2 * np.pi * radius * ((radius - depth) * j0 + j1), 0])
    expected_loss = 2 * np.pi * radius * c * (slip * h**2 / 2 - c * h**3 / (3 * kt))
    force = state["force"][0, :3] * e.force_unit
    torque = state["torque"][0, :3] * e.energy_unit
    assert np.linalg.norm(force - expected_force) < np.linalg.norm(expected_force) * 0.001
    assert np.linalg.norm(torque - expected_torque) < np.linalg.norm(expected_torque) * 0.001
    assert abs(data[6, 0] * e.energy_unit / expected_loss - 1) < 0.001
    ctrl = e.check_errors()
    assert 0 < ctrl[6] / ctrl[2] < 1
    assert data[6, 3] > 0


@pytest.mark.parametrize("geometry", ["sdf", "mesh"])
def test_oracle_rotated_wall_collection_matches_exhaustive_nodes(geometry):
    """``tests/test_wall_boundaries.py:145-195``: a rotated box against a
    tilted plane; the collected nodes are exactly those behind it."""
    from scipy.spatial.transform import Rotation

    base = box_shape([1e-3, 8e-4, 6e-4])
    shape = box_shape([1e-3, 8e-4, 6e-4], nodes=surface_nodes(base.vertices, base.faces, 4096, 0))
    if geometry == "sdf":
        shape = with_sdf(shape, resolution=16)
    normal = np.array([1, 2, 3], float) / np.sqrt(14)
    rotation = Rotation.from_euler("xyz", [0.2, -0.3, 0.4])
    centre = np.array([0.002] * 3)
    arms = rotation.apply(shape.samples)
    offset = (arms @ normal).min() + centre @ normal + 0.00001
    spec = Experiment(periodic=False, contact_geometry=geometry, particles=1, timestep=1e-9,
                      max_overlap_fraction=0.03, contacts_per_particle=4096, planes=[plane(normal, offset)])
    e = OracleEngine(ShapeLibrary([shape]), spec, [centre], [0.006] * 3, [0], [1])
    e.buffers["rotation"][0] = rotation.as_quat().astype(np.float32)
    e.initialize()
    depth = np.maximum(0, offset - (arms + centre) @ normal)
    force = shape.areas[:, None] * depth[:, None] * 1e12 * normal
    expected_force, expected_torque = force.sum(0), np.cross(arms, force).sum(0)
    state = e.state()
    assert state["contacts"] == np.count_nonzero(depth)
    assert set(state["meta"][:, 2]) == set(np.flatnonzero(depth))
    scale = np.linalg.norm(expected_force)
    assert np.linalg.norm(state["force"][0, :3] * e.force_unit - expected_force) < scale * 1e-4
    assert np.linalg.norm(state["torque"][0, :3] * e.energy_unit - expected_torque) < scale * shape.radius * 1e-4


def test_oracle_box_walls_advance_and_invalid_gap_flag():
    """``tests/test_wall_boundaries.py:329-355``: the zmax plane moving at
    -1 m/s for ten steps; a gap that closes raises the boundary-box flag."""
    from sand_atlas_dem_gb300.model import RejectedStep

    shape = analytic_sphere(samples=64)
    spec = Experiment(periodic=False, particles=1, planes=box_planes(0.0005, 0.0055), boundary_box=list(range(6)),
                      timestep=1e-8)
    e = OracleEngine(ShapeLibrary([shape]), spec, [[0.003] * 3], [0.006] * 3, [0], [1])
    e.initialize()
    velocities = np.zeros((6, 3))
    velocities[5, 2] = -1
    e.advance(10, wall_velocities=velocities)
    offsets = (e.buffers["wallPlane"][:, 3].astype(float) + e.buffers["wallRemainder"][:, 3]) * e.length_unit
    assert np.allclose(box_extents(offsets, list(range(6)), [0.006] * 3), [0.005, 0.005, 0.005 - 1e-7], rtol=1e-7)
    before = e.state()
    velocities[5, 2] = -1e6
    with pytest.raises(RejectedStep, match="invalid boundary box"):
        e.advance(1, wall_velocities=velocities)
    after = e.state()
    for name, value in before.items():
        assert np.array_equal(np.asarray(value), np.asarray(after[name])), name


def translation_case(engine_cls, centre, normal):
    """``tests/test_wall_local_frame.py:40-91``: the six-node cube 0.1 um into
    a plane with its centre at ``centre`` on every axis."""
    from sand_atlas_dem_gb300.shapes import exact_cube

    cube = exact_cube()
    h, depth, kn = 1e-4, 1e-7, 1e12
    p = np.full(3, centre)
    n = np.array(normal, float)
    offset = float(p @ n + min(cube.samples @ n) + depth)
    wall = dict(normal=list(normal), offset=offset, velocity=[0, 0, 0], normal_stiffness=kn,
                tangential_stiffness=kn / 2, friction=0)
    spec = Experiment(periodic=False, particles=1, timestep=2e-9, planes=[wall], contacts_per_particle=64,
                      pairs_per_particle=8, bin_capacity=16, max_overlap_fraction=0.1, contact_geometry="mesh")
    e = engine_cls(ShapeLibrary([cube]), spec, [p], [max(0.01, 2 * centre)] * 3, [0], [1])
    e.initialize()
    state = e.state()
    delta = np.maximum(0, offset - p @ n - cube.samples @ n)
    forces = kn * (cube.areas * delta)[:, None] * n
    expected = forces.sum(axis=0)
    torque = np.cross(cube.samples, forces).sum(axis=0)
    scale = np.linalg.norm(expected)
    actual = state["force"][0, :3].astype(float) * e.force_unit
    actual_torque = state["torque"][0, :3].astype(float) * e.force_unit * e.length_unit
    assert np.linalg.norm(actual - expected) / scale <= 1e-4
    assert np.linalg.norm(actual_torque - torque) / (scale * h) <= 1e-4
    restored = (state["position"][0, :3].astype(float) + state["positionRemainder"][0, :3]) * e.length_unit
    assert np.linalg.norm(restored - p) / h <= 1e-7
    assert len(state["meta"]) == np.count_nonzero(delta)
    return state


@pytest.mark.parametrize("centre", [0.005, 5.0])
@pytest.mark.parametrize("normal", [[0, 0, 1], [0.6, 0, 0.8], [1 / 3, 2 / 3, 2 / 3]])
def test_oracle_shallow_contact_preserves_force_and_local_torque_under_translation(centre, normal):
    translation_case(OracleEngine, centre, normal)


def two_stage_case(engine_cls):
    """``tests/test_wall_reductions.py:33-72``: 257 spheres between two planes
    (two partial 256-row groups, then a second reduction pass)."""
    shape = analytic_sphere(samples=2048)
    n = 257
    centres = np.array([[0.002 + (i % 17) * 0.002, 0.002 + (i // 17) * 0.002, 0.002] for i in range(n)])
    walls = [plane([0, 0, 1], 0.00155), plane([0, 0, -1], -0.00245)]
    spec = Experiment(periodic=False, particles=n, timestep=1e-8, max_overlap_fraction=0.1,
                      contacts_per_particle=256, planes=walls)
    e = engine_cls(ShapeLibrary([shape]), spec, centres, [0.04, 0.04, 0.006], [0] * n, [1] * n)
    e.initialize()
    expected = []
    for wall in walls:
        normal = np.array(wall["normal"], float)
        depth = np.maximum(0, wall["offset"] - (shape.samples + centres[0]) @ normal)
        forces = shape.areas[:, None] * 1e12 * depth[:, None] * normal
        reaction = -n * forces.sum(0)
        moment = -np.cross(shape.samples, forces).sum(0) * n - np.cross(centres, forces.sum(0)).sum(0)
        expected.append((n * np.count_nonzero(depth), reaction, moment))
    return e, expected


def test_oracle_two_stage_wall_reduction_counts_reactions_and_moments():
    e, expected = two_stage_case(OracleEngine)
    rows = e.wall_rows()
    for w, (count, reaction, moment) in enumerate(expected):
        assert int(rows[w, 0, 3].view(np.uint32)) == count
        assert np.linalg.norm(rows[w, 0, :3] * e.force_unit - reaction) < np.linalg.norm(reaction) * 1e-4
        assert np.linalg.norm(rows[w, 1, :3] * e.energy_unit - moment) < np.linalg.norm(reaction) * 0.04 * 1e-4
    assert sum(int(rows[w, 0, 3].view(np.uint32)) for w in range(2)) == e.state()["contacts"]


def test_oracle_wall_and_grain_histories_coexist_and_wall_work_reduces_over_bodies():
    """``tests/test_wall_reductions.py:97-151``: two spheres touching each
    other and a moving plane keep both friction histories; the wall's
    reaction and moment balance the grains."""
    shape = analytic_sphere(samples=8192)
    spec = Experiment(periodic=False, particles=2, timestep=1e-8, max_overlap_fraction=0.1,
                      contacts_per_particle=4096, planes=[plane([0, 0, 1], 0.00155)])
    e = OracleEngine(ShapeLibrary([shape]), spec, [[0.002] * 3, [0.002995, 0.002, 0.002]], [0.006] * 3, [0, 0],
                     [1, 1])
    e.initialize()
    velocity = np.zeros((2, 4), np.float32)
    velocity[:, :3] = np.array([[0, 0.01, 0], [0, -0.01, 0]]) * e.time_unit / e.length_unit
    e.buffers["velocity"][...] = velocity
    e.advance(3, wall_velocities=[[0.1, 0, 0.1]])
    state = e.state()
    data, fabric = e.diagnostic_rows()
    walls = e.wall_rows()
    assert round(float(fabric[1, 2])) == 1
    wall_keys = state["meta"][:, 1] == 2
    assert wall_keys.any() and (~wall_keys).any()
    assert len({tuple(k[:3]) for k in state["meta"]}) == state["contacts"]
    assert np.max(np.abs(state["slip"][wall_keys, :3])) > 0
    assert np.max(np.abs(state["slip"][~wall_keys, :3])) > 0
    scale = data[1, 3] * e.energy_unit
    assert abs(data[6, 3] * e.energy_unit - walls[0, 2, 0] * e.energy_unit) < scale * 1e-5
    total_force = state["force"][:, :3].sum(0) * e.force_unit
    reaction = walls[0, 0, :3] * e.force_unit
    assert np.linalg.norm(total_force + reaction) < np.linalg.norm(total_force) * 1e-5
    centres = (state["position"][:, :3].astype(float) + state["positionRemainder"][:, :3]) * e.length_unit
    total_moment = np.cross(centres, state["force"][:, :3] * e.force_unit).sum(0)
    total_moment += state["torque"][:, :3].sum(0) * e.energy_unit
    assert np.linalg.norm(total_moment + walls[0, 1, :3] * e.energy_unit) < np.linalg.norm(total_force) * 0.006 * 1e-5
