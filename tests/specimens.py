"""Shared small specimens for the parity tests (seeded, seconds on the oracle)."""

import numpy as np

from sand_atlas_dem_gb300.shapes import ShapeLibrary, perturbed_grain
from sand_atlas_dem_gb300.spec import Experiment
from sand_atlas_dem_gb300.workloads import contact_lattice


def small_library(frequency=4, count=4, seed=1000):
    return ShapeLibrary([perturbed_grain(frequency, seed=seed + k) for k in range(count)])


def lattice_case(side=4, *, frequency=4, friction=0.5, viscosity=0.0, policy="conservative", speed=0.02,
                 seed=3, dt=2e-9, spacing=0.985):
    library = small_library(frequency)
    case = contact_lattice(library, side, spacing=spacing, seed=seed, speed=speed)
    spec = Experiment(
        particles=side**3, contact_geometry="mesh", timestep=dt, friction=friction,
        normal_viscosity=viscosity, timestep_policy=policy, max_overlap_fraction=0.5,
        contacts_per_particle=256, pairs_per_particle=32,
    )
    return library, spec, case


def upload(engine, name, array):
    buffer = engine.buffers[name]
    if isinstance(buffer, np.ndarray):
        buffer[...] = np.asarray(array, buffer.dtype).reshape(buffer.shape)
    else:
        buffer.copy_from_numpy(np.ascontiguousarray(array))


def build(engine_cls, library, spec, case, **kwargs):
    e = engine_cls(library, spec, case["positions"], case["cell"], case["ids"], case["scales"], **kwargs)
    upload(e, "rotation", case["rotations"])
    v = np.zeros((spec.particles, 4), np.float32)
    v[:, :3] = case["velocities"] * e.time_unit / e.length_unit
    upload(e, "velocity", v)
    return e


def engine_classes():
    """(id, class) pairs: the CPU oracle always, the GPU engine under the gpu mark."""
    import pytest

    from oracle.engine import OracleEngine

    def gpu_engine(*args, **kwargs):
        from sand_atlas_dem_gb300.engine import Engine

        return Engine(*args, **kwargs)

    return [pytest.param(OracleEngine, id="oracle"), pytest.param(gpu_engine, id="gpu", marks=pytest.mark.gpu)]


def read(e, name, rows, dtype=np.float32, width=4):
    buffer = e.buffers[name]
    if isinstance(buffer, np.ndarray):
        return buffer.reshape(-1, width)[:rows].copy() if buffer.ndim > 1 else buffer[:rows].copy()
    return e.read(name, dtype, (rows, width))


_SDF_CUBE = []


def sdf_cube():
    """The exact cube with its signed-distance grid (built once per process)."""
    from sand_atlas_dem_gb300.shapes import exact_cube, with_sdf

    if not _SDF_CUBE:
        _SDF_CUBE.append(with_sdf(exact_cube(), resolution=16))
    return _SDF_CUBE[0]


def cube_pair(engine_cls, *, separation=9.99e-5, friction=0.5, dt=1e-9, viscosity=0.0,
              policy="active-contact", geometry="mesh"):
    """Two exact six-node cubes, h = 0.1 mm (``tests/test_cpu_solver.py:121-173``),
    with the mesh or the SDF contact geometry."""
    from sand_atlas_dem_gb300.shapes import ShapeLibrary, exact_cube

    spec = Experiment(particles=2, periodic=True, contact_geometry=geometry, timestep=dt, timestep_policy=policy,
                      normal_viscosity=viscosity, friction=friction, max_overlap_fraction=0.1,
                      contacts_per_particle=128)
    positions = [[0.005] * 3, [0.005 + separation, 0.005, 0.005]]
    shape = sdf_cube() if geometry == "sdf" else exact_cube()
    return engine_cls(ShapeLibrary([shape]), spec, positions, [0.01] * 3, [0, 0], [1, 1])


def plane(normal=(0, 0, 1), offset=0.00155, velocity=(0, 0, 0), friction=0.3, **extra):
    """One penalty plane in the reference's input form (``tests/test_wall_boundaries.py:23-31``)."""
    return dict(normal=list(normal), offset=offset, velocity=list(velocity), normal_stiffness=1e12,
                tangential_stiffness=5e11, friction=friction, **extra)


def box_planes(low, high, **extra):
    """Six inward axis planes xmin, xmax, ymin, ymax, zmin, zmax bounding [low, high]^3."""
    from sand_atlas_dem_gb300.boundaries import BOX_NORMALS

    return [plane(n, low if i % 2 == 0 else -high, **extra) for i, n in enumerate(BOX_NORMALS.tolist())]


_SDF_GRAINS = {}


def walled_lattice(geometry="mesh", side=3, *, dt=2e-9, friction=0.5, viscosity=0.0, squeeze=0.03,
                   policy="conservative"):
    """``side**3`` jittered lattice grains in a nonperiodic domain, boxed by six
    planes that already press the outer grains (``squeeze`` equivalent
    diameters inside the lattice's outer faces), plus one tilted plane; the
    walls are given inward velocities.  Returns (library, spec, case,
    wall_velocities)."""
    from sand_atlas_dem_gb300.shapes import with_sdf

    library = small_library(4)
    if geometry == "sdf":
        if not _SDF_GRAINS:
            _SDF_GRAINS["lib"] = ShapeLibrary([with_sdf(s, resolution=16) for s in library.shapes])
        library = _SDF_GRAINS["lib"]
    case = contact_lattice(library, side, spacing=1.0, seed=5, speed=0.02)
    l0 = case["cell"][0] / side
    margin = 2 * l0
    case["positions"] = case["positions"] + margin
    case["cell"] = case["cell"] + 2 * margin
    low, high = margin + squeeze * l0, margin + side * l0 - squeeze * l0
    planes = box_planes(low, high, friction=0.4)
    tilt = np.array([1.0, 1.0, 1.0]) / np.sqrt(3.0)
    # Cuts the corner grain at the origin side about 0.05 diameters deep.
    planes.append(plane(tilt, float(tilt @ np.full(3, margin + 0.5 * l0)) - 0.45 * l0, friction=0.2,
                        normal_viscosity=viscosity))
    spec = Experiment(
        particles=side**3, periodic=False, contact_geometry=geometry, timestep=dt, friction=friction,
        normal_viscosity=viscosity, timestep_policy=policy, max_overlap_fraction=0.5,
        contacts_per_particle=512, pairs_per_particle=32, planes=planes, boundary_box=list(range(6)),
    )
    velocities = np.zeros((len(planes), 3))
    for i in range(6):
        velocities[i] = np.array(planes[i]["normal"]) * 0.05
    velocities[6] = [0.01, -0.02, 0.03]
    return library, spec, case, velocities
