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
