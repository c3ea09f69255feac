"""The SDF contact geometry (trilinear signed-distance query,
``solver.slang:188-200``, collected per pair in the reference's 64-lane
order, ``solver.slang:536-572``) on the GPU against the CPU oracle.

Bit-exact gates as for the mesh geometry: pair lists, contact keys and their
order, contact geometry, history slots and the zero-timestep forces; after
timesteps the state is compared at 1e-5 relative (CUDA and libm may round the
integrator's transcendental functions differently in the last place).
"""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from sand_atlas_dem_gb300.shapes import ShapeLibrary, analytic_sphere, perturbed_grain, with_sdf
from sand_atlas_dem_gb300.spec import Experiment
from sand_atlas_dem_gb300.workloads import contact_lattice
from tests.specimens import build

pytestmark = pytest.mark.gpu
REL = 1e-5
_LIBRARIES = {}


def sdf_library(kind):
    if kind not in _LIBRARIES:
        if kind == "sphere":
            shapes = [analytic_sphere(resolution=24, samples=256)]
        else:
            shapes = [with_sdf(perturbed_grain(4, seed=1000 + k, nodes=162), resolution=14) for k in range(2)]
        _LIBRARIES[kind] = ShapeLibrary(shapes)
    return _LIBRARIES[kind]


def sdf_case(kind, side=4, spacing=0.98, speed=0.05, viscosity=4e5):
    library = sdf_library(kind)
    case = contact_lattice(library, side, spacing=spacing, seed=5, speed=speed)
    spec = Experiment(particles=side**3, contact_geometry="sdf", timestep=2e-9, friction=0.5,
                      normal_viscosity=viscosity, max_overlap_fraction=0.5, contacts_per_particle=512,
                      pairs_per_particle=32)
    return library, spec, case


def assert_close(a, b, what):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max() if a.size else 0.0
    assert err <= REL * scale, f"{what}: max error {err:.3e} vs scale {scale:.3e}"


@pytest.mark.parametrize("kind", ["sphere", "grain"])
def test_sdf_initialize_bit_exact(gpu_library, kind):
    library, spec, case = sdf_case(kind)
    o, g = build(OracleEngine, library, spec, case), build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    oc, gc = o.check_errors(), g.check_errors()
    assert oc[1] == gc[1] > 0 and oc[2] == gc[2] > 0
    count, n = int(oc[2]), spec.particles
    so, sg = o.state(), g.state()
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    assert sg["normalArea"].tobytes() == so["normalArea"].tobytes()
    assert g.read("pointDepth", np.float32, (count, 4)).tobytes() == o.buffers["pointDepth"][:count].tobytes()
    for name in ("force", "torque", "particleStress", "accumulated"):
        rows = 3 * n if name == "particleStress" else n
        assert g.read(name, np.float32, (rows, 4)).tobytes() == o.buffers[name][:rows].tobytes(), name


@pytest.mark.parametrize("kind", ["sphere", "grain"])
def test_sdf_steps_match_oracle(gpu_library, kind):
    library, spec, case = sdf_case(kind)
    o, g = build(OracleEngine, library, spec, case), build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    for chunk in (1, 3, 4):
        o.advance(chunk, rate=(-0.5, -0.5, -0.5))
        g.advance(chunk, rate=(-0.5, -0.5, -0.5))
        so, sg = o.state(), g.state()
        assert so["contacts"] == sg["contacts"] > 0
        np.testing.assert_array_equal(sg["meta"], so["meta"])
        for name in ("position", "velocity", "rotation", "momentum", "force", "torque", "slip", "normalArea"):
            assert_close(sg[name], so[name], name)


def test_sdf_restore_collects_identically(gpu_library):
    """Restart from the GPU's own state in both engines: contact keys, history
    slots (through the SDF emit-order keys) and forces agree bit for bit."""
    library, spec, case = sdf_case("grain")
    g = build(Engine, library, spec, case)
    g.initialize()
    g.advance(5)
    state = g.state()
    o, g2 = build(OracleEngine, library, spec, case), build(Engine, library, spec, case)
    o.restore(state, 5)
    g2.restore(state, 5)
    so, sg = o.state(), g2.state()
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    assert sg["slip"].tobytes() == so["slip"].tobytes()
    assert sg["force"].tobytes() == so["force"].tobytes()
    # and the restarted engine continues as the uninterrupted one, to the
    # reference's restart tolerance (test_cpu_solver.py:212-238)
    g.advance(3)
    g2.advance(3)
    a, b = g.state(), g2.state()
    np.testing.assert_array_equal(a["meta"], b["meta"])
    for name in ("position", "velocity", "force", "slip"):
        np.testing.assert_allclose(b[name], a[name], rtol=2e-6, atol=1e-9, err_msg=name)
