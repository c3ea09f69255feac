"""Backend selection through the reference's own ``Simulation``.

The reference's ``Simulation`` (``src/sand_atlas_dem/simulation.py``,
imported from its source tree with stub ``h5py``/``trimesh`` modules, as the
golden fixtures are) wrapped by :func:`sand_atlas_dem_gb300.backend.with_gb300`:
``backend="gb300"`` runs the reference's constructor and its stage loop
(``run``: strain stage, diagnostics rows, manifest, history, checkpoint) on
the engine class the wrapper is given; the reference's own values reach its
constructor unchanged and anything else is rejected with the reference's
rule extended.  Runs where the reference tree is present.  No GPU here: the
engine handed to the wrapper is the CPU oracle behind the GB300 engine's
surface (the GB300 engine's surface is compared with the oracle's by the GPU
tests).
"""

import json
import os
import sys
import types
from pathlib import Path

import numpy as np
import pytest

from sand_atlas_dem_gb300.backend import BACKENDS, select, with_gb300

REFERENCE = Path(os.environ.get("SAND_DEM_REFERENCE", "/root/reference"))
pytestmark = pytest.mark.skipif(not (REFERENCE / "src" / "sand_atlas_dem").exists(),
                                reason="the reference tree is not present")


class _File:
    """In-memory stand-in for ``h5py.File`` (the reference checkpoints through it)."""

    written = {}

    def __init__(self, path, mode="r"):
        self.path, self.attrs, self.data = str(path), {}, {}

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        _File.written[self.path] = (dict(self.attrs), dict(self.data))

    def create_dataset(self, name, data=None, **kwargs):
        self.data[name] = np.asarray(data)


def reference():
    h5py = types.ModuleType("h5py")
    h5py.File = _File
    sys.modules.setdefault("h5py", h5py)
    sys.modules.setdefault("trimesh", types.ModuleType("trimesh"))
    os.environ["SAND_DEM_MESH_CACHE"] = "off"
    if str(REFERENCE / "src") not in sys.path:
        sys.path.insert(0, str(REFERENCE / "src"))
    import sand_atlas_dem.geometry as geometry
    import sand_atlas_dem.simulation as simulation
    import sand_atlas_dem.spec as spec

    return geometry, simulation, spec


def oracle_engine_class():
    """The CPU oracle with the members the laboratory reads beyond the step."""
    from oracle.engine import OracleEngine

    class Device:
        name = "gb300"

        def doctor(self):
            return {"backend": "gb300", "device": "CPU oracle stand-in"}

    class Array(np.ndarray):
        """A host buffer with the device buffers' upload method."""

        def copy_from_numpy(self, array):
            self[...] = np.asarray(array).reshape(self.shape)

    class Engine(OracleEngine):
        constructed = []

        def __init__(self, *args, **kwargs):
            super().__init__(*args, threads=4, **kwargs)
            self.buffers = {k: v.view(Array) for k, v in self.buffers.items()}
            self.m = Device()
            self.estimated_bytes = 0
            self.capacity_retries = []
            Engine.constructed.append(self)

    return Engine


def experiment(spec, shape_file):
    return spec.Experiment(shape_library=str(shape_file), contact_geometry="mesh", particles=27,
                           timestep=2e-9, initial_solid_fraction=0.08, friction=0.5, normal_viscosity=4e5,
                           contacts_per_particle=128, pairs_per_particle=32, diagnostic_interval=20,
                           snapshot_interval=1000,
                           stages=[{"kind": "strain", "steps": 60, "rate": [-800.0, -800.0, -800.0], "drag": 0.0}])


def library(geometry):
    from tests.golden.make_golden import as_reference_shape
    from tests.specimens import small_library

    return geometry.ShapeLibrary([as_reference_shape(geometry, s) for s in small_library().shapes])


def test_backend_values():
    assert BACKENDS == (None, "metal", "cpu", "gb300")
    assert select("gb300") == "gb300" and select(None) is None
    with pytest.raises(ValueError, match="metal, cpu or gb300"):
        select("cuda")


def test_reference_simulation_runs_a_stage_on_the_selected_engine(tmp_path):
    geometry, simulation, spec = reference()
    engine_cls = oracle_engine_class()
    GB300Simulation = with_gb300(simulation.Simulation, engine_cls=engine_cls)
    exp = experiment(spec, Path(__file__))
    lib = library(geometry)
    reference_engine = simulation.Engine
    sim = GB300Simulation(exp, library=lib, backend="gb300")
    assert simulation.Engine is reference_engine  # restored after construction
    assert isinstance(sim.engine, engine_cls) and sim.engine.step == 0
    # The reference's constructor placed, oriented and initialized the grains.
    assert sim.engine.n == 27 and sim.engine.history
    result = sim.run(tmp_path / "run")
    assert result.status == "complete", json.loads((tmp_path / "run" / "manifest.json").read_text())
    assert sim.engine.step == 60 and len(result.rows) == 4
    manifest = json.loads((tmp_path / "run" / "manifest.json").read_text())
    assert manifest["backend"]["backend"] == "gb300"
    attrs, data = _File.written[str(tmp_path / "run" / "checkpoint.h5")]
    assert attrs["backend"] == "gb300" and attrs["step"] == 60
    assert data["position"].shape == (27, 4)


def test_other_values_reach_the_reference_unchanged():
    geometry, simulation, spec = reference()
    GB300Simulation = with_gb300(simulation.Simulation, engine_cls=oracle_engine_class())
    exp = experiment(spec, Path(__file__))
    lib = library(geometry)
    with pytest.raises(ValueError, match="metal, cpu or gb300"):
        GB300Simulation(exp, library=lib, backend="cuda")
    with pytest.raises(ValueError, match="Metal device"):
        GB300Simulation(exp, library=lib, backend="gb300", metal=object())
    # "cpu" goes to the reference's own CPU adapter, which needs SlangPy
    # (absent here): its import error, not the wrapper's, is what surfaces.
    with pytest.raises(ImportError):
        GB300Simulation(exp, library=lib, backend="cpu")
