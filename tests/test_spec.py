"""The experiment contract accepts reference case JSON and rejects what it must."""

import json

import pytest

from sand_atlas_dem_gb300.model import HostLayout
from sand_atlas_dem_gb300.shapes import ShapeLibrary, exact_cube
from sand_atlas_dem_gb300.spec import Experiment


def test_defaults_and_checkpoint_formats():
    e = Experiment()
    assert e.contact_geometry == "sdf" and e.checkpoint_format == "sand-dem-checkpoint/3"
    assert Experiment(normal_viscosity=1.0).checkpoint_format == "sand-dem-checkpoint/5"


def test_round_trip_through_json(tmp_path):
    e = Experiment(contact_geometry="mesh", particles=8, stages=[dict(kind="strain", steps=4, rate=[-1, 0, 0])])
    path = tmp_path / "case.json"
    path.write_text(json.dumps(dict(e.to_dict(), shape_library="shapes.h5")))
    loaded = Experiment.load(path)
    assert loaded.particles == 8 and loaded.shape_library.endswith("shapes.h5")


@pytest.mark.parametrize("bad", [dict(contact_geometry="voxel"), dict(particles=0), dict(timestep=-1.0),
                                 dict(stages=[]), dict(stages=[dict(kind="strain", steps=1)]),
                                 dict(periodic=True, planes=[dict(normal=[0, 0, 1])])])
def test_invalid_cases_raise(bad):
    with pytest.raises(ValueError):
        Experiment(**bad)


def test_backend_scope_is_explicit():
    library = ShapeLibrary([exact_cube()])
    # The default geometry is the SDF one, which needs a grid on every shape.
    with pytest.raises(ValueError, match="signed-distance grid"):
        HostLayout(library, Experiment(particles=2, timestep=1e-9), [[0.005] * 3, [0.0051, 0.005, 0.005]],
                   [0.01] * 3, [0, 0], [1, 1])
    with pytest.raises(ValueError, match="conservative estimate"):
        HostLayout(library, Experiment(particles=2, contact_geometry="mesh", timestep=0.01),
                   [[0.005] * 3, [0.0051, 0.005, 0.005]], [0.01] * 3, [0, 0], [1, 1])
