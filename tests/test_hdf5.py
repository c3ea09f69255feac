"""HDF5 checkpoints and shape libraries without h5py.

The reader is checked against HDF5 files the reference wrote with h5py (its
``assets/generated`` shape libraries: version-0 superblock, symbol-table
groups, variable-length string attributes, gzip-chunked datasets) when the
reference tree is present; the writer by round trips through the reader, in
both layouts, across several symbol nodes and a two-level chunk tree; the
checkpoint format by a restart of the CPU oracle engine.
"""

import json
import os
from pathlib import Path

import numpy as np
import pytest

from sand_atlas_dem_gb300 import checkpoint, hdf5
from sand_atlas_dem_gb300.shapes import ShapeLibrary, analytic_sphere, exact_cube, with_sdf
from tests.specimens import build, lattice_case

ASSETS = Path(os.environ.get("SAND_DEM_REFERENCE", "/root/reference")) / "assets" / "generated"


@pytest.mark.skipif(not ASSETS.exists(), reason="the reference tree is not present")
def test_reads_the_reference_shape_libraries():
    sphere = hdf5.read(ASSETS / "sphere.h5")
    assert sphere.attrs == {"format": "sand-dem-shapes/1", "units": "m"}
    g = sphere["0"]
    assert g.attrs["id"] == "analytical-sphere" and g.attrs["radius"] == 5e-4
    assert json.loads(g.attrs["provenance"])["fixture"] == "analytical_sphere"
    # The grid of the reference's sphere fixture, recomputed here, bit for bit.
    fixture = analytic_sphere(resolution=32, samples=512)
    assert g["sdf"].dtype == np.float32 and np.array_equal(g["sdf"], fixture.sdf)
    assert np.array_equal(g["origin"], fixture.origin) and g.attrs["spacing"] == fixture.spacing
    np.testing.assert_allclose(g["samples"], fixture.samples, rtol=0, atol=1e-18)
    library = checkpoint.load_shape_library(ASSETS / "concave-prism.h5")
    prism = library.shapes[0]
    assert prism.id == "original-concave-prism" and prism.faces.shape == (20, 3)
    assert prism.sdf.shape == (38, 38, 26) and prism.sdf.min() < 0 < prism.sdf.max()
    assert checkpoint.load_shape_library(ASSETS / "controller-sphere-r32-s512.h5").shapes[0].samples.shape == (512, 3)


@pytest.mark.parametrize("compress", [False, True])
def test_writer_round_trips(tmp_path, compress):
    members = {f"d{k:02d}": np.arange(k * 7, dtype=np.float32).reshape(-1, 7) for k in range(1, 20)}
    members["big"] = np.arange(300_000, dtype=np.uint32).reshape(-1, 4)  # many chunks
    members["empty"] = np.zeros((0, 4), np.float32)
    members["sub"] = hdf5.Group({"id": "grain", "n": 3}, {"v": np.ones((5, 3)), "f": np.arange(6).reshape(2, 3)})
    root = hdf5.Group({"format": "sand-dem-checkpoint/5", "step": 12, "x": 1.5, "flag": True,
                       "arr": np.arange(3.0), "text": "å-ü " * 300}, members)
    path = tmp_path / "f.h5"
    hdf5.write(path, root, compress=compress)
    back = hdf5.read(path)
    assert back.attrs["format"] == "sand-dem-checkpoint/5" and back.attrs["step"] == 12
    assert back.attrs["x"] == 1.5 and bool(back.attrs["flag"]) and back.attrs["text"] == root.attrs["text"]
    assert np.array_equal(back.attrs["arr"], np.arange(3.0))
    assert list(back) == sorted(members)
    for name, value in members.items():
        if isinstance(value, hdf5.Group):
            assert back[name].attrs == value.attrs
            for k, v in value.members.items():
                assert back[name][k].dtype == v.dtype and np.array_equal(back[name][k], v)
        else:
            assert back[name].dtype == value.dtype and np.array_equal(back[name], value), name


def test_shape_library_round_trip(tmp_path):
    library = ShapeLibrary([analytic_sphere(resolution=16, samples=64), with_sdf(exact_cube(), resolution=12)])
    path = tmp_path / "shapes.h5"
    checkpoint.save_shape_library(path, library)
    back = checkpoint.load_shape_library(path)
    for a, b in zip(library.shapes, back.shapes):
        assert a.id == b.id and a.spacing == b.spacing and a.provenance == b.provenance
        for name in checkpoint.SHAPE_DATASETS:
            assert np.array_equal(np.asarray(getattr(a, name)), getattr(b, name)), name


def test_checkpoint_restarts_the_oracle(tmp_path):
    from oracle.engine import OracleEngine

    library, spec, case = lattice_case(viscosity=4e5)
    e = build(OracleEngine, library, spec, case)
    e.initialize()
    e.advance(3)
    e.m = type("Adapter", (), {"name": "cpu"})()
    path = tmp_path / "checkpoint.h5"
    checkpoint.save_checkpoint(path, e, stage_index=1, rows=[{"step": 3}])
    attrs, state = checkpoint.load_checkpoint(path)
    assert attrs["format"] == "sand-dem-checkpoint/5" and attrs["step"] == 3 and attrs["backend"] == "cpu"
    assert attrs["experiment"] == spec and json.loads(attrs["rows"]) == [{"step": 3}]
    expected = e.state()
    for name, value in expected.items():
        if name == "contacts":
            assert state[name] == value
        else:
            assert state[name].tobytes() == value.tobytes(), name
    restarted = build(OracleEngine, library, spec, case)
    checkpoint.resume(restarted, path)
    e.advance(2)
    restarted.advance(2)
    a, b = e.state(), restarted.state()
    np.testing.assert_array_equal(a["meta"], b["meta"])
    for name in ("position", "velocity", "force", "slip"):
        np.testing.assert_allclose(b[name], a[name], rtol=2e-6, atol=1e-9, err_msg=name)


def test_unsupported_files_are_refused(tmp_path):
    path = tmp_path / "other.h5"
    hdf5.write(path, hdf5.Group({"format": "something-else"}))
    with pytest.raises(ValueError, match="Unsupported checkpoint"):
        checkpoint.load_checkpoint(path)
    with pytest.raises(ValueError, match="Unsupported shape format"):
        checkpoint.load_shape_library(path)
    (tmp_path / "bad.h5").write_bytes(b"not hdf5")
    with pytest.raises(ValueError, match="Not an HDF5 file"):
        hdf5.read(tmp_path / "bad.h5")
    with pytest.raises(ValueError, match="signed-distance grid"):
        checkpoint.save_shape_library(tmp_path / "s.h5", ShapeLibrary([exact_cube()]))
