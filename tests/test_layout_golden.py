"""Host layout against fixtures produced by the reference implementation.

``golden/packing.npz`` holds ``mesh.pack_meshes`` output and
``golden/layout.npz`` the buffers and Config block the reference ``Engine``
constructor builds (both written by ``golden/make_golden.py``).  The packed
layout decides node keys and every FP32 bound, so it must be byte-identical.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from sand_atlas_dem_gb300.model import HostLayout
from sand_atlas_dem_gb300.packing import REFERENCE_ARRAYS, pack_library
from sand_atlas_dem_gb300.shapes import ShapeLibrary, box_shape, exact_cube, perturbed_grain
from sand_atlas_dem_gb300.spec import Experiment

GOLDEN = Path(__file__).resolve().parent / "golden"


def shapes():
    return [perturbed_grain(4, seed=1000), perturbed_grain(5, seed=1001, axes=(0.7, 0.9, 1.0)),
            exact_cube(), box_shape([1e-3, 2e-3, 3e-3])]


def test_packing_matches_reference_bytes():
    ours = pack_library(ShapeLibrary(shapes()), 1e-3)
    with np.load(GOLDEN / "packing.npz") as ref:
        assert set(ref.files) == set(REFERENCE_ARRAYS)
        for name in REFERENCE_ARRAYS:
            assert ours[name].dtype == ref[name].dtype and ours[name].shape == ref[name].shape, name
            assert ours[name].tobytes() == ref[name].tobytes(), name


def test_tree_arrays_match_reference_bytes():
    """``golden/packing_trees.npz``: the reference's trees over 3,000 sample
    nodes and 2,880 triangles, and over coordinates with many ties and signed
    zeros (the stable sort's order decides the node keys' leaves)."""
    from tests.golden.make_golden import stored_tree_shapes

    ours = pack_library(ShapeLibrary(stored_tree_shapes()), 1e-3)
    with np.load(GOLDEN / "packing_trees.npz") as ref:
        for name in (f for f in ref.files if f.startswith("mesh")):
            assert ours[name].dtype == ref[name].dtype and ours[name].shape == ref[name].shape, name
            assert ours[name].tobytes() == ref[name].tobytes(), name


def test_leaf_tables_cover_every_node_once():
    packed = pack_library(ShapeLibrary(shapes()), 1e-3)
    ranges = packed["meshClusterRanges"]
    for shape, (first, count, _, _) in enumerate(packed["meshLeafInfo"]):
        leaves = packed["meshLeaves"][first:first + count]
        assert np.all(ranges[leaves, 1] > 0) and np.all(ranges[leaves, 1] <= 64)
        keys = np.concatenate([packed["meshSampleIndices"][ranges[c, 0]:ranges[c, 0] + ranges[c, 1]] for c in leaves])
        assert sorted(keys.tolist()) == list(range(len(shapes()[shape].samples)))
        rank = packed["meshSampleRank"][np.cumsum([0] + [len(s.samples) for s in shapes()])[shape]:][: len(keys)]
        assert np.array_equal(np.sort(rank), np.arange(len(keys)))


@pytest.fixture(scope="module")
def reference_layout():
    with np.load(GOLDEN / "layout.npz") as z:
        return {k: z[k] for k in z.files}


def test_engine_setup_matches_reference(reference_layout):
    ref = reference_layout
    library = ShapeLibrary(shapes()[:2])
    spec = Experiment(particles=64, contact_geometry="mesh", timestep=1e-9, friction=0.4, normal_viscosity=3e5,
                      contacts_per_particle=64, pairs_per_particle=16)
    h = HostLayout(library, spec, ref["positions"], ref["cell"], ref["ids"], ref["scales"])
    units = json.loads(str(ref["units"]))
    for name in ("length_unit", "time_unit", "mass_unit", "force_unit", "stress_unit", "energy_unit", "skin",
                 "cutoff"):
        assert getattr(h, name) == pytest.approx(units[name], rel=1e-15), name
    for name in ("pair_capacity", "contact_capacity", "hash_size", "bin_count", "bin_capacity"):
        assert getattr(h, name) == units[name], name
    assert h.bins.tolist() == units["bins"]
    config = json.loads(str(ref["config"]))
    ours = h.config(dt=spec.timestep, history=False)
    for key, value in config.items():
        if key == "bins":
            assert [ours["bins0"], ours["bins1"], ours["bins2"]] == value
        else:
            assert np.float32(ours[key]) == np.float32(value), key
    state = h.initial_state()
    arrays = dict(h.geometry)
    arrays.update(state)
    for name in ("position", "positionRemainder", "body", "invI", "cell", "referenceCell", "control", "shapeId",
                 "rotation", "sample", "sampleInfo", *REFERENCE_ARRAYS):
        expected = ref["buffer_" + name]
        assert np.ascontiguousarray(arrays[name]).view(np.uint8).reshape(-1).tobytes() == expected.tobytes(), name
