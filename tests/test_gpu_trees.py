"""The packed layout's median-split trees built on the GPU, against the host
recursion (itself pinned byte for byte to the reference's ``mesh.pack_meshes``
by ``test_layout_golden.py``).

Bit-exact: item order, node records (escape, first, count, depth) and the
outward-rounded FP32 bounds, for single points (the source-node cluster tree,
leaf 64) and boxed items (the triangle BVH, leaf 4); sizes on both sides of
every threshold of the device builder (leaf, the 256-item shared-memory sort,
the 2,048-item radix tile, the 8,192-item reduction piece); many ties and
signed zeros; several shapes in one call; and whole packed libraries.
"""

import numpy as np
import pytest

from sand_atlas_dem_gb300.packing import host_median_trees, pack_library
from sand_atlas_dem_gb300.shapes import ShapeLibrary, synthetic_library
from sand_atlas_dem_gb300.trees import device_median_trees

pytestmark = pytest.mark.gpu


def same(a, b):
    assert len(a) == len(b) == 4
    for x, y, name in zip(a, b, ("order", "records", "low", "high")):
        assert x.dtype == y.dtype and x.shape == y.shape, name
        assert x.tobytes() == y.tobytes(), name


def cloud(rng, n, ties):
    p = rng.normal(size=(n, 3)).astype(np.float32)
    if ties:
        p = np.round(p * 4) / 4  # many equal coordinates, exact zeros
        p[::5] *= -1  # some -0.0
    return p.astype(np.float32)


SIZES = [1, 4, 5, 64, 65, 129, 256, 257, 2048, 2049, 8192, 8193, 20000]


@pytest.mark.parametrize("ties", [False, True])
def test_point_trees_match_host(gpu_library, ties):
    rng = np.random.default_rng(7 + ties)
    for n in SIZES:
        items = [(cloud(rng, n, ties), None, None)]
        same(device_median_trees(items, 64), host_median_trees(items, 64))


@pytest.mark.parametrize("ties", [False, True])
def test_box_trees_match_host(gpu_library, ties):
    rng = np.random.default_rng(11 + ties)
    for n in SIZES:
        centre = cloud(rng, n, ties)
        half = np.abs(cloud(rng, n, ties)) * np.float32(0.1)
        items = [(centre, centre - half, centre + half)]
        same(device_median_trees(items, 4), host_median_trees(items, 4))


def test_many_shapes_in_one_call(gpu_library):
    """Shapes of different depths share every level's launches."""
    rng = np.random.default_rng(5)
    sizes = [1, 3000, 65, 40000, 7, 257, 9000]
    items = [(cloud(rng, n, k % 2 == 1), None, None) for k, n in enumerate(sizes)]
    same(device_median_trees(items, 64), host_median_trees(items, 64))
    boxes = [(c, c - np.float32(0.01), c + np.float32(0.02)) for c, _, _ in items]
    same(device_median_trees(boxes, 4), host_median_trees(boxes, 4))


def test_large_shape(gpu_library):
    """300,000 nodes: 37 reduction pieces and 147 radix tiles at the root."""
    rng = np.random.default_rng(3)
    items = [(cloud(rng, 300_000, True), None, None)]
    same(device_median_trees(items, 64), host_median_trees(items, 64))


@pytest.mark.parametrize("kind,count", [("uneven", 12), ("f8", 4)])
def test_packed_library_matches_host(gpu_library, kind, count):
    library = synthetic_library(kind, count)
    host = pack_library(library, 1e-3)
    device = pack_library(library, 1e-3, trees=device_median_trees)
    assert set(host) == set(device)
    for name in host:
        assert host[name].dtype == device[name].dtype and host[name].shape == device[name].shape, name
        assert host[name].tobytes() == device[name].tobytes(), name


def test_golden_tree_shapes_on_device(gpu_library):
    """The reference's own trees (``golden/packing_trees.npz``)."""
    from pathlib import Path

    from tests.golden.make_golden import stored_tree_shapes

    packed = pack_library(ShapeLibrary(stored_tree_shapes()), 1e-3, trees=device_median_trees)
    with np.load(Path(__file__).resolve().parent / "golden" / "packing_trees.npz") as ref:
        for name in (f for f in ref.files if f.startswith("mesh")):
            assert packed[name].tobytes() == ref[name].tobytes(), name


def test_rejects_nonfinite_and_mixed_boxes(gpu_library):
    p = np.zeros((10, 3), np.float32)
    bad = p.copy()
    bad[3, 1] = np.nan
    with pytest.raises(ValueError):
        device_median_trees([(bad, None, None)], 64)
    with pytest.raises(ValueError):
        device_median_trees([(p, p, p), (p, None, None)], 4)
