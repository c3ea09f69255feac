"""The backend's derived BVH records agree bit for bit with the packed tree."""

import numpy as np

from sand_atlas_dem_gb300.packing import LEAF_MARK, pack_library
from sand_atlas_dem_gb300.shapes import synthetic_library


def test_child_records_copy_children_bounds_and_links():
    g = pack_library(synthetic_library("f4", 3), 1e-3)
    links, low, high = g["meshLinks"], g["meshMin"], g["meshMax"]
    rec = g["meshChildren"].reshape(-1, 4, 4)
    bits = rec.view(np.uint32)
    assert len(rec) == len(links)
    for node in range(len(links)):
        if links[node, 2] == 0:
            a, b = node + 1, int(links[node + 1, 0])
            assert bits[node, 0, 3] == b
            for k, (src, row) in enumerate(((low, a), (high, a), (low, b), (high, b))):
                assert rec[node, k, :3].tobytes() == src[row, :3].tobytes()
        else:
            assert bits[node, 0, 3] == LEAF_MARK
            assert bits[node, 0, 0] == links[node, 1] and bits[node, 0, 1] == links[node, 2]


def test_tiled_packing_repeats_every_grain_by_whole_cells():
    """``tile_packing``: 2 x 2 x 2 copies shifted by whole cells in a doubled
    cell, so every grain keeps its neighbours (the minimum-image separation
    of any two grains of one copy is the original's) and the solid fraction
    is unchanged."""
    from sand_atlas_dem_gb300.workloads import tile_packing

    rng = np.random.default_rng(3)
    n = 11
    record = dict(positions=rng.uniform(0, 1, (n, 3)) * [2.0, 3.0, 4.0], cell=np.array([2.0, 3.0, 4.0]),
                  rotations=rng.normal(size=(n, 4)).astype(np.float32), ids=rng.integers(0, 5, n).astype(np.uint32),
                  scales=rng.uniform(0.8, 1.2, n), meta={"achieved_solid_fraction": 0.5})
    t = tile_packing(record)
    assert t["positions"].shape == (8 * n, 3) and np.array_equal(t["cell"], 2 * record["cell"])
    assert np.array_equal(t["ids"], np.tile(record["ids"], 8)) and np.array_equal(t["scales"], np.tile(record["scales"], 8))
    assert np.array_equal(t["rotations"], np.tile(record["rotations"], (8, 1)))
    for copy in range(8):
        block = t["positions"][copy * n:(copy + 1) * n]
        shift = block - record["positions"]
        assert np.allclose(shift, shift[0]) and np.allclose(np.round(shift[0] / record["cell"]) * record["cell"], shift[0])
        d = block[:, None, :] - block[None, :, :]
        d0 = record["positions"][:, None, :] - record["positions"][None, :, :]
        d0 -= np.round(d0 / record["cell"]) * record["cell"]
        # Within the doubled cell the nearest image of a same-copy pair may be
        # in a neighbouring copy: compare the separations modulo the small cell.
        d -= np.round(d / record["cell"]) * record["cell"]
        assert np.allclose(d, d0)


def test_edge_key_unique_orders_as_row_unique():
    """The packer takes the unique undirected edges through one int64 key
    per edge (low * stride + high); it must give the rows, inverse and counts
    np.unique(rows, axis=0) gives (``mesh.py:115-121``)."""
    rng = np.random.default_rng(17)
    for vertices in (5, 300, 70_000):
        edges = np.sort(rng.integers(0, vertices, (4_000, 2)), axis=1)
        stride = int(edges.max()) + 1
        keys, inverse, count = np.unique(edges[:, 0] * stride + edges[:, 1], return_inverse=True,
                                         return_counts=True)
        rows = np.column_stack([keys // stride, keys % stride])
        ref_rows, ref_inverse, ref_count = np.unique(edges, axis=0, return_inverse=True, return_counts=True)
        assert np.array_equal(rows, ref_rows)
        assert np.array_equal(inverse.ravel(), ref_inverse.ravel())
        assert np.array_equal(count, ref_count)
