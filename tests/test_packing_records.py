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
