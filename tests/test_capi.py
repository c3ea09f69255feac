"""The C ABI library loads and exports every entry point the header declares.

No compute call is made here (no GPU needed); the symbol set and the buffer
and value counts are checked against ``include/sand_dem_gb300.h`` and the
host-side buffer order.
"""

import ctypes as ct
import re
from pathlib import Path

import pytest

from sand_atlas_dem_gb300 import native
from sand_atlas_dem_gb300.engine import BUFFER_ORDER, EXTENSION_ORDER, TUNING_KEYS
from sand_atlas_dem_gb300.model import CONFIG_ORDER, RESOURCE_ORDER

HEADER = Path(__file__).resolve().parent.parent / "include" / "sand_dem_gb300.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(sdg_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    if not native.LIBRARY.exists():
        native.build()
    return ct.CDLL(str(native.LIBRARY))


def test_header_and_exports_agree(library):
    names = declared()
    assert set(names) == set(native.EXPORTS)
    for name in names:
        assert hasattr(library, name), name


def test_buffer_and_value_counts(library):
    text = HEADER.read_text()
    buffers = int(re.search(r"#define SDG_BUFFER_COUNT (\d+)", text)[1])
    values = int(re.search(r"#define SDG_VALUE_COUNT (\d+)", text)[1])
    library.sdg_buffer_count.restype = ct.c_int
    library.sdg_value_count.restype = ct.c_int
    assert library.sdg_buffer_count() == buffers == len(BUFFER_ORDER) == len(RESOURCE_ORDER) + len(EXTENSION_ORDER)
    assert library.sdg_value_count() == values == len(CONFIG_ORDER) + 5 + len(TUNING_KEYS) + 3
    assert len(RESOURCE_ORDER) == 77


def test_argument_errors_are_reported_without_a_device(library):
    lib = native.load()
    rc = lib.sdg_dispatch(b"beginStep", 1, None, None, None, 0, None)
    assert rc == 1
    assert b"buffers" in lib.sdg_last_error()


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setattr(native, "_LIB", None)
    monkeypatch.setattr(native, "LIBRARY", tmp_path / "absent.so")
    with pytest.raises(RuntimeError, match="not built"):
        native.load()


def test_host_sizes_match_device_constants():
    """Buffer sizes the host computes use the device layout's constants."""
    from sand_atlas_dem_gb300 import engine

    text = (native.CSRC / "dem_device.cuh").read_text()
    cells = int(re.search(r"constexpr uint32_t WALK_CELLS = (\d+);", text)[1])
    grid = int(re.search(r"constexpr uint32_t GRID = (\d+);", text)[1])
    assert engine.WALK_BUCKETS == cells**3
    assert engine.DISTANCE_GRID == grid


def test_plane_configurations_are_checked_before_any_launch(library):
    """Planes bound one nonperiodic specimen, and their buffers must hold the
    (wall, grain) rows: rejected in argument checking, with no device touched."""
    lib = native.load()
    count = len(BUFFER_ORDER)
    pointers = (ct.c_void_p * count)()
    config = dict.fromkeys(CONFIG_ORDER, 0.0)
    config.update(N=10, shapes=1, pairCapacity=16, contactCapacity=16, binCapacity=4, binCount=1, bins0=1,
                  bins1=1, bins2=1, hashSize=32, dt=1e-3, kn=1.0, wallCount=2, periodic=1.0)
    extra = dict(leafWords=1.0, candidateCapacity=1.0, viscousCapture=0.0, specimens=1.0, cullerEnabled=0.0)

    def dispatch(config, extra, sizes):
        values = [config[k] for k in CONFIG_ORDER] + list(extra.values()) + [0.0] * len(TUNING_KEYS) + [1.0, 0.0, 0.0]
        rc = lib.sdg_dispatch(b"step", 10, pointers, (ct.c_uint64 * count)(*sizes),
                              (ct.c_double * len(values))(*values), len(values), None)
        return rc, lib.sdg_last_error()

    large = [1 << 40] * count
    rc, message = dispatch(config, extra, large)
    assert rc == 1 and b"planes" in message
    rc, message = dispatch(dict(config, periodic=0.0), dict(extra, specimens=2.0), large)
    assert rc == 1 and b"planes" in message
    small = list(large)
    small[BUFFER_ORDER.index("wallRows")] = 16
    rc, message = dispatch(dict(config, periodic=0.0), extra, small)
    assert rc == 1 and b"smaller than its configured capacity" in message
    small = list(large)
    small[BUFFER_ORDER.index("oldWallStart")] = 8
    rc, message = dispatch(dict(config, periodic=0.0), extra, small)
    assert rc == 1 and b"smaller than its configured capacity" in message
    # 3 x planes x grains rows must fit the 32-bit row index.
    rc, message = dispatch(dict(config, periodic=0.0, N=float(1 << 30)), extra, large)
    assert rc == 1 and b"2^32" in message


@pytest.mark.parametrize("leaf", [4, 64])
def test_tree_node_counts_match_the_recursion(leaf):
    """``sdg_median_tree_nodes`` (host arithmetic, no device call) against the
    node count of the reference recursion on the same item count."""
    import numpy as np

    from sand_atlas_dem_gb300.packing import host_median_trees

    lib = native.load()
    rng = np.random.default_rng(leaf)
    for n in (1, leaf, leaf + 1, 2 * leaf + 1, 257, 1000, 4099):
        _, records, _, _ = host_median_trees([(rng.normal(size=(n, 3)).astype(np.float32), None, None)], leaf)
        assert lib.sdg_median_tree_nodes(n, leaf) == len(records) == records[0, 0]
    assert lib.sdg_median_tree_nodes(0, leaf) == 0


def test_tree_scratch_rejects_empty_shapes():
    import numpy as np

    lib = native.load()
    counts = np.array([10, 0, 5], np.uint32)
    assert lib.sdg_median_trees_scratch(counts.ctypes.data_as(ct.c_void_p), 3, 64) == 0
    assert b"no items" in lib.sdg_last_error()
    counts = np.array([10, 3000], np.uint32)
    assert lib.sdg_median_trees_scratch(counts.ctypes.data_as(ct.c_void_p), 2, 64) > 0


@pytest.mark.parametrize("leaf", [4, 64])
def test_tree_level_plan_matches_the_recursion(leaf):
    """``trees.tree_levels`` (items per level, in internal nodes, small and
    large internal nodes) against the depths and sizes of the host recursion's
    nodes, for several shapes at once."""
    import numpy as np

    from sand_atlas_dem_gb300.packing import host_median_trees
    from sand_atlas_dem_gb300.trees import tree_launches, tree_levels

    rng = np.random.default_rng(leaf + 1)
    counts = [1, leaf + 1, 300, 2049, 5000]
    items = [(rng.normal(size=(n, 3)).astype(np.float32), None, None) for n in counts]
    _, records, _, _ = host_median_trees(items, leaf)
    sizes = np.zeros(len(records), np.int64)
    # A node's item count: the leaves' counts summed over its subtree.
    for node in range(len(records) - 1, -1, -1):
        escape = int(records[node, 0])
        sizes[node] = records[node, 2] if records[node, 2] else sizes[node + 1] + sizes[int(records[node + 1, 0])]
        assert escape > node
    expected = {}
    for node, size in enumerate(sizes):
        d = int(records[node, 3])
        level = expected.setdefault(d, [0, 0, 0, 0])
        level[0] += size
        if size > leaf:
            level[1] += size
            level[2 if size <= 256 else 3] += 1
    assert [tuple(expected[d]) for d in sorted(expected)] == tree_levels(counts, leaf)
    # Iota and local-row kernels, then per level: reduce, nodes, and the small
    # sort and four radix passes (count, offsets, scatter) where present.
    assert tree_launches(counts, leaf) >= 2 + 2 * len(expected)


def test_tree_builder_rejects_bad_arguments_before_any_device_call():
    """``sdg_median_trees`` checks its arguments on the host and returns 1
    with a message, launching nothing: empty shapes, more than 2^30 items,
    null buffers, boxes given for only one side, scratch too small."""
    import numpy as np

    lib = native.load()
    P = ct.c_void_p
    fake = P(256)  # never dereferenced: every call below fails its checks first

    def call(counts, leaf=64, keys=fake, low=None, high=None, order=fake, scratch=fake, size=1 << 40):
        c = np.asarray(counts, np.uint32)
        return lib.sdg_median_trees(keys, low, high, c.ctypes.data_as(P), len(c), leaf, order, fake, fake, fake,
                                    scratch, size, None)

    assert call([5, 0]) == 1 and b"no items" in lib.sdg_last_error()
    assert call([1 << 29, 1 << 29, 1]) == 1 and b"2^30" in lib.sdg_last_error()
    assert call([10], leaf=0) == 1
    assert call([10], keys=None) == 1 and b"null" in lib.sdg_last_error()
    assert call([10], low=fake) == 1 and b"both" in lib.sdg_last_error()
    assert call([10], order=None) == 1
    assert call([10], size=16) == 1 and b"scratch" in lib.sdg_last_error()
