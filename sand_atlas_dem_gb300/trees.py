"""The packed layout's median-split trees, built on the GPU.

:func:`device_median_trees` has the signature and results of
``packing.host_median_trees`` (the reference's recursions of
``mesh.py:33-56`` and ``mesh.py:164-201``), bit for bit, and runs
``sdg_median_trees`` (``csrc/trees.cu``): every shape's tree at once, level by
level, with the sorts and reductions on the device.  It is what the GB300
engine packs its library with; there is no host fallback here (the call
raises when the CUDA library or device is missing).
"""

import ctypes as ct
import time

import numpy as np

from . import native


def _ptr(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def device_median_trees(items, leaf, *, timing=None):
    """``items``: per shape ``(keys, low, high)``, FP32 (n, 3) arrays, with
    ``low``/``high`` both None (boxes are the key points) or both given for
    every shape.  Returns ``(order, records, low, high)`` as
    ``packing.host_median_trees`` does.  ``timing`` (a dict) receives the
    device time of the build (``device_ms``, CUDA events on the stream) and
    the wall time of the whole call with its copies (``wall_ms``)."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("device_median_trees requires a CUDA device")
    lib = native.load()
    boxes = items[0][1] is not None
    if any((lo is not None) != boxes or (hi is not None) != boxes for _, lo, hi in items):
        raise ValueError("Item boxes must be given for every shape or for none")
    counts = np.array([len(k) for k, _, _ in items], np.uint32)
    if len(counts) == 0 or np.any(counts == 0):
        raise ValueError("Every shape needs at least one item")
    n = int(counts.sum(dtype=np.uint64))
    device = torch.device("cuda", torch.cuda.current_device())
    wall = time.perf_counter()
    firsts = np.cumsum(counts, dtype=np.int64) - counts

    def rows(arrays):
        # Each shape's (n, 3) rows go straight into one padded device array.
        out = torch.zeros((n, 4), dtype=torch.float32, device=device)
        for first, x in zip(firsts, arrays):
            x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
            if not np.all(np.isfinite(x)):
                raise ValueError("Item coordinates must be finite")
            out[first:first + len(x), :3] = torch.from_numpy(x).to(device, non_blocking=False)
        return out

    keys = rows([k for k, _, _ in items])
    low = rows([lo for _, lo, _ in items]) if boxes else None
    high = rows([hi for _, _, hi in items]) if boxes else None
    nodes = sum(int(lib.sdg_median_tree_nodes(int(c), leaf)) for c in counts)
    order = torch.empty(n, dtype=torch.int32, device=device)
    records = torch.empty((nodes, 4), dtype=torch.int32, device=device)
    node_low = torch.empty((nodes, 4), dtype=torch.float32, device=device)
    node_high = torch.empty((nodes, 4), dtype=torch.float32, device=device)
    counts_ptr = counts.ctypes.data_as(ct.c_void_p)
    size = int(lib.sdg_median_trees_scratch(counts_ptr, len(counts), leaf))
    if size == 0:
        native.check(1)
    scratch = torch.empty(size, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device)
    start = end = None
    if timing is not None:
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
    native.check(lib.sdg_median_trees(_ptr(keys), _ptr(low), _ptr(high), counts_ptr, len(counts), leaf,
                                      _ptr(order), _ptr(records), _ptr(node_low), _ptr(node_high), _ptr(scratch),
                                      size, ct.c_void_p(stream.cuda_stream)))
    if timing is not None:
        end.record(stream)
        end.synchronize()
        timing["device_ms"] = start.elapsed_time(end)
    out = (order.cpu().numpy().view(np.uint32), records.cpu().numpy().view(np.uint32), node_low.cpu().numpy(), node_high.cpu().numpy())
    if timing is not None:
        timing["wall_ms"] = 1e3 * (time.perf_counter() - wall)
    return out

def tree_levels(counts, leaf, small=256):
    """Per level of the trees over shapes of ``counts`` items: items in the
    level's nodes, items in its internal nodes, and its internal nodes of at
    most ``small`` items and of more (the device builder's shared-memory and
    radix sorts).  A node's size alone decides its children's, so each
    shape's level is at most two (size, number) pairs."""
    levels = []
    for c in counts:
        sizes = {int(c): 1}
        d = 0
        while sizes:
            if len(levels) <= d:
                levels.append([0, 0, 0, 0])
            nxt = {}
            for size, mult in sizes.items():
                levels[d][0] += size * mult
                if size > leaf:
                    levels[d][1] += size * mult
                    levels[d][2 if size <= small else 3] += mult
                    for half in (size // 2, size - size // 2):
                        nxt[half] = nxt.get(half, 0) + mult
            sizes = nxt
            d += 1
    return [tuple(level) for level in levels]


def tree_launches(counts, leaf):
    """Kernel launches of one ``sdg_median_trees`` call."""
    return 2 + sum(2 + (small > 0) + 12 * (large > 0) for _, _, small, large in tree_levels(counts, leaf))
