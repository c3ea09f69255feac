"""Packed static mesh layout read by the device kernels (host side, run once).

The layout is the reference's contract (``src/sand_atlas_dem/mesh.py:10-222``),
kept array-for-array identical because the contact key of a node (its sample
index) and every FP32 bound enter the exact contact decision:

* per shape, a preorder source-node cluster tree (<= 64 nodes per leaf, split
  at the median of the widest axis, escape links; ``mesh.py:33-56``) and a
  32-root frontier of disjoint subtrees (``mesh.py:59-70``);
* outward-rounded convex-hull planes in six dominant-axis groups
  (``mesh.py:74-90``);
* manifold/winding checks and angle-weighted feature pseudonormals, 7 per
  triangle (face, 3 edges, 3 vertices; ``mesh.py:91-158``);
* a median-split triangle BVH (<= 4 triangles per leaf, depth <= 30) in
  preorder with escape links (``mesh.py:164-201``).

Two arrays are added for this backend and have no reference counterpart:
``meshLeafInfo`` (per shape: first leaf slot, leaf count) and ``meshLeaves``
(leaf cluster ids in preorder), which let the collector cull all leaves of a
shape in parallel; and ``meshSampleRank`` (per packed sample: its position in
``meshSampleIndices``), the in-pair sort key of the friction-history merge;
and ``meshChildren``, the triangle BVH re-laid as one record per node holding
both children's bounds (see :func:`child_records`).
"""

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
from scipy.sparse import coo_matrix
from scipy.sparse.csgraph import connected_components
from scipy.spatial import ConvexHull

F32 = np.float32
UINT_ARRAYS = (
    "meshFrontier",
    "meshClusterInfo",
    "meshClusterRanges",
    "meshSampleIndices",
    "meshHullInfo",
    "meshRoots",
    "meshLinks",
)
FLOAT_ARRAYS = (
    "meshClusterMin",
    "meshClusterMax",
    "meshPlanes",
    "meshMin",
    "meshMax",
    "meshTriangles",
    "meshNormals",
)


def _down(x):
    return np.nextafter(x, F32(-np.inf))


def _up(x):
    return np.nextafter(x, F32(np.inf))


def host_median_trees(items, leaf):
    """Median-split trees over every shape, by the reference's recursion
    (``mesh.py:33-56`` with leaf 64, ``mesh.py:164-201`` with leaf 4): a node
    over more than ``leaf`` items sorts them stably along the axis of largest
    key extent and gives the first half to its left child; its bounds are the
    items' boxes' FP32 minimum and maximum, one ulp outward.

    ``items``: per shape ``(keys, low, high)``, FP32 (n, 3) arrays (``low`` and
    ``high`` None: the boxes are the key points).  Returns ``order`` (per
    position, the item's row within its shape; shapes one after another),
    ``records`` (per preorder node: escape index, first position and count of
    a leaf or 0, 0, depth) and the node bounds ``low``/``high`` (nodes, 4).
    :func:`device_median_trees` (``trees.py``) builds the same on the GPU.
    """
    records, low_out, high_out, order = [], [], [], []
    for keys, low, high in items:
        keys = np.asarray(keys, F32)
        low = keys if low is None else np.asarray(low, F32)
        high = keys if high is None else np.asarray(high, F32)

        def split(ids, depth):
            node = len(records)
            records.append([0, 0, 0, depth])
            low_out.append(_down(low[ids].min(0)))
            high_out.append(_up(high[ids].max(0)))
            if len(ids) > leaf:
                k = keys[ids]
                axis = np.ptp(k, axis=0).argmax()
                ids = ids[np.argsort(k[:, axis], kind="stable")]
                half = len(ids) // 2
                split(ids[:half], depth + 1)
                split(ids[half:], depth + 1)
            else:
                records[node][1] = len(order)
                records[node][2] = len(ids)
                order.extend(ids.tolist())
            records[node][0] = len(records)

        split(np.arange(len(keys)), 0)

    def rows(a):
        return np.pad(np.asarray(a, F32).reshape(-1, 3), ((0, 0), (0, 1)))

    return np.asarray(order, np.uint32), np.asarray(records, np.uint32).reshape(-1, 4), rows(low_out), rows(high_out)


def _frontier(ranges, base):
    """Up to 32 disjoint complete subtrees; split the largest internal first."""
    pending = [0]
    while len(pending) < 32:
        internal = [n for n in pending if ranges[n][1] == 0]
        if not internal:
            break
        node = max(internal, key=lambda n: ranges[n][2] - n)
        at = pending.index(node)
        pending[at : at + 1] = [node + 1, ranges[node + 1][2]]
    rows = [[base + n, base + ranges[n][2], 0, 0] for n in pending]
    return rows + [[0, 0, 0, 0]] * (32 - len(rows))


def _hull_groups(vertices):
    rounded = vertices.astype(F32).astype(float)
    hull = ConvexHull(rounded)
    margin = 16 * np.finfo(F32).eps * (1 + abs(rounded).max())
    planes = hull.equations.astype(F32)
    planes[:, 3] = _down((hull.equations[:, 3] - margin).astype(F32))
    planes = np.unique(planes, axis=0)
    n = planes[:, :3]
    dominant = np.abs(n).argmax(axis=1)
    group = 2 * dominant + (n[np.arange(len(n)), dominant] >= 0)
    return [planes[group == g] for g in range(6)]


def _feature_normals(vertices, faces):
    tri = vertices[faces]
    cross = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    norm = np.linalg.norm(cross, axis=1)
    if np.any(norm <= 0):
        raise ValueError("Degenerate source triangle")
    face_normal = cross / norm[:, None]
    corner_angle = []
    for corner in range(3):
        u = tri[:, (corner + 1) % 3] - tri[:, corner]
        w = tri[:, (corner + 2) % 3] - tri[:, corner]
        corner_angle.append(np.arctan2(np.linalg.norm(np.cross(u, w), axis=1), (u * w).sum(1)))
    angle = np.stack(corner_angle, axis=1)
    vertex_normal = np.zeros_like(vertices)
    np.add.at(vertex_normal, faces.ravel(), (face_normal[:, None, :] * angle[:, :, None]).reshape(-1, 3))
    edges = faces[:, [[0, 1], [1, 2], [2, 0]]].reshape(-1, 2)
    # Unique undirected edges in lexicographic (low, high) order, as
    # np.unique(rows, axis=0) orders them, through one int64 key per edge.
    ordered = np.sort(edges, axis=1)
    stride = int(faces.max()) + 1
    keys, inverse, count = np.unique(ordered[:, 0] * stride + ordered[:, 1], return_inverse=True,
                                     return_counts=True)
    unique = np.column_stack([keys // stride, keys % stride])
    if np.any(count != 2):
        raise ValueError("Mesh query requires exactly two faces per edge")
    direction = np.where(edges[:, 0] < edges[:, 1], 1, -1)
    oriented = np.zeros(len(unique), int)
    np.add.at(oriented, inverse, direction)
    if np.any(oriented):
        raise ValueError("Inconsistent source winding")
    # Each vertex link must be a single cycle of corners.
    occurrence = np.arange(3 * len(faces))
    corner_a = 3 * (occurrence // 3) + occurrence % 3
    corner_b = 3 * (occurrence // 3) + (occurrence % 3 + 1) % 3
    corners = np.stack([corner_a, corner_b], axis=1)
    corners[direction < 0] = corners[direction < 0, ::-1]
    paired = corners[np.argsort(inverse, kind="stable")].reshape(-1, 2, 2)
    graph = coo_matrix(
        (np.ones(paired[:, 0].size), (paired[:, 0].ravel(), paired[:, 1].ravel())),
        shape=(3 * len(faces),) * 2,
    )
    if connected_components(graph, directed=False)[0] != len(np.unique(faces)):
        raise ValueError("Disconnected vertex fans in source mesh")
    edge_normal = np.zeros((len(unique), 3))
    np.add.at(edge_normal, inverse, np.repeat(face_normal, 3, axis=0))
    feature = np.concatenate(
        [face_normal[:, None, :], edge_normal[inverse.reshape(-1, 3)], vertex_normal[faces]], axis=1
    )
    length = np.linalg.norm(feature, axis=2)
    if np.any(length < 1e-12):
        raise ValueError("Undefined mesh feature pseudonormal")
    return feature / length[:, :, None]


def _prepare(shape, length_unit):
    """One shape's host-side parts: FP32 sample points, hull plane groups,
    feature pseudonormals, FP32 triangles (``mesh.py:21-162``) and the
    triangles' split keys and boxes: centres as the reference computes them
    (``mesh.py:191``, the mean of the three FP32 vertices) and the vertices'
    minimum and maximum."""
    if shape.provenance.get("display_mesh_only"):
        raise ValueError("Mesh query requires physical source triangles, not a display-only fixture mesh")
    vertices = np.asarray(shape.vertices, float) / length_unit
    faces = np.asarray(shape.faces, np.int64)
    points = (np.asarray(shape.samples) / length_unit).astype(F32)
    if len(points) == 0 or not np.all(np.isfinite(points)):
        raise ValueError("Shape samples must be finite and nonempty")
    hull = _hull_groups(vertices)
    feature = _feature_normals(vertices, faces)
    tri = vertices[faces].astype(F32)
    if not np.all(np.isfinite(tri)):
        raise ValueError("Shape vertices must be finite")
    if np.any(np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1) == 0):
        raise ValueError("Triangle degenerates in normalized FP32")
    low = np.minimum(np.minimum(tri[:, 0], tri[:, 1]), tri[:, 2])
    high = np.maximum(np.maximum(tri[:, 0], tri[:, 1]), tri[:, 2])
    return points, hull, feature, tri, (tri.mean(axis=1), low, high)


def pack_library(library, length_unit, trees=host_median_trees):
    """Pack every shape; returns uint32/float32 arrays keyed by buffer name.

    ``trees`` builds the two median-split trees of all shapes at once
    (:func:`host_median_trees`, or the GPU builder
    ``trees.device_median_trees``; both give the same bytes).  Triangle
    centres are the mean of the three FP32 vertices, computed per triangle
    as the reference computes them per subset (``mesh.py:191``).
    """
    out = {k: [] for k in UINT_ARRAYS + FLOAT_ARRAYS}
    # The per-shape host work (hull, pseudonormals, manifold checks) is
    # independent between shapes: prepared on a thread pool, kept in order.
    if not library.shapes:
        raise ValueError("Shape library is empty")
    with ThreadPoolExecutor(max_workers=min(len(library.shapes), os.cpu_count() or 1)) as pool:
        prepared = list(pool.map(lambda shape: _prepare(shape, length_unit), library.shapes))
    sample_items, triangle_items, tris, features, planes = [], [], [], [], []
    plane_count = 0
    for points, hull, feature, tri, boxed in prepared:
        sample_items.append((points, None, None))
        for subset in hull:
            out["meshHullInfo"].append([plane_count, len(subset), 0, 0])
            planes.append(subset)
            plane_count += len(subset)
        features.append(feature)
        tris.append(tri)
        triangle_items.append(boxed)
    out["meshPlanes"] = np.concatenate(planes).astype(F32).reshape(-1, 4)

    sample_order, cluster, cluster_low, cluster_high = trees(sample_items, 64)
    tri_order, links, tri_low, tri_high = trees(triangle_items, 4)

    # Per shape: its first cluster, sample, BVH node and triangle (serial,
    # through the roots' escape links), then the per-shape assembly on the
    # thread pool, each shape writing its own slices.
    starts, node, item, bvh, tri_item = [], 0, 0, 0, 0
    for (points, _, _), tri in zip(sample_items, tris):
        starts.append((node, item, bvh, tri_item))
        node = int(cluster[node, 0])
        bvh = int(links[bvh, 0])
        item += len(points)
        tri_item += len(tri)
    ranks = np.empty(len(sample_order), np.uint32)
    triangles = np.zeros((3 * tri_item, 4), F32)
    normals = np.zeros((7 * tri_item, 4), F32)

    def assemble(k):
        node, item, bvh, tri_item = starts[k]
        n = len(sample_items[k][0])
        count = int(cluster[node, 0]) - node  # the root's escape link
        ranges = cluster[node:node + count]
        # (first, count, escape) with the escape link local to the shape.
        local = np.column_stack([ranges[:, 1], ranges[:, 2], ranges[:, 0] - node]).astype(np.int64)
        frontier = _frontier(local, node)
        shape_leaves = node + np.flatnonzero(ranges[:, 2] > 0)
        ranks[item + sample_order[item:item + n].astype(np.int64)] = np.arange(n, dtype=np.uint32)
        tri, feature = tris[k], features[k]
        nodes = int(links[bvh, 0]) - bvh
        depth = int(links[bvh:bvh + nodes, 3].max())
        rows = tri_order[tri_item:tri_item + len(tri)].astype(np.int64)
        triangles[3 * tri_item:3 * (tri_item + len(tri)), :3] = tri[rows].reshape(-1, 3)
        normals[7 * tri_item:7 * (tri_item + len(tri)), :3] = feature[rows].reshape(-1, 3)
        return count, frontier, shape_leaves, nodes, depth

    with ThreadPoolExecutor(max_workers=min(len(library.shapes), os.cpu_count() or 1)) as pool:
        assembled = list(pool.map(assemble, range(len(sample_items))))
    leaf_info, leaves, leaf_total = [], [], 0
    for (node, _, bvh, _), (count, frontier, shape_leaves, nodes, depth) in zip(starts, assembled):
        out["meshClusterInfo"].append([node, count, 0, 0])
        out["meshFrontier"].extend(frontier)
        leaf_info.append([leaf_total, len(shape_leaves), 0, 0])
        leaves.append(shape_leaves)
        leaf_total += len(shape_leaves)
        if depth > 30:
            raise ValueError("Mesh hierarchy exceeds GPU traversal stack depth")
        out["meshRoots"].append([bvh, bvh + nodes, depth, 0])
    out["meshClusterRanges"] = np.column_stack(
        [cluster[:, 1], cluster[:, 2], cluster[:, 0], np.zeros(len(cluster), np.uint32)])
    out["meshClusterMin"] = cluster_low
    out["meshClusterMax"] = cluster_high
    out["meshSampleIndices"] = sample_order
    out["meshLinks"] = np.column_stack([links[:, :3], np.zeros(len(links), np.uint32)])
    out["meshMin"] = tri_low
    out["meshMax"] = tri_high

    packed = {}
    for name in UINT_ARRAYS:
        packed[name] = np.ascontiguousarray(np.asarray(out[name], np.uint32))
    out["meshTriangles"], out["meshNormals"] = triangles, normals
    for name in FLOAT_ARRAYS:
        packed[name] = np.ascontiguousarray(np.asarray(out[name], F32))
    packed["meshLeafInfo"] = np.asarray(leaf_info, np.uint32)
    packed["meshLeaves"] = np.concatenate(leaves).astype(np.uint32)
    packed["meshSampleRank"] = ranks
    packed["meshChildren"] = child_records(packed["meshLinks"], packed["meshMin"], packed["meshMax"])
    return packed


LEAF_MARK = np.uint32(0xFFFFFFFF)


def child_records(links, low, high):
    """One 64-byte record per triangle-BVH node, read by the exact walk in a
    single round of loads.  Internal node n (children a = n + 1 and b = the
    escape link of a): (low[a], b), (high[a], 0), (low[b], 0), (high[b], 0),
    the bounds copied bit for bit.  Leaf: (first triangle, count, 0,
    0xFFFFFFFF) as integers, the rest zero."""
    n = len(links)
    records = np.zeros((n, 4, 4), F32)
    bits = records.view(np.uint32)
    internal = links[:, 2] == 0
    nodes = np.flatnonzero(internal)
    a = nodes + 1
    b = links[a, 0].astype(np.int64)
    records[nodes, 0, :3] = low[a, :3]
    records[nodes, 1, :3] = high[a, :3]
    records[nodes, 2, :3] = low[b, :3]
    records[nodes, 3, :3] = high[b, :3]
    bits[nodes, 0, 3] = b
    leaves = np.flatnonzero(~internal)
    bits[leaves, 0, 0] = links[leaves, 1]
    bits[leaves, 0, 1] = links[leaves, 2]
    bits[leaves, 0, 3] = LEAF_MARK
    return records.reshape(-1, 4)


REFERENCE_ARRAYS = UINT_ARRAYS + FLOAT_ARRAYS
