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


class _ClusterTree:
    """Preorder median-split tree over FP32 node coordinates."""

    def __init__(self, points, first_sample):
        self.points = points
        self.ranges, self.low, self.high, self.order = [], [], [], []
        self.first_sample = first_sample
        self._split(np.arange(len(points)))

    def _split(self, ids):
        node = len(self.ranges)
        self.ranges.append([0, 0, 0, 0])
        p = self.points[ids]
        self.low.append([*_down(p.min(0)), 0])
        self.high.append([*_up(p.max(0)), 0])
        if len(ids) > 64:
            axis = np.ptp(p, axis=0).argmax()
            ordered = ids[np.argsort(p[:, axis], kind="stable")]
            half = len(ordered) // 2
            self._split(ordered[:half])
            self._split(ordered[half:])
        else:
            self.ranges[node][0] = self.first_sample + len(self.order)
            self.ranges[node][1] = len(ids)
            self.order.extend(ids.tolist())
        self.ranges[node][2] = len(self.ranges)


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
    unique, inverse, count = np.unique(
        np.sort(edges, axis=1), axis=0, return_inverse=True, return_counts=True
    )
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


class _TriangleTree:
    """Preorder median-split BVH over FP32 triangles (<= 4 per leaf)."""

    def __init__(self, tri, first_node, first_triangle):
        self.tri = tri
        self.first_node, self.first_triangle = first_node, first_triangle
        self.low, self.high, self.links, self.order, self.depth = [], [], [], [], 0
        self._build(np.arange(len(tri)), 0)

    def _build(self, ids, depth):
        node = len(self.links)
        self.depth = max(self.depth, depth)
        t = self.tri[ids]
        self.low.append([*_down(t.min(axis=(0, 1))), 0])
        self.high.append([*_up(t.max(axis=(0, 1))), 0])
        self.links.append([0, 0, 0, 0])
        if len(ids) <= 4:
            self.links[node][1] = self.first_triangle + len(self.order)
            self.links[node][2] = len(ids)
            self.order.extend(ids.tolist())
        else:
            centres = t.mean(axis=1)
            axis = np.ptp(centres, axis=0).argmax()
            ids = ids[np.argsort(centres[:, axis], kind="stable")]
            half = len(ids) // 2
            self._build(ids[:half], depth + 1)
            self._build(ids[half:], depth + 1)
        self.links[node][0] = self.first_node + len(self.links)


def pack_library(library, length_unit):
    """Pack every shape; returns uint32/float32 arrays keyed by buffer name."""
    out = {k: [] for k in UINT_ARRAYS + FLOAT_ARRAYS}
    leaf_info, leaves, ranks = [], [], []
    for shape in library.shapes:
        if shape.provenance.get("display_mesh_only"):
            raise ValueError(
                "Mesh query requires physical source triangles, not a display-only fixture mesh"
            )
        vertices = np.asarray(shape.vertices, float) / length_unit
        faces = np.asarray(shape.faces, np.int64)
        points = (np.asarray(shape.samples) / length_unit).astype(F32)
        base = len(out["meshClusterRanges"])
        tree = _ClusterTree(points, len(out["meshSampleIndices"]))
        ranges = tree.ranges
        out["meshClusterInfo"].append([base, len(ranges), 0, 0])
        out["meshFrontier"].extend(_frontier(ranges, base))
        # Stored escape links are absolute cluster indices.
        out["meshClusterRanges"].extend([[r[0], r[1], base + r[2], 0] for r in ranges])
        out["meshClusterMin"].extend(tree.low)
        out["meshClusterMax"].extend(tree.high)
        out["meshSampleIndices"].extend(tree.order)
        shape_leaves = [base + n for n, r in enumerate(ranges) if r[1] > 0]
        leaf_info.append([len(leaves), len(shape_leaves), 0, 0])
        leaves.extend(shape_leaves)
        rank = np.empty(len(points), np.uint32)
        rank[np.asarray(tree.order, np.int64)] = np.arange(len(points), dtype=np.uint32)
        ranks.append(rank)
        for subset in _hull_groups(vertices):
            out["meshHullInfo"].append([len(out["meshPlanes"]), len(subset), 0, 0])
            out["meshPlanes"].extend(subset)
        feature = _feature_normals(vertices, faces)
        tri = vertices[faces].astype(F32)
        if np.any(np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1) == 0):
            raise ValueError("Triangle degenerates in normalized FP32")
        bvh = _TriangleTree(tri, len(out["meshLinks"]), len(out["meshTriangles"]) // 3)
        if bvh.depth > 30:
            raise ValueError("Mesh hierarchy exceeds GPU traversal stack depth")
        out["meshRoots"].append([bvh.first_node, bvh.first_node + len(bvh.links), bvh.depth, 0])
        out["meshMin"].extend(bvh.low)
        out["meshMax"].extend(bvh.high)
        out["meshLinks"].extend(bvh.links)
        out["meshTriangles"].extend(tri[bvh.order].reshape(-1, 3))
        out["meshNormals"].extend(feature[bvh.order].reshape(-1, 3))

    def f4(a):
        a = np.asarray(a, F32).reshape(-1, 3)
        return np.pad(a, ((0, 0), (0, 1)))

    packed = {}
    for name in UINT_ARRAYS:
        packed[name] = np.asarray(out[name], np.uint32)
    for name in FLOAT_ARRAYS:
        if name in ("meshTriangles", "meshNormals"):
            packed[name] = f4(out[name])
        else:
            packed[name] = np.asarray(out[name], F32)
    packed["meshLeafInfo"] = np.asarray(leaf_info, np.uint32)
    packed["meshLeaves"] = np.asarray(leaves, np.uint32)
    packed["meshSampleRank"] = np.concatenate(ranks).astype(np.uint32)
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
