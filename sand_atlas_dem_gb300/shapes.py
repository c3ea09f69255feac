"""Grain shapes for the mesh-surface contact method (host side, run once).

A :class:`Shape` carries the fields the mesh path of the reference reads from a
shape asset (``src/sand_atlas_dem/geometry.py:17-29``): triangle mesh, surface
quadrature nodes with area weights, volume, unit-density inertia and bounding
radius.  Lengths are metres.  Signed-distance grids are not carried: this
backend implements the mesh contact geometry only.

The synthetic library follows the seeded recipe used for the benchmark
workloads: geodesic icospheres of frequency ``nu`` (T = 20 nu^2 triangles,
V = 10 nu^2 + 2 vertices), vertex radii perturbed by N(0, 0.08) R, optional
axis ratios, V surface nodes drawn by the scrambled-Sobol area recipe of
``geometry.py:219-232`` with equal area weights, and mass properties from the
divergence theorem.
"""

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Shape:
    id: str
    vertices: np.ndarray
    faces: np.ndarray
    samples: np.ndarray
    areas: np.ndarray
    volume: float
    inertia: np.ndarray
    radius: float
    provenance: dict = field(default_factory=dict)

    def validate(self):
        """Checks of ``geometry.py:32-58`` that apply without an SDF grid."""
        for a in (self.vertices, self.samples, self.areas, self.inertia):
            if not np.isfinite(a).all():
                raise ValueError("Nonfinite shape data")
        if self.volume <= 0 or self.radius <= 0 or np.any(self.areas <= 0):
            raise ValueError("Invalid shape measure")
        if len(self.samples) != len(self.areas) or self.samples.shape[1:] != (3,):
            raise ValueError("Invalid surface samples")
        if np.linalg.eigvalsh(self.inertia).min() <= 0:
            raise ValueError("Inertia is not positive definite")


class ShapeLibrary:
    """Ordered, uniquely identified shapes (``geometry.py:106-112``)."""

    def __init__(self, shapes):
        self.shapes = list(shapes)
        if not self.shapes or len({s.id for s in self.shapes}) != len(self.shapes):
            raise ValueError("Shape library must contain uniquely identified shapes")
        for shape in self.shapes:
            shape.validate()


def mass_properties(vertices, faces):
    """Volume, centre of mass and unit-density inertia about the centre of mass.

    Signed tetrahedra from the origin (divergence theorem); exact for a closed,
    outward-wound triangle mesh.
    """
    v = np.asarray(vertices, float)
    tri = v[np.asarray(faces)]
    a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
    det = np.einsum("ij,ij->i", a, np.cross(b, c))
    volume = det.sum() / 6.0
    centre = (det[:, None] * (a + b + c)).sum(0) / (24.0 * volume)
    # Second moments of each tetrahedron (0, a, b, c): integral of x_i x_j.
    s = a + b + c
    second = (
        np.einsum("n,ni,nj->ij", det, a, a)
        + np.einsum("n,ni,nj->ij", det, b, b)
        + np.einsum("n,ni,nj->ij", det, c, c)
        + np.einsum("n,ni,nj->ij", det, s, s)
    ) / 120.0
    second -= volume * np.outer(centre, centre)
    inertia = np.trace(second) * np.eye(3) - second
    return float(volume), centre, inertia


def icosphere(frequency):
    """Geodesic unit sphere: 20 f^2 outward-wound triangles, 10 f^2 + 2 vertices."""
    t = (1.0 + 5.0**0.5) / 2.0
    base = np.array(
        [
            [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
            [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
            [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1],
        ],
        float,
    )
    base /= np.linalg.norm(base, axis=1)[:, None]
    ico = np.array(
        [
            [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
            [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
            [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
            [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
        ]
    )
    f = int(frequency)
    index = {}
    points = []

    def vertex(face, i, j):
        # Lattice point a + (b-a) i/f + (c-a) j/f keyed canonically so shared
        # edge and corner points are created once.
        a, b, c = ico[face]
        k = f - i - j
        weights = {a: k, b: i, c: j}
        key = tuple(sorted((int(v), int(w)) for v, w in weights.items() if w))
        if key not in index:
            p = sum(base[v] * w for v, w in key) / f
            index[key] = len(points)
            points.append(p / np.linalg.norm(p))
        return index[key]

    faces = []
    for face in range(20):
        for i in range(f):
            for j in range(f - i):
                p0, p1, p2 = vertex(face, i, j), vertex(face, i + 1, j), vertex(face, i, j + 1)
                faces.append([p0, p1, p2])
                if i + j < f - 1:
                    p3 = vertex(face, i + 1, j + 1)
                    faces.append([p1, p3, p2])
    vertices = np.array(points)
    faces = np.array(faces, np.int64)
    # Orient every face outward.
    tri = vertices[faces]
    normal = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    flip = np.einsum("ij,ij->i", normal, tri.mean(1)) < 0
    faces[flip] = faces[flip][:, ::-1]
    return vertices, faces


def surface_nodes(vertices, faces, count, seed):
    """Scrambled-Sobol area sampling with equal weights (``geometry.py:219-232``)."""
    from scipy.stats import qmc

    tri = np.asarray(vertices, float)[faces]
    area = 0.5 * np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1)
    total = area.sum()
    u = qmc.Sobol(3, scramble=True, seed=seed).random_base2(int(np.ceil(np.log2(count))))[:count]
    face = np.searchsorted(np.cumsum(area) / total, u[:, 0], side="right")
    face = np.minimum(face, len(faces) - 1)
    t = tri[face]
    root = np.sqrt(u[:, 1])
    v = u[:, 2]
    points = (
        (1 - root[:, None]) * t[:, 0]
        + (root * (1 - v))[:, None] * t[:, 1]
        + (root * v)[:, None] * t[:, 2]
    )
    return points, np.full(count, total / count)


def perturbed_grain(frequency, *, radius=5e-4, sigma=0.08, axes=(1.0, 1.0, 1.0), seed=1000,
                    shape_id=None, nodes=None):
    """One seeded grain: perturbed geodesic icosphere, nodes per vertex count.

    Vertex radii are ``radius * (1 + eps)``, eps ~ N(0, sigma) (clipped to keep
    the surface star-shaped), then scaled by the axis ratios.  The mesh is
    translated to its centre of mass, as ``geometry.py:193-195`` does.
    """
    rng = np.random.default_rng(seed)
    unit, faces = icosphere(frequency)
    eps = np.clip(rng.normal(0.0, sigma, len(unit)), -0.5, 0.5)
    vertices = unit * (radius * (1.0 + eps))[:, None] * np.asarray(axes, float)
    volume, centre, _ = mass_properties(vertices, faces)
    vertices = vertices - centre
    volume, _, inertia = mass_properties(vertices, faces)
    count = len(vertices) if nodes is None else int(nodes)
    samples, areas = surface_nodes(vertices, faces, count, seed)
    return Shape(
        shape_id or f"icosphere-f{frequency}-s{seed}",
        vertices,
        faces,
        samples,
        areas,
        volume,
        inertia,
        float(np.linalg.norm(vertices, axis=1).max()),
        dict(
            generator="perturbed-geodesic-icosphere",
            frequency=int(frequency),
            radius_m=radius,
            sigma=sigma,
            axes=[float(a) for a in axes],
            seed=int(seed),
            sampling="scrambled_sobol_area",
            sample_count=count,
        ),
    )


def synthetic_library(kind, count=64, *, seed=1000, radius=5e-4):
    """Seeded 64-shape libraries of the benchmark workloads.

    ``kind`` is ``"f4"`` (320 triangles, 162 nodes), ``"f8"`` (1,280 / 642) or
    ``"uneven"`` (log-uniform 320..5,120 triangles, axis ratios U(0.6, 1)).
    """
    shapes = []
    for k in range(count):
        s = seed + k
        if kind == "f4":
            shapes.append(perturbed_grain(4, radius=radius, seed=s))
        elif kind == "f8":
            shapes.append(perturbed_grain(8, radius=radius, seed=s))
        elif kind == "uneven":
            rng = np.random.default_rng(s + 7919)
            t = np.exp(rng.uniform(np.log(320), np.log(5120)))
            frequency = int(np.clip(round((t / 20) ** 0.5), 4, 16))
            axes = rng.uniform(0.6, 1.0, 3)
            shapes.append(perturbed_grain(frequency, radius=radius, axes=axes, seed=s))
        else:
            raise ValueError("Unknown synthetic library kind")
    return ShapeLibrary(shapes)


def box_shape(extents, *, nodes=None, shape_id="box"):
    """Closed box mesh (12 outward triangles) with optional explicit nodes.

    Used for the exact six-node cube known-answer cases of the reference
    tests (``tests/test_cpu_solver.py:105-118``).
    """
    e = np.asarray(extents, float) / 2
    v = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], float) * e
    faces = np.array(
        [
            [0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5],
            [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
            [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3],
        ],
        np.int64,
    )
    tri = v[faces]
    normal = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    flip = np.einsum("ij,ij->i", normal, tri.mean(1)) < 0
    faces[flip] = faces[flip][:, ::-1]
    volume, _, inertia = mass_properties(v, faces)
    if nodes is None:
        samples, areas = surface_nodes(v, faces, 64, 0)
    else:
        samples, areas = nodes
    return Shape(shape_id, v, faces, np.asarray(samples, float), np.asarray(areas, float),
                 volume, inertia, float(np.linalg.norm(v, axis=1).max()), {"generator": "box"})


def exact_cube(h=1e-4):
    """Six-node cube of the reference's closed-form pair-force case."""
    samples = np.concatenate([np.eye(3), -np.eye(3)]) * h / 2
    return box_shape([h] * 3, nodes=(samples, np.full(6, h * h)), shape_id="exact-cube")
