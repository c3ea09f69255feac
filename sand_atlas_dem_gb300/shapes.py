"""Grain shapes for the mesh-surface contact method (host side, run once).

A :class:`Shape` carries the fields the mesh path of the reference reads from a
shape asset (``src/sand_atlas_dem/geometry.py:17-29``): triangle mesh, surface
quadrature nodes with area weights, volume, unit-density inertia and bounding
radius.  Lengths are metres.  For the SDF contact geometry a shape also
carries its signed-distance grid (negative inside) with the grid origin and
spacing (``geometry.py:24-26``); :func:`with_sdf` builds one from the mesh the
way the reference lays it out, :func:`analytic_sphere` is the reference's
exact-sphere fixture.

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
    sdf: np.ndarray = None      # signed distance at the grid points, negative inside
    origin: np.ndarray = None   # position of grid point (0, 0, 0)
    spacing: float = 0.0        # grid spacing

    def validate(self):
        """Checks of ``geometry.py:32-58`` (the grid ones when a grid is carried)."""
        for a in (self.vertices, self.samples, self.areas, self.inertia):
            if not np.isfinite(a).all():
                raise ValueError("Nonfinite shape data")
        if self.sdf is not None:
            g = self.sdf
            if (g.ndim != 3 or min(g.shape) < 4 or not (g.min() < 0 < g.max()) or not np.isfinite(g).all()
                    or not self.spacing > 0 or np.shape(self.origin) != (3,)):
                raise ValueError("Invalid signed-distance grid")
            faces = np.concatenate([g[0].ravel(), g[-1].ravel(), g[:, 0].ravel(), g[:, -1].ravel(),
                                    g[:, :, 0].ravel(), g[:, :, -1].ravel()])
            if faces.min() <= 0:
                raise ValueError("Signed-distance grid boundary must lie outside the shape")
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


def _closest_on_triangles(p, a, b, c):
    """Nearest points of triangles (a, b, c) to points p, all (..., 3), FP64
    (the region test of the reference's closestTriangle, solver.slang:203-219)."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = np.einsum("...i,...i", ab, ap), np.einsum("...i,...i", ac, ap)
    bp = p - b
    d3, d4 = np.einsum("...i,...i", ab, bp), np.einsum("...i,...i", ac, bp)
    cp = p - c
    d5, d6 = np.einsum("...i,...i", ab, cp), np.einsum("...i,...i", ac, cp)
    vc, vb, va = d1 * d4 - d3 * d2, d5 * d2 - d1 * d6, d3 * d6 - d5 * d4
    with np.errstate(divide="ignore", invalid="ignore"):
        denom = va + vb + vc
        face = a + ab * (vb / denom)[..., None] + ac * (vc / denom)[..., None]
        e_ab = a + ab * (d1 / (d1 - d3))[..., None]
        e_ac = a + ac * (d2 / (d2 - d6))[..., None]
        e_bc = b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))[..., None]
    out = face
    regions = [
        ((va <= 0) & (d4 - d3 >= 0) & (d5 - d6 >= 0), e_bc),
        ((vb <= 0) & (d2 >= 0) & (d6 <= 0), e_ac),
        ((d6 >= 0) & (d5 <= d6), c),
        ((vc <= 0) & (d1 >= 0) & (d3 <= 0), e_ab),
        ((d3 >= 0) & (d4 <= d3), b),
        ((d1 <= 0) & (d2 <= 0), a),
    ]
    for mask, value in regions:  # later entries take precedence, as the early returns do
        out = np.where(mask[..., None], np.broadcast_to(value, out.shape), out)
    return out


def signed_distance(vertices, faces, points, chunk=1024):
    """Exact signed distance of points to a closed, outward-wound triangle
    mesh (negative inside), FP64: nearest point over all triangles, sign from
    the generalized winding number (solid angles, Van Oosterom-Strackee)."""
    tri = np.asarray(vertices, float)[np.asarray(faces)]
    a, b, c = tri[None, :, 0], tri[None, :, 1], tri[None, :, 2]
    points = np.asarray(points, float)
    out = np.empty(len(points))
    for start in range(0, len(points), chunk):
        p = points[start:start + chunk, None, :]
        q = _closest_on_triangles(p, a, b, c)
        distance = np.sqrt(np.min(np.einsum("pti,pti->pt", p - q, p - q), axis=1))
        x, y, z = a - p, b - p, c - p
        lx, ly, lz = (np.linalg.norm(v, axis=-1) for v in (x, y, z))
        det = np.einsum("pti,pti->pt", x, np.cross(y, z))
        den = (lx * ly * lz + np.einsum("pti,pti->pt", x, y) * lz + np.einsum("pti,pti->pt", y, z) * lx
               + np.einsum("pti,pti->pt", z, x) * ly)
        winding = np.sum(np.arctan2(det, den), axis=1) / (2 * np.pi)
        out[start:start + chunk] = np.where(winding > 0.5, -distance, distance)
    return out


def with_sdf(shape, resolution=32):
    """The shape with a signed-distance grid laid out as the reference lays it
    out (``geometry.py:195-215``): spacing = largest extent / (resolution - 1),
    origin three spacings below the mesh bounds, ceil(extents / spacing) + 7
    points per axis; values from :func:`signed_distance` in float32."""
    from dataclasses import replace

    vertices = np.asarray(shape.vertices, float)
    low, high = vertices.min(0), vertices.max(0)
    extents = high - low
    dx = float(extents.max() / (resolution - 1))
    origin = low - 3 * dx
    dims = np.ceil(extents / dx).astype(int) + 7
    ijk = np.stack(np.meshgrid(*(np.arange(d) for d in dims), indexing="ij"), -1).reshape(-1, 3)
    sdf = signed_distance(vertices, shape.faces, origin + dx * ijk).reshape(tuple(dims)).astype(np.float32)
    out = replace(shape, sdf=sdf, origin=origin, spacing=dx,
                  provenance=dict(shape.provenance, sdf_sign="negative_inside", sdf_resolution=int(resolution)))
    out.validate()
    return out


def analytic_sphere(radius=5e-4, resolution=32, samples=512):
    """The reference's analytical sphere fixture (``geometry.py:285-315``):
    exact grid values |x| - r over resolution + 6 points per axis, Fibonacci
    nodes with equal areas, analytic volume and inertia.  Its mesh (a
    frequency-4 geodesic sphere) serves only the host layout."""
    dx = 2 * radius / (resolution - 1)
    origin = np.full(3, -radius - 3 * dx)
    dims = resolution + 6
    grid = np.stack(np.meshgrid(*([np.arange(dims)] * 3), indexing="ij"), -1) * dx + origin
    sdf = (np.linalg.norm(grid, axis=-1) - radius).astype(np.float32)
    k = np.arange(samples)
    z = 1 - 2 * (k + 0.5) / samples
    angle = k * (np.pi * (3 - np.sqrt(5)))
    nodes = radius * np.column_stack([np.sqrt(1 - z * z) * np.cos(angle), np.sqrt(1 - z * z) * np.sin(angle), z])
    unit, faces = icosphere(4)
    volume = 4 * np.pi * radius**3 / 3
    shape = Shape("analytical-sphere", unit * radius, faces, nodes, np.full(samples, 4 * np.pi * radius**2 / samples),
                  volume, np.eye(3) * 0.4 * volume * radius**2, radius,
                  dict(fixture="analytical_sphere", radius_m=radius, display_mesh_only=True),
                  sdf=sdf, origin=origin, spacing=dx)
    shape.validate()
    return shape


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
