"""Host-side set-up of one mesh-surface DEM specimen (periodic, or bounded by planes).

Everything here runs once per engine on the host, in float64 numpy, and ends
as the float32/uint32 arrays the device step reads.  It restates the set-up
half of the reference ``Engine.__init__`` (``src/sand_atlas_dem/gpu.py:95-368``)
and its timestep preflight (``gpu.py:370-413``): normalized units
(L0 = median equivalent diameter, T0 = sqrt(rho L0 / kn), F0 = kn L0^3),
per-grain ``body``/``invI`` rows, Verlet skin and cutoff, cell-list bins,
capacities and the packed mesh layout.  The resulting arrays are checked
against the reference's own ``Engine`` in the golden tests.
"""

import math

import numpy as np

from .boundaries import box_extents
from .packing import host_median_trees, pack_library
from .spec import finite_array

ERRORS = {
    2: "degenerate contact distance gradient",
    4: "excessive penetration",
    8: "bin capacity",
    16: "pair capacity",
    32: "contact capacity",
    64: "history hash full",
    128: "contact-list cycle",
    256: "periodic image ambiguity",
    512: "nonfinite state",
    1024: "mesh traversal stack capacity",
    2048: "nonperiodic domain escape",
    4096: "invalid boundary box",
    8192: "active-contact timestep bound",
    16384: "coincident centres unsupported by experimental source-normal contacts",
    65536: "device wait limit",
}
CAPACITY_FLAGS = 8 | 16 | 32 | 64

# Reference ``Resources`` field order (``shaders/solver.slang:20-100``); the
# C ABI of both the CUDA library and the CPU oracle binds buffers in it.
RESOURCE_ORDER = (
    "control", "cell", "position", "positionRemainder", "velocityRemainder",
    "momentumRemainder", "rotationRemainder", "referencePositionRemainder", "cellLog",
    "accumulatedRemainder", "velocity", "rotation", "momentum", "force", "torque",
    "referencePosition", "referenceCell", "shapeId", "body", "invI", "grids", "sampleInfo",
    "gridOrigin", "distance", "sample", "meshRoots", "meshHullInfo", "meshPlanes", "meshMin",
    "meshMax", "meshLinks", "meshTriangles", "meshNormals", "meshFrontier", "meshPairMask",
    "meshPairTransform", "meshClusterInfo", "meshClusterRanges", "meshClusterMin",
    "meshClusterMax", "meshSampleIndices", "binCounts", "binParticles", "pairCounts",
    "pairOffsets", "pairs", "contactCounts", "contactOffsets", "meta", "pointDepth",
    "normalArea", "slip", "contactForce", "normalLossPower", "normalDamping", "forceVelocity",
    "forceOmega", "oldMeta", "oldSlip", "oldNormal", "oldHash", "hash", "heads", "next",
    "particleStress", "timestepRows", "particleDiagnostic", "diagnosticRows", "accumulated",
    "fabricRows", "wallPlane", "wallRemainder", "wallVelocity", "wallMaterial", "wallBoxIds",
    "wallRows", "wallAccumulated",
)
# Flattened ``Config`` scalars in declaration order (``solver.slang:12-19``).
CONFIG_ORDER = (
    "activeTimestep", "N", "shapes", "pairCapacity", "contactCapacity", "binCapacity",
    "binCount", "bins0", "bins1", "bins2", "hashSize", "dt", "kn", "kt", "mu",
    "normalViscosity", "skin", "drag", "maxOverlap", "historyStep", "meshGeometry",
    "periodic", "wallCount", "wallBoxEnabled", "sourceSurfaceNormal",
)

DAMPING_STATE = ("normalDamping", "forceVelocity", "forceOmega")
WALL_STATE = ("wallPlane", "wallRemainder", "wallVelocity", "wallAccumulated", "wallRows")
RESIDUAL_STATE = (
    "positionRemainder", "velocityRemainder", "momentumRemainder", "rotationRemainder",
    "accumulatedRemainder", "cellLog",
)
STATE_NAMES = (
    "position", "velocity", "rotation", "momentum", "cell", "force", "torque", "accumulated",
    *RESIDUAL_STATE,
)


def f4(x):
    a = np.asarray(x, np.float32)
    return np.pad(a, ((0, 0), (0, 4 - a.shape[1])))


class RejectedStep(RuntimeError):
    """A chunk raised solver flags and was rolled back (``gpu.py:51-57``)."""

    def __init__(self, flags):
        self.flags = int(flags)
        super().__init__(
            "GPU step rejected: " + ", ".join(v for k, v in ERRORS.items() if self.flags & k)
        )


def conservative_timestep(library, spec, ids, scales):
    """Smallest per-grain conservative bound 0.1 min(elastic, viscous) (``gpu.py:370-413``)."""
    limits = []
    for i, s in zip(np.asarray(ids), np.asarray(scales, float)):
        sh = library.shapes[int(i)]
        mass = spec.density * sh.volume * s**3
        stiffness = (
            spec.normal_stiffness + spec.tangential_stiffness
            + sum(p["normal_stiffness"] + p["tangential_stiffness"] for p in spec.planes)
        ) * sh.areas.sum() * s * s
        smallest = np.linalg.eigvalsh(sh.inertia * spec.density * s**5).min()
        elastic = math.sqrt(min(mass / stiffness, smallest / (stiffness * (sh.radius * s) ** 2)))
        viscous = math.inf
        viscosity = (
            spec.normal_viscosity + sum(p.get("normal_viscosity", 0) for p in spec.planes)
        ) * sh.areas.sum() * s**2
        if viscosity > 0:
            viscous = min(mass / viscosity, smallest / (viscosity * (sh.radius * s) ** 2))
        limits.append(0.1 * min(elastic, viscous))
    return min(limits)


class HostLayout:
    """Units, per-grain rows, capacities and static geometry of the grains.

    One periodic specimen (the reference ``Engine``), or with
    :meth:`batch` several independent specimens sharing one library and
    material: grains concatenated, one cell per specimen, one bin grid per
    specimen, one set of capacities for all.
    """

    @classmethod
    def batch(cls, library, spec, specimens, trees=host_median_trees):
        """``specimens``: sequence of (positions, cell, shape_ids, scales)."""
        specimens = list(specimens)
        if not specimens:
            raise ValueError("At least one specimen required")
        positions = np.concatenate([np.asarray(s[0], float) for s in specimens])
        ids = np.concatenate([np.asarray(s[2], np.uint32) for s in specimens])
        scales = np.concatenate([np.asarray(s[3], float) for s in specimens])
        cells = np.array([finite_array(s[1], (3,), positive=True) for s in specimens])
        counts = [len(s[0]) for s in specimens]
        return cls(library, spec, positions, cells[0], ids, scales, cells=cells, counts=counts, trees=trees)

    def __init__(self, library, spec, positions, cell, shape_ids, scales, *, cells=None, counts=None,
                 trees=host_median_trees):
        # Builder of the packed layout's median-split trees (host recursion,
        # or the GPU builder the engine passes); the bytes are the same.
        self.trees = trees
        positions = finite_array(positions)
        cell = finite_array(cell, (3,), positive=True)
        if cells is None:
            cells, counts = cell[None, :], [len(positions)]
        self.cells = np.asarray(cells, float)
        self.counts = list(counts)
        self.specimens = len(self.counts)
        if sum(self.counts) != len(positions) or len(self.cells) != self.specimens:
            raise ValueError("Specimen grain counts and cells do not match the grains")
        if positions.ndim != 2 or positions.shape[1] != 3 or len(positions) < 1:
            raise ValueError("At least one three-dimensional position required")
        self.grain_specimen = np.repeat(np.arange(self.specimens, dtype=np.uint32), self.counts)
        if not spec.periodic and (np.any(positions < 0) or np.any(positions >= self.cells[self.grain_specimen])):
            raise ValueError("Nonperiodic particle centres must lie in [0, cell)")
        if spec.contact_geometry not in ("mesh", "sdf"):
            raise ValueError("Contact geometry must be mesh or sdf")
        if spec.contact_geometry == "sdf":
            if any(getattr(s, "sdf", None) is None for s in library.shapes):
                raise ValueError("The SDF contact geometry needs a signed-distance grid on every shape")
            if spec.contact_normal == "source-surface-experimental":
                raise ValueError("The source-surface normal needs the mesh contact geometry")
        if spec.planes and self.specimens != 1:
            raise ValueError("Planes bound a single specimen")
        if spec.boundary_box is not None:
            box_extents(np.array([p["offset"] for p in spec.planes]), spec.boundary_box, self.cells[0])
        self.spec = spec
        self.library = library
        self.n = len(positions)
        self.viscous = spec.viscous
        shapes = library.shapes
        self.length_unit = float(np.median([(6 * s.volume / np.pi) ** (1 / 3) for s in shapes]))
        self.time_unit = math.sqrt(spec.density * self.length_unit / spec.normal_stiffness)
        self.mass_unit = spec.density * self.length_unit**3
        self.force_unit = spec.normal_stiffness * self.length_unit**3
        self.stress_unit = spec.normal_stiffness * self.length_unit
        self.energy_unit = self.force_unit * self.length_unit
        self.ids = np.asarray(shape_ids, np.uint32)
        self.scales = np.asarray(scales, float)
        if len(self.ids) != self.n or len(self.scales) != self.n:
            raise ValueError("One shape id and scale per particle required")
        if self.ids.size and int(self.ids.max()) >= len(shapes):
            raise ValueError("Shape id outside the library")
        l = self.length_unit
        self.body = np.array(
            [
                [
                    s,
                    spec.density * shapes[int(i)].volume * s**3 / self.mass_unit,
                    shapes[int(i)].radius * s / l,
                    (6 * shapes[int(i)].volume / np.pi) ** (1 / 3) * s / l,
                ]
                for i, s in zip(self.ids, self.scales)
            ],
            np.float32,
        )
        inertia = np.array(
            [
                np.linalg.inv(
                    shapes[int(i)].inertia * spec.density * s**5 / (self.mass_unit * l * l)
                )
                for i, s in zip(self.ids, self.scales)
            ]
        )
        self.invI = f4(inertia.reshape(-1, 3))
        self.skin = float(spec.skin * 2 * self.body[:, 2].max())
        self.cutoff = float(2 * self.body[:, 2].max() + self.skin)
        boxes = self.cells / l
        if spec.periodic and self.cutoff >= 0.5 * boxes.min():
            raise ValueError("Cell too small for unique periodic images")
        self.boxes = boxes
        self.box = boxes[0]
        bins = np.maximum(1, np.minimum(64, np.floor(boxes / self.cutoff))).astype(np.uint32)
        self.specimen_bins = np.zeros((self.specimens, 4), np.uint32)
        self.specimen_bins[:, :3] = bins
        self.specimen_bins[1:, 3] = np.cumsum(bins.prod(axis=1))[:-1]
        self.bins = bins[0]
        self.bin_count = int(bins.prod(axis=1).sum())
        self.pair_capacity = max(1, self.n * spec.pairs_per_particle)
        self.contact_capacity = max(16, self.n * spec.contacts_per_particle)
        self.hash_size = 1 << math.ceil(math.log2(max(32, 2 * self.contact_capacity)))
        self.bin_capacity = spec.bin_capacity
        self.preflight_dt()
        self.initial_cell = np.asarray(cell, float)
        if spec.boundary_box is not None:
            self.initial_cell = box_extents(np.array([p["offset"] for p in spec.planes]), spec.boundary_box, cell)
        self.wall_count = len(spec.planes)
        self.walls = self.wall_arrays()
        self.normalized_position = np.asarray(positions, float) / l
        self.geometry = self.static_geometry()
        self.max_leaves = int(self.geometry["meshLeafInfo"][:, 1].max())
        self.max_nodes = int(self.geometry["sampleInfo"][:, 1].max())

    def wall_arrays(self):
        """Normalized plane rows and per-(wall, grain) rows (``gpu.py:232-285``):
        FP32 normal and offset with the offset's FP32 residual, velocity,
        material (kn, kt relative to the grain kn; friction; viscosity over
        the grain kn and time unit), box plane ids and zeroed work rows."""
        spec, l, n = self.spec, self.length_unit, self.n
        count = self.wall_count
        plane = np.zeros((max(1, count), 4), np.float64)
        velocity = np.zeros_like(plane)
        material = np.zeros_like(plane)
        for index, p in enumerate(spec.planes):
            plane[index] = [*p["normal"], p["offset"] / l]
            velocity[index, :3] = np.array(p["velocity"]) * self.time_unit / l
            material[index, :3] = [p["normal_stiffness"] / spec.normal_stiffness,
                                   p["tangential_stiffness"] / spec.normal_stiffness, p["friction"]]
            material[index, 3] = p.get("normal_viscosity", 0) / (spec.normal_stiffness * self.time_unit)
        rounded = plane.astype(np.float32)
        residual = (plane - rounded).astype(np.float32)
        if (not np.isfinite(rounded).all() or not np.isfinite(residual).all()
                or not np.isfinite(velocity.astype(np.float32)).all()
                or not np.isfinite(material.astype(np.float32)).all()
                or (count and np.any(material[:count, :2].astype(np.float32) <= 0))):
            raise ValueError("Plane data cannot be represented in normalized FP32 units")
        for index, p in enumerate(spec.planes):
            if p.get("normal_viscosity", 0) > 0 and np.float32(material[index, 3]) <= 0:
                raise ValueError("Plane viscosity cannot be represented in normalized FP32 units")
        return {
            "wallPlane": rounded,
            "wallRemainder": residual,
            "wallVelocity": velocity.astype(np.float32),
            "wallMaterial": material.astype(np.float32),
            "wallBoxIds": np.array(spec.boundary_box or [0] * 6, np.uint32),
            "wallAccumulated": np.zeros((max(1, count * n), 4), np.float32),
            "wallRows": np.zeros((max(1, 3 * count * n), 4), np.float32),
        }

    def preflight_dt(self):
        """Conservative timestep bound (``gpu.py:370-413``)."""
        spec = self.spec
        if spec.timestep_policy == "active-contact":
            return
        limit = self.timestep_limit()
        if spec.timestep > limit:
            raise ValueError(f"Timestep exceeds conservative estimate {limit:.6g} s")

    def timestep_limit(self):
        return conservative_timestep(self.library, self.spec, self.ids, self.scales)

    def static_geometry(self):
        """Packed mesh arrays (mesh geometry) or the signed-distance grids (SDF
        geometry, with one-row mesh placeholders), plus the per-shape node
        table (``gpu.py:421-488``)."""
        l = self.length_unit
        if self.spec.contact_geometry == "sdf":
            return self._sdf_geometry()
        data = pack_library(self.library, self.length_unit, trees=self.trees)
        info, samples, offset = [], [], 0
        for s in self.library.shapes:
            info.append([offset, len(s.samples), 0, 0])
            samples.append(np.column_stack([s.samples / l, s.areas / l**2]).astype(np.float32))
            offset += len(s.samples)
        data["sampleInfo"] = np.asarray(info, np.uint32)
        data["sample"] = np.concatenate(samples)
        # The SDF grids are unused by the mesh path; one-element placeholders
        # keep the reference buffer order.
        data["grids"] = np.zeros((1, 4), np.uint32)
        data["gridOrigin"] = np.zeros((1, 4), np.float32)
        data["distance"] = np.zeros(4, np.float32)
        return data

    def _sdf_geometry(self):
        """``gpu.py:421-488`` for the SDF geometry: each shape's grid packed as
        (first value, nx, ny, nz), origin and spacing over the length unit, and
        the values in x-major order; mesh arrays are one-row placeholders."""
        l = self.length_unit
        shapes = self.library.shapes
        data = {name: np.zeros((1, 4), np.uint32) for name in
                ("meshRoots", "meshLinks", "meshHullInfo", "meshFrontier", "meshClusterInfo", "meshClusterRanges")}
        for name in ("meshPlanes", "meshMin", "meshMax", "meshTriangles", "meshNormals", "meshClusterMin",
                     "meshClusterMax"):
            data[name] = np.zeros((1, 4), np.float32)
        data["meshSampleIndices"] = np.zeros(4, np.uint32)
        # This backend's mesh extensions, empty: no shape has leaf clusters.
        data["meshLeafInfo"] = np.zeros((len(shapes), 4), np.uint32)
        data["meshLeaves"] = np.zeros(4, np.uint32)
        data["meshChildren"] = np.zeros((4, 4), np.float32)
        grids, origins, fields, info, samples = [], [], [], [], []
        first = offset = 0
        for s in shapes:
            grids.append([first, *s.sdf.shape])
            origins.append([*(np.asarray(s.origin) / l), s.spacing / l])
            fields.append((s.sdf / l).astype(np.float32).ravel())
            info.append([offset, len(s.samples), 0, 0])
            samples.append(np.column_stack([s.samples / l, s.areas / l**2]).astype(np.float32))
            first += s.sdf.size
            offset += len(s.samples)
        data["meshSampleRank"] = np.zeros(max(offset, 1), np.uint32)
        data["grids"] = np.asarray(grids, np.uint32)
        data["gridOrigin"] = np.asarray(origins, np.float32)
        data["distance"] = np.concatenate(fields).astype(np.float32)
        data["sampleInfo"] = np.asarray(info, np.uint32)
        data["sample"] = np.concatenate(samples)
        return data

    def config(self, *, dt, drag=0.0, history=False):
        """Normalized ``Config`` block (``gpu.py:490-518``)."""
        spec = self.spec
        return {
            "activeTimestep": int(spec.timestep_policy == "active-contact"),
            "N": self.n,
            "shapes": len(self.library.shapes),
            "pairCapacity": self.pair_capacity,
            "contactCapacity": self.contact_capacity,
            "binCapacity": self.bin_capacity,
            "binCount": self.bin_count,
            "bins0": int(self.bins[0]),
            "bins1": int(self.bins[1]),
            "bins2": int(self.bins[2]),
            "hashSize": self.hash_size,
            "dt": dt / self.time_unit,
            "kn": 1.0,
            "kt": spec.tangential_stiffness / spec.normal_stiffness,
            "mu": spec.friction,
            "normalViscosity": spec.normal_viscosity / (spec.normal_stiffness * self.time_unit),
            "skin": self.skin,
            "drag": drag * self.time_unit,
            "maxOverlap": spec.max_overlap_fraction,
            "historyStep": int(history),
            "meshGeometry": int(spec.contact_geometry == "mesh"),
            "sourceSurfaceNormal": int(spec.contact_normal == "source-surface-experimental"),
            "periodic": int(spec.periodic),
            "wallCount": self.wall_count,
            "wallBoxEnabled": int(spec.boundary_box is not None),
        }

    def config_values(self, config):
        return np.array([float(config[k]) for k in CONFIG_ORDER], np.float64)

    def initial_state(self):
        """Per-grain state rows at construction (``gpu.py:193-292``)."""
        n = self.n
        p = self.normalized_position
        z = lambda rows=n: np.zeros((rows, 4), np.float32)  # noqa: E731
        state = {
            "position": f4(p),
            "velocity": z(),
            "rotation": np.tile(np.array([0, 0, 0, 1], np.float32), (n, 1)),
            "momentum": z(),
            "force": z(),
            "torque": z(),
            "referencePosition": z(),
            "particleDiagnostic": z(),
            "timestepRows": z(),
            "particleStress": z(3 * n),
            "diagnosticRows": z(8 * n),
            "accumulated": z(),
            "referencePositionRemainder": z(),
        }
        for name in DAMPING_STATE:
            state[name] = z()
        for name in RESIDUAL_STATE:
            residual = z(2 if name == "cellLog" else n)
            if name == "positionRemainder":
                residual[:, :3] = p - p.astype(np.float32).astype(float)
            state[name] = residual
        state["cell"] = np.concatenate(
            [np.array([list(b) + [0], [0, 0, 0, 0], list(b) + [0]], np.float32) for b in self.boxes])
        state["referenceCell"] = np.concatenate(
            [np.array([list(b) + [0], [0, 0, 0, self.cutoff]], np.float32) for b in self.boxes])
        state["cellLog"] = np.zeros((2 * self.specimens, 4), np.float32)
        state["grainSpecimen"] = self.grain_specimen.copy()
        state["specimenBins"] = self.specimen_bins.copy()
        ctrl = np.zeros(16, np.uint32)
        ctrl[4] = 1
        state["control"] = ctrl
        state["shapeId"] = self.ids.copy()
        state["body"] = self.body.copy()
        state["invI"] = self.invI.copy()
        return state

    def estimated_bytes(self):
        """Device working set of this backend, including its own scratch."""
        n, p, c = self.n, self.pair_capacity, self.contact_capacity
        geometry = sum(a.nbytes for a in self.geometry.values())
        candidates = 2 * p * self.max_leaves
        return int(
            1184 * n
            + 8 * self.bin_count * self.bin_capacity
            + 196 * p + 2 * 8 * p * (self.max_leaves + 31) // 32
            + 16 * candidates
            + 2 * 96 * c + 64 * c
            + geometry
        )
