"""GB300 timestep engine: the reference ``Engine`` surface over the CUDA step.

Mirrors ``src/sand_atlas_dem/gpu.py:94-1092``: constructor arguments,
``initialize``, ``advance`` (transactional chunks with rollback and capacity
growth), ``diagnostics``, ``state``/``restore`` in the checkpoint array schema,
``timestep_limits``, ``check_errors``, ``profile_step``, the unit attributes
and ``buffers[name].copy_from_numpy``.  Device buffers are torch CUDA tensors
(memory only); every kernel runs in the sm_103a library through its C ABI,
one CUDA stream per engine, the step replayed as a captured CUDA graph.
"""

import ctypes as ct
import math
import time
import weakref

import numpy as np

from . import native
from .boundaries import box_extents
from .model import (
    CAPACITY_FLAGS,
    DAMPING_STATE,
    RESIDUAL_STATE,
    RESOURCE_ORDER,
    STATE_NAMES,
    WALL_STATE,
    HostLayout,
    RejectedStep,
    f4,
)
from .spec import finite_array
from .trees import device_median_trees

# Launch shapes the autotuner sets (values after the extension values; 0 =
# built-in default).  They never change results.
TUNING_KEYS = ("query_blocks_per_sm", "query_warps", "cull_blocks_per_sm", "contact_blocks_per_sm",
               "gather_warps_per_sm", "walk_blocks_per_sm")

EXTENSION_ORDER = (
    "meshLeafInfo", "meshLeaves", "meshSampleRank", "byJCounts", "byJOffsets", "byJCursor",
    "byJPairs", "dpairBranch", "dpairLeafCount", "dpairCandOffset", "leafMask", "candidates",
    "candHitCount", "candHitOffset", "candHitMask", "contactPair", "sidePairOffsets", "sidePairB",
    "sideContactStart", "oldPairOffsets", "oldPairB", "oldContactStart", "work", "scanPartials",
    "hitScratch", "candSurvCount", "dpairPlane", "grainSpecimen", "specimenBins", "cullerParams", "cullerW1",
    "cullerMargin", "cullerStats", "candSurvMask", "candSurvOffset", "survivors", "survKeep", "keepOffset",
    "walkList", "dpairSourcePlane", "meshChildren", "distanceGrid", "distanceGridInfo", "distanceGridTriangle",
    "filterRefRotation", "filterRefBranch", "filterRefPairs", "walkKey", "walkBucketCount", "walkBucketOffset",
    "sdfLaneCounts", "walkCertPoint", "walkCertTriangle", "wallCounts", "wallOffsets", "sideWallStart",
    "oldWallStart", "walkNode", "walkItem",
)
DISTANCE_GRID = 48  # cells per axis of each shape's distance-bound grid (csrc GRID)
WALK_BUCKETS = 24**3  # walk-order buckets per shape (csrc WALK_BUCKETS)
CULLER_PARAMS = 3 * 64 + 64 + 64 * 64 + 64 + 64 + 4
CULLER_MARGINS = 1 + 8**3  # per shape: whole-shape margin, then one per cell (csrc CULLER_MARGINS)
BUFFER_ORDER = RESOURCE_ORDER + EXTENSION_ORDER
# History side fields: (name bound as the side being written, name bound as committed).
SIDE_FIELDS = (
    ("meta", "oldMeta"), ("slip", "oldSlip"), ("normalArea", "oldNormal"), ("hash", "oldHash"),
    ("sidePairOffsets", "oldPairOffsets"), ("sidePairB", "oldPairB"),
    ("sideContactStart", "oldContactStart"), ("sideWallStart", "oldWallStart"),
)
SCAN_BLOCKS = 608
# Default reach of the stored node-filter results: 0.1% of a unit-median
# shape's size in its own frame.
FILTER_MARGIN = 1e-3


def _torch():
    import torch

    return torch


STAGING_BYTES = 1 << 16  # pinned host staging per engine for small uploads and reads


class DeviceBuffer:
    """One device allocation; the reference Buffer surface (``cpu.py:431-447``)."""

    def __init__(self, engine, nbytes):
        torch = _torch()
        self._engine = weakref.ref(engine)
        self.size = int(max(16, nbytes))
        # Allocated and zeroed on the engine stream, which every later use of
        # the buffer is ordered on.
        with torch.cuda.stream(engine.stream):
            self.tensor = torch.zeros(self.size, dtype=torch.uint8, device=engine.device)

    def ptr(self):
        return self.tensor.data_ptr()

    def copy_from_numpy(self, array):
        data = np.ascontiguousarray(array).view(np.uint8).reshape(-1)
        if data.size != self.size:
            raise ValueError("GB300 buffer upload size mismatch")
        self._upload(data)

    def write_prefix(self, array):
        data = np.ascontiguousarray(array).view(np.uint8).reshape(-1)
        if data.size > self.size:
            raise ValueError("GB300 buffer prefix out of bounds")
        if data.size:
            self._upload(data)

    def _upload(self, data):
        """Host -> device on the engine stream; small uploads go through the
        engine's pinned staging buffer (one DMA, no pageable bounce)."""
        torch = _torch()
        engine = self._engine()
        n = data.size
        with torch.cuda.stream(engine.stream):
            if n <= STAGING_BYTES:
                stage = engine._staging[:n]
                stage.numpy()[:] = data
                self.tensor[:n].copy_(stage, non_blocking=True)
            else:
                self.tensor[:n].copy_(torch.from_numpy(data.copy()))
        engine.stream.synchronize()
        engine.h2d_bytes += n
        engine._uploaded(self)

    def to_numpy(self, dtype=np.uint8, count=None):
        torch = _torch()
        engine = self._engine()
        nbytes = self.size if count is None else int(count) * np.dtype(dtype).itemsize
        engine.d2h_bytes += nbytes
        if nbytes <= STAGING_BYTES:
            # Small reads land in the pinned staging buffer.
            stage = engine._staging[:nbytes]
            with torch.cuda.stream(engine.stream):
                stage.copy_(self.tensor[:nbytes], non_blocking=True)
            engine.stream.synchronize()
            return stage.numpy().view(dtype).copy()
        engine.stream.synchronize()
        return self.tensor[:nbytes].cpu().numpy().view(dtype).copy()


def read_batch(engine, requests):
    """Several small reads ((buffer, bytes, dtype) each) staged side by side in
    the engine's pinned buffer and waited for once."""
    torch = _torch()
    offsets, total = [], 0
    for _, nbytes, _ in requests:
        offsets.append(total)
        total += (int(nbytes) + 15) // 16 * 16
    if total > STAGING_BYTES:
        return [buffer.to_numpy(dtype, nbytes // np.dtype(dtype).itemsize) for buffer, nbytes, dtype in requests]
    with torch.cuda.stream(engine.stream):
        for (buffer, nbytes, _), offset in zip(requests, offsets):
            engine._staging[offset:offset + nbytes].copy_(buffer.tensor[:nbytes], non_blocking=True)
    engine.stream.synchronize()
    host = engine._staging.numpy()
    out = []
    for (_, nbytes, dtype), offset in zip(requests, offsets):
        engine.d2h_bytes += nbytes
        out.append(host[offset:offset + nbytes].view(dtype).copy())
    return out


class GB300Device:
    """The adapter surface callers read through ``engine.m`` (``cpu.py:540-689``)."""

    name = "gb300"

    def __init__(self, engine):
        self._engine = weakref.ref(engine)

    def read(self, buffer, dtype=np.float32, shape=None):
        array = buffer.to_numpy(dtype)
        return array if shape is None else array[: int(np.prod(shape))].reshape(shape)

    def read_prefix(self, buffer, count, dtype=np.float32, shape=None):
        if type(count) is not int or count < 0 or count * np.dtype(dtype).itemsize > buffer.size:
            raise ValueError("GB300 buffer prefix out of bounds")
        array = buffer.to_numpy(dtype, count)
        return array if shape is None else array.reshape(shape)

    def write_prefix(self, buffer, array):
        buffer.write_prefix(array)

    def doctor(self):
        torch = _torch()
        lib = native.load()
        props = torch.cuda.get_device_properties(self._engine().device)
        return dict(
            format="sand-dem-doctor/1",
            backend="gb300",
            fallback=False,
            adapter=props.name,
            compute_capability=f"{props.major}.{props.minor}",
            multiprocessors=props.multi_processor_count,
            library=str(native.LIBRARY),
            abi_version=lib.sdg_abi_version(),
            numerics="sm_103a CUDA FP32 in the reference operation order (no FMA contraction), "
            "FP64 minimum image, compensated state, canonical contact order, deterministic gather",
            job_parallelism="one engine per CUDA stream",
        )


class Engine:
    """GPU-resident DEM engine: mesh or SDF contact geometry, periodic cells or
    one nonperiodic specimen bounded by penalty planes."""

    @classmethod
    def batch(cls, library, spec, specimens, **kwargs):
        """Independent periodic specimens stepped together in one launch per
        phase: ``specimens`` is a sequence of (positions, cell, shape_ids,
        scales).  Per-specimen cell rates are set with ``advance(rate=...)``
        given one row per specimen."""
        layout = HostLayout.batch(library, spec, specimens, trees=device_median_trees)
        return cls(library, spec, None, None, None, None, layout=layout, **kwargs)

    def __init__(self, library, spec, positions, cell, shape_ids, scales, *, metal=None, device=None,
                 use_graph=True, layout=None, distance_grid=True, filter_margin=FILTER_MARGIN):
        torch = _torch()
        if metal is not None:
            raise ValueError("The GB300 engine owns its device; no adapter may be passed")
        if not torch.cuda.is_available():
            raise RuntimeError("The GB300 backend requires a CUDA device; there is no CPU fallback")
        self.lib = native.load()
        if self.lib.sdg_buffer_count() != len(BUFFER_ORDER):
            raise RuntimeError("GB300 library buffer ABI mismatch")
        self.layout = h = layout or HostLayout(library, spec, positions, cell, shape_ids, scales,
                                               trees=device_median_trees)
        self.specimens = h.specimens
        self.spec, self.library, self.n = spec, library, h.n
        self.viscous = spec.viscous
        self.wall_count = h.wall_count
        self.step = 0
        self.history = False
        self.active = 0
        self.capacity_retries = []
        self.use_graph = use_graph
        self.culler = None
        self.tuning = {}
        # Skip nodes the certified distance-bound grid places outside their
        # target (exact: no contact changes); off reproduces the reference's
        # own filters alone.
        self.distance_grid = bool(distance_grid)
        # Reach (target shape frame, unscaled) of the stored node-filter
        # results: the leaf cull and node filter run with their tests grown by
        # it and are reused while no grain has moved that far relative to a
        # partner (exact: no contact changes); 0 runs them every step.
        self.filter_margin = float(filter_margin)
        if not np.isfinite(self.filter_margin) or self.filter_margin < 0:
            raise ValueError("Finite nonnegative filter margin required")
        # The SDF geometry queries every node of a pair on its grid: the mesh
        # filters, their stored results and the distance-bound grid do not apply.
        self.sdf = spec.contact_geometry == "sdf"
        if self.sdf:
            self.distance_grid, self.filter_margin = False, 0.0
        self._reduce_scratch = {}
        self._array_cache = {}
        # Host copies that spare a device read: the control words as last
        # read (valid while no device work or upload followed) and the
        # strain-rate rows last written into the cell.
        self._device_version = 0
        self._ctrl_cache = None
        self._diagnostic_scratch = None
        self._rates = None
        # Host<->device bytes moved by this engine's own reads and uploads.
        self.h2d_bytes = self.d2h_bytes = 0
        for name in ("length_unit", "time_unit", "mass_unit", "force_unit", "stress_unit", "energy_unit",
                     "ids", "scales", "body", "skin", "cutoff", "bins", "bin_count", "pair_capacity",
                     "contact_capacity", "hash_size", "bin_capacity", "initial_cell"):
            setattr(self, name, getattr(h, name))
        self.estimated_bytes = h.estimated_bytes()
        volumes = np.array([shape.volume for shape in library.shapes])
        self.solid_volume = float(np.sum(volumes[self.ids] * np.asarray(self.scales, float) ** 3))
        self.leaf_words = (h.max_leaves + 31) // 32
        self.candidate_capacity = max(1, 2 * h.pair_capacity * h.max_leaves)
        # Nodes left for the exact query after the conservative filters, per
        # step; overflow raises the contact-capacity flag and grows with it.
        self.survivor_capacity = 4 * h.contact_capacity
        self.device = torch.device(device or "cuda")
        self.stream = torch.cuda.Stream(self.device)
        self._staging = torch.empty(STAGING_BYTES, dtype=torch.uint8).pin_memory()
        self.m = GB300Device(self)
        self.buffers = {}
        n, pc, cc = h.n, h.pair_capacity, h.contact_capacity
        for name, array in h.geometry.items():
            self._add(name, array)
        for name, array in h.initial_state().items():
            self._add(name, array)
        for name, array in h.walls.items():
            self._add(name, array)
        walls = h.wall_count * n
        sizes = {
            "meshPairMask": 4 * pc, "meshPairTransform": 16 * 8 * pc, "fabricRows": 16 * 2 * pc,
            "binCounts": 4 * h.bin_count, "binParticles": 4 * h.bin_count * h.bin_capacity,
            "pairCounts": 4 * n, "pairOffsets": 4 * n, "pairs": 8 * pc, "contactCounts": 4 * pc,
            "contactOffsets": 4 * pc, "pointDepth": 16 * cc, "contactForce": 16 * cc,
            "normalLossPower": 4 * cc, "heads": 4 * n, "next": 16,
            "byJCounts": 4 * (n + 1), "byJOffsets": 4 * (n + 1), "byJCursor": 4 * n, "byJPairs": 4 * pc,
            "dpairBranch": 16 * 2 * pc, "dpairLeafCount": 4 * (2 * pc + 1),
            "dpairCandOffset": 4 * (2 * pc + 1), "leafMask": 4 * 2 * pc * self.leaf_words,
            "candidates": 8 * self.candidate_capacity, "candHitCount": 4 * (self.candidate_capacity + 1),
            "candHitOffset": 4 * (self.candidate_capacity + 1), "candHitMask": 8 * self.candidate_capacity,
            "contactPair": 4 * cc, "work": 4 * 64, "scanPartials": 4 * 2 * SCAN_BLOCKS,
            "hitScratch": 32 * self.survivor_capacity, "candSurvCount": 4 * (self.candidate_capacity + 1),
            "dpairPlane": 16 * 2 * pc, "candSurvMask": 8 * self.candidate_capacity,
            "candSurvOffset": 4 * (self.candidate_capacity + 1), "survivors": 8 * self.survivor_capacity,
            "survKeep": 4 * (self.survivor_capacity + 1), "keepOffset": 4 * (self.survivor_capacity + 1),
            "walkList": 4 * self.survivor_capacity, "dpairSourcePlane": 16 * 4 * pc,
            "distanceGrid": 4 * len(library.shapes) * DISTANCE_GRID**3, "distanceGridInfo": 16 * len(library.shapes),
            "distanceGridTriangle": 4 * len(library.shapes) * DISTANCE_GRID**3,
            "cullerParams": 4 * CULLER_PARAMS * len(library.shapes), "cullerW1": 2 * 4096 * len(library.shapes),
            "cullerMargin": 4 * CULLER_MARGINS * len(library.shapes), "cullerStats": 16,
            "filterRefRotation": 16 * n, "filterRefBranch": 16 * pc, "filterRefPairs": 8 * pc,
            "walkKey": 4 * self.survivor_capacity, "walkBucketCount": 4 * (len(library.shapes) * WALK_BUCKETS + 1),
            "walkBucketOffset": 4 * (len(library.shapes) * WALK_BUCKETS + 1),
            "sdfLaneCounts": 4 * 32 * pc if spec.contact_geometry == "sdf" else 16,
            "walkCertPoint": 16 * self.survivor_capacity, "walkCertTriangle": 8 * self.survivor_capacity,
            "walkNode": 16 * self.survivor_capacity, "walkItem": 8 * self.survivor_capacity,
            "wallCounts": 4 * walls, "wallOffsets": 4 * (walls + 1),
        }
        for name, nbytes in sizes.items():
            self.buffers[name] = DeviceBuffer(self, nbytes)
        side_sizes = {
            "meta": 16 * cc, "slip": 16 * cc, "normalArea": 16 * cc, "hash": 16,
            "sidePairOffsets": 4 * (n + 1), "sidePairB": 4 * pc, "sideContactStart": 4 * (pc + 1),
            "sideWallStart": 4 * (walls + 1),
        }
        self.sides = [{k: DeviceBuffer(self, v) for k, v in side_sizes.items()} for _ in (0, 1)]
        for name in BUFFER_ORDER:
            if name not in self.buffers and name not in dict(SIDE_FIELDS) and name not in dict(
                (o, k) for k, o in SIDE_FIELDS
            ):
                raise RuntimeError(f"unallocated buffer {name}")
        backup_names = (
            "position", "velocity", "rotation", "momentum", "cell", "force", "torque", "referencePosition",
            "referenceCell", "control", "pairs", "pairCounts", "pairOffsets", "particleStress",
            "particleDiagnostic", "timestepRows", "accumulated", "referencePositionRemainder",
            *RESIDUAL_STATE, *DAMPING_STATE, "contactCounts", "byJOffsets", "byJPairs",
            *(WALL_STATE if self.wall_count else ()),
        )
        self.backups = {name: DeviceBuffer(self, self.buffers[name].size) for name in backup_names}
        self.history_backup = {k: DeviceBuffer(self, self.sides[0][k].size) for k in side_sizes}
        self._native = self.lib.sdg_engine_create()
        if not self._native:
            raise MemoryError("GB300 engine allocation failed")
        self._finalizer = weakref.finalize(self, self.lib.sdg_engine_destroy, self._native)
        # Certified distance bounds of every shape, built once from the packed library.
        if not self.sdf:
            self.dispatch("distanceGrid", 0, self.config(dt=0))
        self.stream.synchronize()

    # ------------------------------------------------------------ plumbing
    def _add(self, name, array):
        data = np.ascontiguousarray(array)
        self.buffers[name] = DeviceBuffer(self, data.nbytes)
        if data.nbytes:
            self.buffers[name].copy_from_numpy(
                data if data.nbytes >= 16 else np.pad(data.view(np.uint8).reshape(-1), (0, 16 - data.nbytes))
            )

    def _bound(self, active):
        new, old = self.sides[active], self.sides[1 - active]
        view = dict(self.buffers)
        for k, o in SIDE_FIELDS:
            view[k], view[o] = new[k], old[k]
        return view

    def _arrays(self, active):
        """Pointer and size blocks for one history-side orientation (built
        once: the buffers never move while the engine lives)."""
        cached = self._array_cache.get(active)
        if cached is None:
            view = self._bound(active)
            ptrs = (ct.c_void_p * len(BUFFER_ORDER))(*(view[k].ptr() for k in BUFFER_ORDER))
            sizes = (ct.c_uint64 * len(BUFFER_ORDER))(*(view[k].size for k in BUFFER_ORDER))
            cached = self._array_cache[active] = (ptrs, sizes)
        return cached

    def config(self, dt=None, drag=0.0, history=None):
        return self.layout.config(
            dt=self.spec.timestep if dt is None else dt, drag=drag,
            history=self.history if history is None else history,
        )

    def _values(self, config):
        values = list(self.layout.config_values(config)) + [
            float(self.leaf_words), float(self.candidate_capacity), 0.0, float(self.specimens),
            float(self.culler is not None),
        ] + [float(self.tuning.get(k, 0)) for k in TUNING_KEYS] + [float(self.survivor_capacity),
                                                                     float(self.distance_grid),
                                                                     self.filter_margin]
        return (ct.c_double * len(values))(*values), len(values)

    def _touch(self):
        """Device work or an upload follows: host copies of device words are stale."""
        self._device_version += 1

    def _uploaded(self, buffer):
        self._touch()
        if buffer is self.buffers.get("cell"):
            self._rates = None

    def dispatch(self, name, count, config, active=None):
        """Launch one named kernel or phase on the engine stream (test and probe entry)."""
        self._touch()
        ptrs, sizes = self._arrays(self.active if active is None else active)
        values, nv = self._values(config)
        native.check(self.lib.sdg_dispatch(name.encode(), int(count), ptrs, sizes, values, nv,
                                           ct.c_void_p(self.stream.cuda_stream)))

    def synchronize(self):
        self.stream.synchronize()

    def read(self, name, dtype=np.float32, shape=None):
        return self.m.read(self.buffers[name], dtype, shape)

    def forces(self, config, *, capture_kinematics=True):
        """``Engine.forces`` (``gpu.py:547-565``) as one launch sequence."""
        self.dispatch("forces" if capture_kinematics else "forcesNoCapture", self.n, config)

    # --------------------------------------------------------- public API
    def check_errors(self):
        ctrl = self.read("control", np.uint32, (16,))
        return self._checked(ctrl)

    def _checked(self, ctrl):
        self._ctrl_cache = (self._device_version, ctrl.copy())
        if ctrl[15] != 0:
            raise RuntimeError("Arithmetic materialization mask must remain zero")
        if ctrl[0]:
            raise RejectedStep(ctrl[0])
        return ctrl

    def initialize(self):
        self.forces(self.config(dt=0))
        self.synchronize()
        self.check_errors()
        self.history = True
        self.active = 1 - self.active

    def timestep_limits(self):
        if self.spec.timestep_policy != "active-contact":
            raise ValueError("Contact limits require active-contact policy")
        rows = self.read("timestepRows", np.float32, (self.n, 4))
        with np.errstate(divide="ignore"):
            elastic = 0.1 / np.sqrt(rows[:, 0].astype(float)) * self.time_unit
            viscous = 0.1 / rows[:, 1].astype(float) * self.time_unit
        return {"elastic_seconds": elastic, "viscous_seconds": viscous}

    def advance(self, steps, *, rate=(0, 0, 0), drag=0, wall_velocities=None):
        """Transactional chunk with capacity growth (``gpu.py:597-647``)."""
        from dataclasses import replace

        if type(steps) is not int or steps < 0:
            raise ValueError("Nonnegative integer step count required")
        rate = finite_array(rate)
        if rate.shape not in {(3,), (self.specimens, 3)}:
            raise ValueError("Cell rate must be (3,) or one row per specimen")
        if not self.spec.periodic and np.any(rate != 0):
            raise ValueError("Affine cell rates require a periodic domain")
        if not np.isfinite(drag) or drag < 0:
            raise ValueError("Finite nonnegative drag required")
        if wall_velocities is not None:
            if not self.wall_count:
                raise ValueError("Wall velocities require planes")
            wall_velocities = finite_array(wall_velocities, (self.wall_count, 3))
        for attempt in range(5):
            try:
                return self._advance_once(steps, rate=rate, drag=drag, wall_velocities=wall_velocities)
            except RejectedStep as exc:
                capacity = exc.flags & CAPACITY_FLAGS
                if not capacity or exc.flags & ~CAPACITY_FLAGS or attempt == 4:
                    raise
                state = self.state()
                old = self.spec
                settings = {}
                if capacity & 8:
                    settings["bin_capacity"] = old.bin_capacity * 2
                if capacity & 16:
                    settings["pairs_per_particle"] = old.pairs_per_particle * 2
                if capacity & (32 | 64):
                    settings["contacts_per_particle"] = max(
                        old.contacts_per_particle * 2, math.ceil(2 * self.contact_capacity / self.n)
                    )
                log = self.capacity_retries + [
                    {"step": self.step, "flags": exc.flags, "new_capacities": settings}
                ]
                positions = state["position"][:, :3] * self.length_unit
                starts = np.cumsum([0] + self.layout.counts)
                specimens = [
                    (positions[a:b], state["cell"][3 * k, :3] * self.length_unit, self.ids[a:b], self.scales[a:b])
                    for k, (a, b) in enumerate(zip(starts[:-1], starts[1:]))
                ]
                replacement = Engine(
                    self.library, replace(old, **settings), None, None, None, None,
                    layout=HostLayout.batch(self.library, replace(old, **settings), specimens,
                                            trees=device_median_trees),
                    device=self.device, use_graph=self.use_graph, distance_grid=self.distance_grid,
                    filter_margin=self.filter_margin,
                )
                replacement.initial_cell = self.initial_cell.copy()
                replacement.tuning = dict(self.tuning)
                if self.culler is not None:
                    self.culler.attach(replacement)
                replacement.restore(state, self.step)
                self._adopt(replacement)
                self.capacity_retries = log

    def _adopt(self, replacement):
        """Take over a grown replacement engine's buffers (capacity retry)."""
        self._finalizer()
        replacement._finalizer.detach()
        self.__dict__.update(replacement.__dict__)
        self._finalizer = weakref.finalize(self, self.lib.sdg_engine_destroy, self._native)
        self.m = GB300Device(self)
        me = weakref.ref(self)
        for group in (self.buffers, self.backups, self.history_backup, *self.sides):
            for buffer in group.values():
                buffer._engine = me

    def _backup(self, restore=False):
        committed = self.sides[1 - self.active]
        if restore:
            count = self._backup_count
            self._touch()
        elif self._ctrl_cache is not None and self._ctrl_cache[0] == self._device_version:
            count = int(self._ctrl_cache[1][2])
        else:
            count = int(self.read("control", np.uint32, (16,))[2])
        if count < 0 or count > self.contact_capacity:
            raise ValueError("Committed contact count is outside capacity")
        copies = []
        for name, backup in self.backups.items():
            src, dst = (backup, self.buffers[name]) if restore else (self.buffers[name], backup)
            copies.append((dst, src, min(dst.size, src.size)))
        for name, backup in self.history_backup.items():
            src, dst = (backup, committed[name]) if restore else (committed[name], backup)
            nbytes = 16 * count if name in ("meta", "slip", "normalArea") else min(dst.size, src.size)
            copies.append((dst, src, nbytes))
        n = len(copies)
        native.check(self.lib.sdg_copy_buffers(
            (ct.c_void_p * n)(*(d.ptr() for d, _, _ in copies)), (ct.c_void_p * n)(*(s.ptr() for _, s, _ in copies)),
            (ct.c_uint64 * n)(*(b for _, _, b in copies)), n, ct.c_void_p(self.stream.cuda_stream)))
        self._backup_count = count

    def _advance_once(self, steps, *, rate=(0, 0, 0), drag=0, wall_velocities=None):
        if getattr(self, "invalid", False):
            raise RuntimeError("Engine is invalid; restore a checkpoint")
        if steps < 1:
            return
        rows = (np.broadcast_to(np.asarray(rate, float), (self.specimens, 3)) * self.time_unit).astype(np.float32)
        original_cell = None
        if self._rates is None or not np.array_equal(self._rates, rows):
            # Only the rate rows change; the device advances the box rows.
            cell = self.read("cell", np.float32, (3 * self.specimens, 4))
            original_cell = cell.copy()
            cell[1::3, :3] = rows
            self.buffers["cell"].copy_from_numpy(cell)
            self._rates = rows
        self._backup()
        original_active, original_history = self.active, self.history
        original_velocity = None
        if wall_velocities is not None:
            # gpu.py:682-713: new wall velocities; the committed rows' wall
            # power is refreshed, or with viscous planes (whose contact law
            # reads the wall velocity) the committed contacts are re-resolved.
            original_velocity = self.read("wallVelocity", np.float32, (self.wall_count, 4))
            velocity = np.zeros((self.wall_count, 4), np.float32)
            velocity[:, :3] = f4(wall_velocities * self.time_unit / self.length_unit)[:, :3]
            if not np.isfinite(velocity).all():
                raise ValueError("Wall velocities cannot be represented in normalized FP32 units")
            self.buffers["wallVelocity"].copy_from_numpy(velocity)
            if any(p.get("normal_viscosity", 0) > 0 for p in self.spec.planes) and not np.array_equal(
                original_velocity, velocity
            ):
                self.forces(self.config(dt=0, drag=drag))
                self.active = 1 - self.active
                self.history = True
            else:
                self.dispatch("refreshWallPower", self.n * self.wall_count, self.config(drag=drag))
        done = 0
        if not self.history:
            # The first step after construction has no committed history.
            self._launch_steps(1, drag)
            self.history = True
            done = 1
        self._launch_steps(steps - done, drag)
        self.synchronize()
        try:
            self.check_errors()
        except RuntimeError:
            self.active, self.history = original_active, original_history
            self._backup(restore=True)
            self.synchronize()
            if original_cell is not None:
                self.buffers["cell"].copy_from_numpy(original_cell)
            if original_velocity is not None:
                self.buffers["wallVelocity"].copy_from_numpy(original_velocity)
            raise
        self.step += steps

    def _launch_steps(self, steps, drag):
        if steps <= 0:
            return
        self._touch()
        ptrs, sizes = self._arrays(self.active)
        values, nv = self._values(self.config(drag=drag))
        native.check(self.lib.sdg_engine_advance(
            ct.c_void_p(self._native), ptrs, sizes, values, nv, steps, int(self.use_graph),
            ct.c_void_p(self.stream.cuda_stream)))
        self.active ^= steps & 1

    def state(self):
        """Checkpoint arrays (``gpu.py:893-936``)."""
        out = {}
        for name in STATE_NAMES:
            rows = 3 * self.specimens if name == "cell" else 2 * self.specimens if name == "cellLog" else self.n
            out[name] = self.read(name, np.float32, (rows, 4))
        if self.viscous:
            for name in DAMPING_STATE:
                out[name] = self.read(name, np.float32, (self.n, 4))
        ctrl = self.check_errors()
        count = int(ctrl[2])
        side = self.sides[1 - self.active]
        out["contacts"] = count
        for name in ("meta", "slip", "normalArea"):
            out[name] = self.m.read_prefix(side[name], 4 * count, np.uint32 if name == "meta" else np.float32,
                                           shape=(count, 4))
        if self.wall_count:
            for name in WALL_STATE:
                out[name] = self.read(name, np.float32, (self.buffers[name].size // 16, 4))
        return out

    def _history_tables(self, meta):
        """Committed-side runs for a contact list in arbitrary order.

        Sorts the grain-grain contacts by (first grain, second grain,
        direction, node rank) and the plane contacts after them by (wall,
        grain, node rank); returns the permutation with the per-grain pair
        runs, per-pair contact starts and per-(wall, grain) starts the device
        merge reads.
        """
        g = self.layout.geometry
        n = self.n
        src, dst, node = (meta[:, k].astype(np.int64) for k in range(3))
        if len(meta) and (src.max() >= n or dst.max() >= n + self.wall_count):
            raise ValueError("Checkpoint contact refers to a missing grain")
        wall = dst >= n
        grains, planes = np.flatnonzero(~wall), np.flatnonzero(wall)
        if self.sdf:
            wall_key = node[planes]
        else:
            wall_key = g["meshSampleRank"][g["sampleInfo"][self.ids[src[planes]], 0].astype(np.int64)
                                           + node[planes]].astype(np.int64)
        wall_order = planes[np.lexsort((wall_key, src[planes], dst[planes]))]
        item = (dst[wall_order] - n) * n + src[wall_order]
        wall_starts = (len(grains) + np.searchsorted(item, np.arange(self.wall_count * n + 1))).astype(np.uint32)
        src, dst, node = src[grains], dst[grains], node[grains]
        a, b = np.minimum(src, dst), np.maximum(src, dst)
        if self.sdf:
            # The SDF emit order: s by virtual lane (s mod 64), then s / 64.
            s = np.where(src > dst, g["sampleInfo"][self.ids[a], 1].astype(np.int64) + node, node)
            key = ((s & 63) << 24) | (s >> 6)
        else:
            base = g["sampleInfo"][self.ids[src], 0].astype(np.int64)
            rank = g["meshSampleRank"][base + node].astype(np.int64)
            key = ((src > dst).astype(np.int64) << 31) | rank
        order = np.lexsort((key, b, a))
        a, b = a[order], b[order]
        pair_start = np.flatnonzero(np.r_[True, (a[1:] != a[:-1]) | (b[1:] != b[:-1])]) if len(a) else np.zeros(0, int)
        pair_a = a[pair_start]
        offsets = np.searchsorted(pair_a, np.arange(n + 1)).astype(np.uint32)
        starts = np.r_[pair_start, len(a)].astype(np.uint32)
        order = np.r_[grains[order], wall_order].astype(np.int64)
        return order, offsets, b[pair_start].astype(np.uint32), starts, wall_starts

    def restore(self, state, step):
        """Restart from checkpoint arrays (``gpu.py:1016-1092``)."""
        if self.wall_count:
            for name in WALL_STATE:
                value = finite_array(state[name])
                if value.shape != (self.buffers[name].size // 16, 4):
                    raise ValueError("Checkpoint wall state shape mismatch")
            normals = np.array([p["normal"] for p in self.spec.planes], np.float32)
            if not np.array_equal(np.asarray(state["wallPlane"])[:, :3], normals):
                raise ValueError("Checkpoint plane normal identity mismatch")
            if self.spec.boundary_box is not None:
                offsets = (np.asarray(state["wallPlane"][:, 3], float) + state["wallRemainder"][:, 3]) * self.length_unit
                box_extents(offsets, self.spec.boundary_box,
                            np.asarray(state["cell"][0, :3], float) * self.length_unit)
        for name in DAMPING_STATE:
            value = state[name] if self.viscous else np.zeros((self.n, 4), np.float32)
            self.buffers[name].copy_from_numpy(np.asarray(value, np.float32))
        for name in STATE_NAMES:
            self.buffers[name].copy_from_numpy(np.asarray(state[name], np.float32))
        if self.wall_count:
            for name in WALL_STATE:
                self.buffers[name].copy_from_numpy(np.asarray(state[name], np.float32))
        count = int(state["contacts"])
        if count < 0 or count > self.contact_capacity:
            raise ValueError("Checkpoint contact count is outside capacity")
        values = {}
        for name in ("meta", "slip", "normalArea"):
            v = np.asarray(state[name], np.uint32 if name == "meta" else np.float32)
            if v.shape != (count, 4):
                raise ValueError("Checkpoint contact history shape mismatch")
            values[name] = v
        order, offsets, pair_b, starts, wall_starts = self._history_tables(values["meta"])
        committed = self.sides[1]
        for name in ("meta", "slip", "normalArea"):
            committed[name].write_prefix(values[name][order])
        committed["sidePairOffsets"].write_prefix(offsets)
        committed["sidePairB"].write_prefix(pair_b)
        committed["sideContactStart"].write_prefix(starts)
        if self.wall_count:
            committed["sideWallStart"].write_prefix(wall_starts)
        ctrl = np.zeros(16, np.uint32)
        ctrl[2], ctrl[4] = count, 1
        self.buffers["control"].copy_from_numpy(ctrl)
        self.active, self.history = 0, True
        self.forces(self.config(dt=0), capture_kinematics=False)
        self.synchronize()
        self.check_errors()
        self.active = 1
        self.step = step

    def _diagnostic_rows(self, config):
        """The reduced diagnostic and fabric rows, the cell rows and the control
        words (``sdg_engine_diagnostics``)."""
        if self._diagnostic_scratch is None:
            size = 16 * 8 * ((max(self.n, self.pair_capacity) + 255) // 256)
            self._diagnostic_scratch = (DeviceBuffer(self, size), DeviceBuffer(self, size), size)
        a, b, size = self._diagnostic_scratch
        self._touch()
        ptrs, sizes = self._arrays(self.active)
        values, nv = self._values(config)
        host = self._staging[:272]
        native.check(self.lib.sdg_engine_diagnostics(ptrs, sizes, values, nv, ct.c_void_p(a.ptr()),
                                                     ct.c_void_p(b.ptr()), size, ct.c_void_p(host.data_ptr()),
                                                     ct.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        raw = host.numpy().copy()
        self.d2h_bytes += 272
        return (raw[:128].view(np.float32), raw[128:160].view(np.float32), raw[160:208].view(np.float32),
                raw[208:272].view(np.uint32))

    def _reduce(self, name, rows, max_row, read=True):
        """Reference 256-wide tree reduction to one row set (``diagnostic.slang:3-28``);
        with ``read=False`` the device buffer holding the rows is returned."""
        src = self.buffers[name]
        n = self.n if name == "diagnosticRows" else self.pair_capacity
        level = 0
        while n > 1:
            groups = (n + 255) // 256
            key = (name, level)
            out = self._reduce_scratch.get(key)
            if out is None or out.size < 16 * rows * groups:
                out = self._reduce_scratch[key] = DeviceBuffer(self, 16 * rows * groups)
            native.check(self.lib.sdg_reduce_rows(ct.c_void_p(src.ptr()), ct.c_void_p(out.ptr()), n, rows,
                                                  max_row, ct.c_void_p(self.stream.cuda_stream)))
            src, n, level = out, groups, level + 1
        return self.m.read_prefix(src, 4 * rows, np.float32, shape=(rows, 4)) if read else src

    def _reduce_walls(self):
        """Per-wall sums of the (wall, grain) rows (``gpu.py:774-786``); the
        device buffer holding one row set per wall."""
        src, n, level, w = self.buffers["wallRows"], self.n, 0, self.wall_count
        while n > 1:
            groups = (n + 255) // 256
            key = ("wallRows", level)
            out = self._reduce_scratch.get(key)
            if out is None or out.size < 48 * w * groups:
                out = self._reduce_scratch[key] = DeviceBuffer(self, 48 * w * groups)
            native.check(self.lib.sdg_reduce_wall_rows(ct.c_void_p(src.ptr()), ct.c_void_p(out.ptr()), n, w,
                                                       ct.c_void_p(self.stream.cuda_stream)))
            src, n, level = out, groups, level + 1
        return src

    def _wall_results(self, wall_data, plane, remainder, velocity):
        """The ``walls`` rows of :meth:`diagnostics` (``gpu.py:803-833``) and
        the plane offsets in metres."""
        plane, remainder = plane.astype(float), remainder.astype(float)
        offsets = (plane[:, 3] + remainder[:, 3]) * self.length_unit
        results = [
            dict(
                index=w,
                normal=plane[w, :3].tolist(),
                offset=float(offsets[w]),
                velocity=(velocity[w, :3] * self.length_unit / self.time_unit).tolist(),
                reaction=(wall_data[w, 0, :3] * self.force_unit).tolist(),
                reaction_moment_origin=(wall_data[w, 1, :3] * self.energy_unit).tolist(),
                active_surface_contacts=int(wall_data[w, 0, 3].view(np.uint32)),
                power=float(wall_data[w, 1, 3] * self.energy_unit / self.time_unit),
                work=float(wall_data[w, 2, 0] * self.energy_unit),
            )
            for w in range(self.wall_count)
        ]
        return results, offsets

    def diagnostics(self):
        """Stress, energies, contact counts, fabric and wall rows (``gpu.py:746-891``)."""
        c = self.config()
        w = self.wall_count
        if w:
            self.dispatch("diagnosticRows", self.n, c)
            rows = self._reduce("diagnosticRows", 8, 4, read=False)
            self.dispatch("fabricRows", self.pair_capacity, c)
            fabric_rows = self._reduce("fabricRows", 2, -1, read=False)
            reads = [(rows, 16 * 8, np.float32), (fabric_rows, 16 * 2, np.float32),
                     (self.buffers["cell"], 16 * 3, np.float32), (self.buffers["control"], 4 * 16, np.uint32)]
            reads += [(self._reduce_walls(), 48 * w, np.float32), (self.buffers["wallPlane"], 16 * w, np.float32),
                      (self.buffers["wallRemainder"], 16 * w, np.float32),
                      (self.buffers["wallVelocity"], 16 * w, np.float32)]
            # One wait for all the small reads.
            data, fabric_data, cell, ctrl, *wall_reads = read_batch(self, reads)
        else:
            # Without planes: the rows, their reductions and the reads in one
            # native call and one wait.
            data, fabric_data, cell, ctrl = self._diagnostic_rows(c)
            wall_reads = []
        data, fabric_data, cell = data.reshape(8, 4), fabric_data.reshape(2, 4), cell.reshape(3, 4)
        ctrl = self._checked(ctrl)
        active_pairs = round(float(fabric_data[1, 2]))
        fabric = np.array(
            [
                [fabric_data[0, 0], fabric_data[0, 3], fabric_data[1, 0]],
                [fabric_data[0, 3], fabric_data[0, 1], fabric_data[1, 1]],
                [fabric_data[1, 0], fabric_data[1, 1], fabric_data[0, 2]],
            ]
        ) / max(active_pairs, 1)
        box = cell[0, :3].astype(float) * self.length_unit
        domain = box.copy()
        walls = []
        if w:
            wall_data, plane, remainder, velocity = wall_reads
            walls, offsets = self._wall_results(wall_data.reshape(w, 3, 4), plane.reshape(w, 4),
                                                remainder.reshape(w, 4), velocity.reshape(w, 4))
            if self.spec.boundary_box is not None:
                box = box_extents(offsets, self.spec.boundary_box, domain)
        volume = float(box.prod())
        contact = data[:3, :3].astype(float) * self.energy_unit / volume
        kinetic = data[3:6, :3].astype(float) * self.energy_unit / volume
        total = contact + kinetic
        symmetric = 0.5 * (total + total.T)
        radial = 0.5 * (symmetric[0, 0] + symmetric[1, 1])
        solid = self.solid_volume
        return {
            "step": self.step,
            "elapsed_time": self.step * self.spec.timestep,
            "cell": box.tolist(),
            "domain_cell": domain.tolist(),
            "walls": walls,
            "stress": total.tolist(),
            "contact_stress": contact.tolist(),
            "kinetic_stress": kinetic.tolist(),
            "stress_antisymmetry": float(np.linalg.norm(total - total.T) / max(np.linalg.norm(total), 1e-30)),
            "p": float(np.trace(symmetric) / 3),
            "q": float(symmetric[2, 2] - radial),
            "axial_strain": float(1 - box[2] / self.initial_cell[2]),
            "volumetric_strain": float(np.sum(1 - box / self.initial_cell)),
            "volume_ratio": float(volume / np.prod(self.initial_cell)),
            "log_strain": (-np.log(box / self.initial_cell)).tolist(),
            "void_ratio": float(volume / solid - 1),
            "kinetic_energy": float(data[0, 3] * self.energy_unit),
            "elastic_energy_proxy": float(data[1, 3] * self.energy_unit),
            "contact_normal": self.spec.contact_normal,
            "elastic_energy_interpretation": "proxy; source-normal forces are not its gradient"
            if self.spec.contact_normal == "source-surface-experimental"
            else "existing nodal spring energy proxy",
            "unbalanced_force": float(data[2, 3] / max(data[3, 3], 1e-30)),
            "max_overlap_fraction": float(data[4, 3]),
            "friction_dissipation_last_step": float(data[5, 3] * self.energy_unit),
            "candidate_pairs": int(ctrl[1]),
            "active_surface_contacts": int(ctrl[2]),
            "active_grain_pairs": active_pairs,
            "coordination": 2 * active_pairs / self.n,
            "fabric": fabric.tolist(),
            "sliding_fraction": float(ctrl[6] / max(ctrl[2], 1)),
            "cell_log_rate": (cell[1, :3] / self.time_unit).tolist(),
            "friction_dissipation": float(data[6, 0] * self.energy_unit),
            "drag_dissipation": float(data[6, 1] * self.energy_unit),
            "cell_work": float(data[6, 2] * self.energy_unit),
            "wall_work": float(data[6, 3] * self.energy_unit),
            "normal_contact_dissipation": float(data[7, 0] * self.energy_unit),
            "normal_contact_power": float(data[7, 1] * self.energy_unit / self.time_unit),
        }

    def run_steps(self, steps, *, drag=0.0):
        """Launch ``steps`` timesteps with no host synchronization, backup or
        error check (the device-resident inner loop of :meth:`advance`)."""
        self._launch_steps(int(steps), drag)
        self.history = True
        self.step += int(steps)

    def profile_phases(self, *, drag=0.0):
        """Device milliseconds per phase of one committed step (CUDA events)."""
        self._touch()
        ptrs, sizes = self._arrays(self.active)
        values, nv = self._values(self.config(drag=drag))
        out = (ct.c_float * len(native.PHASES))()
        native.check(self.lib.sdg_engine_profile(ct.c_void_p(self._native), ptrs, sizes, values, nv, out,
                                                 ct.c_void_p(self.stream.cuda_stream)))
        self.active ^= 1
        self.history = True
        self.step += 1
        return dict(zip(native.PHASES, map(float, out)))

    def profile_step(self):
        """One real step timed by subsystem (``gpu.py:938-1014``), CUDA events."""
        if self.spec.timestep_policy == "active-contact":
            raise ValueError("Use advance for active-contact policy: profiling has no rollback")
        ms = self.profile_phases()
        self.check_errors()
        seconds = {
            "drift": ms["drift"] / 1e3,
            "neighbours": ms["neighbours"] / 1e3,
            "contact_geometry": (ms["pair_cull"] + ms["node_filter"] + ms["node_query"] + ms["contact_emit"]) / 1e3,
            "friction_and_history": ms["friction_and_history"] / 1e3,
            "force_reduction": ms["force_reduction"] / 1e3,
            "final_kick": ms["final_kick"] / 1e3,
        }
        return {
            "timestamp_frequency_hz": 1e3,
            "timing_source": "CUDA events between launch groups on the engine stream",
            "seconds": seconds,
            "phases_ms": ms,
            "total_gpu_seconds": sum(seconds.values()),
        }
