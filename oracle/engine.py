"""CPU ORACLE engine — test infrastructure only (never imported by the product).

Drives the serial C++ oracle kernels (``dem_oracle.cpp``) with numpy buffers in
the reference's dispatch order for one mesh-surface DEM step:
``Engine.forces`` (``src/sand_atlas_dem/gpu.py:547-565``) inside
``Engine._advance_once`` (``gpu.py:714-726``), with the reference's
double-buffered friction history (``gpu.py:305-316``, ``:490-527``),
``initialize`` (``gpu.py:580-587``), ``state`` (``gpu.py:893-936``),
``restore`` (``gpu.py:1016-1092``) and ``diagnostics`` reductions
(``gpu.py:746-891``, tree order of ``cpu.py:491-537``).

Optionally the collector phase runs the reference's own compiled collector
(``oracle/_ref/collector_ref.so``, built by ``build_ref.sh``) instead of the
restatement; both bind the same 77 buffers.
"""

import ctypes as ct
import subprocess
from pathlib import Path

import numpy as np

from sand_atlas_dem_gb300.model import (
    DAMPING_STATE,
    RESOURCE_ORDER,
    STATE_NAMES,
    WALL_STATE,
    HostLayout,
    RejectedStep,
)

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "libdem_oracle.so"
# The same source built in double precision: the FP64 drift oracle.
ORACLE_LIB64 = HERE / "_build" / "libdem_oracle64.so"
REF_LIB = HERE / "_ref" / "collector_ref.so"


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return ORACLE_LIB


_LIBS = {}


def library(precision="fp32"):
    if precision not in _LIBS:
        path = ORACLE_LIB64 if precision == "fp64" else ORACLE_LIB
        if not path.exists():
            build()
        lib = ct.CDLL(str(path))
        lib.oracle_dispatch.argtypes = [
            ct.c_char_p, ct.c_uint32, ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_uint64),
            ct.POINTER(ct.c_double), ct.c_uint32,
        ]
        lib.oracle_dispatch.restype = ct.c_int
        _LIBS[precision] = lib
    return _LIBS[precision]


class ReferenceCollector:
    """ctypes binding of the reference's archived ``cpu_dispatch`` (``cpu.py:391-428``)."""

    def __init__(self, path=REF_LIB):
        self.lib = ct.CDLL(str(path))
        self.fn = self.lib.cpu_dispatch
        self.fn.argtypes = [ct.c_uint32, ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_uint64),
                            ct.POINTER(ct.c_double), ct.c_void_p]
        self.fn.restype = ct.c_int
        create = self.lib.cpu_scratch_create
        create.restype = ct.c_void_p
        self.destroy = self.lib.cpu_scratch_destroy
        self.destroy.argtypes = [ct.c_void_p]
        self.scratch = create()

    def __del__(self):
        if getattr(self, "scratch", None):
            self.destroy(self.scratch)

    def dispatch(self, count, pointers, sizes, values, threads=1):
        vals = (ct.c_double * (len(values) + 1))(*values, float(threads))
        if self.fn(count, pointers, sizes, vals, self.scratch):
            raise RuntimeError("reference collector failed")


def _zeros4(rows, dtype=np.float32):
    return np.zeros((max(1, rows), 4), dtype)


class OracleEngine:
    """Reference-order CPU engine over the restated kernels.

    ``precision="fp64"`` runs the same kernels in double precision (every
    float buffer float64, every FP32 operation in double): the FP64 drift
    oracle.  Its state arrays are float64; a position is held whole in
    ``position`` (its remainder row stays zero)."""

    def __init__(self, library_, spec, positions, cell, shape_ids, scales, *, collector=None, threads=1,
                 precision="fp32"):
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision is fp32 or fp64")
        if precision == "fp64" and collector is not None:
            raise ValueError("the reference's compiled collector is FP32 only")
        self.precision = precision
        real = np.float64 if precision == "fp64" else np.float32
        self.layout = h = HostLayout(library_, spec, positions, cell, shape_ids, scales)
        self.spec, self.library, self.n = spec, library_, h.n
        self.viscous = spec.viscous
        self.step = 0
        self.history = False
        self.active = 0
        self.collector = collector  # None: restated collector; else ReferenceCollector
        self.threads = max(1, int(threads))
        for name in ("length_unit", "time_unit", "mass_unit", "force_unit", "stress_unit",
                     "energy_unit", "ids", "scales", "pair_capacity", "contact_capacity",
                     "hash_size", "bin_count", "bin_capacity", "initial_cell"):
            setattr(self, name, getattr(h, name))
        b = dict(h.geometry)
        b.update(h.initial_state())
        if precision == "fp64":
            b = {k: (v.astype(np.float64) if v.dtype == np.float32 else v) for k, v in b.items()}
            # The whole FP64 centre in one value (hi + lo is exact in double).
            b["position"] = b["position"] + b["positionRemainder"]
            b["positionRemainder"][...] = 0
            b["position"][:, :3] = np.asarray(h.normalized_position, np.float64)
        pc, cc, n = h.pair_capacity, h.contact_capacity, h.n
        b["meshPairMask"] = np.zeros(pc, np.uint32)
        b["meshPairTransform"] = _zeros4(8 * pc, real)
        b["fabricRows"] = _zeros4(2 * pc, real)
        b["binCounts"] = np.zeros(h.bin_count, np.uint32)
        b["binParticles"] = np.zeros(h.bin_count * h.bin_capacity, np.uint32)
        for name, count in (("pairCounts", n), ("pairOffsets", n), ("contactCounts", pc),
                            ("contactOffsets", pc), ("heads", n), ("next", 2 * cc)):
            b[name] = np.zeros(count, np.uint32)
        b["pairs"] = np.zeros((pc, 2), np.uint32)
        b["pointDepth"] = _zeros4(cc, real)
        b["contactForce"] = _zeros4(cc, real)
        b["normalLossPower"] = np.zeros(cc, real)
        self.wall_count = h.wall_count
        b.update({k: (v.astype(real) if v.dtype == np.float32 else v.copy()) for k, v in h.walls.items()})
        self.buffers = b
        self.sides = [
            {
                "meta": np.zeros((cc, 4), np.uint32),
                "slip": _zeros4(cc, real),
                "normalArea": _zeros4(cc, real),
                "hash": np.full(h.hash_size, 0xFFFFFFFF, np.uint32),
            }
            for _ in (0, 1)
        ]

    # -- dispatch ---------------------------------------------------------
    def _resources(self):
        new, old = self.sides[self.active], self.sides[1 - self.active]
        view = dict(self.buffers)
        view.update(meta=new["meta"], slip=new["slip"], normalArea=new["normalArea"],
                    hash=new["hash"], oldMeta=old["meta"], oldSlip=old["slip"],
                    oldNormal=old["normalArea"], oldHash=old["hash"])
        return [view[name] for name in RESOURCE_ORDER]

    def config(self, dt=None, drag=0.0, history=None):
        return self.layout.config(
            dt=self.spec.timestep if dt is None else dt, drag=drag,
            history=self.history if history is None else history,
        )

    def dispatch(self, name, count, config, extra=(), uniforms=()):
        arrays = self._resources() + list(extra)
        for a in arrays:
            assert a.flags.c_contiguous
        pointers = (ct.c_void_p * len(arrays))(*(a.ctypes.data for a in arrays))
        sizes = (ct.c_uint64 * len(arrays))(*(a.nbytes for a in arrays))
        values = list(self.layout.config_values(config)) + [float(u) for u in uniforms]
        if name == "collectMeshFrontiers":
            if self.collector is not None:
                self.collector.dispatch(count, pointers, sizes, values, self.threads)
                return
            values.append(float(self.threads))
        vals = (ct.c_double * len(values))(*values)
        if library(self.precision).oracle_dispatch(name.encode(), int(count), pointers, sizes, vals, len(values)):
            raise ValueError(f"oracle has no kernel {name}")

    # -- the reference step ---------------------------------------------
    def neighbours(self, c):
        n = self.n
        self.dispatch("clearBins", self.bin_count, c)
        self.dispatch("fillBins", n, c)
        self.dispatch("countPairs", n, c)
        self.dispatch("scanPairs", 1, c)
        self.dispatch("emitPairs", n, c)

    def collect(self, c, exhaustive=False):
        pc = self.pair_capacity
        if self.spec.contact_geometry == "sdf":  # gpu.py:537-543
            self.dispatch("countContacts", pc, c)
            self.dispatch("scanContacts", 1, c)
            self.dispatch("contactTotal", 1, c)
            self.dispatch("emitContacts", pc, c)
        elif exhaustive:
            self.dispatch("exhaustiveContacts", 1, c)
        else:
            self.dispatch("resetMeshContacts", pc, c)
            self.dispatch("prepareMeshPairs", pc, c)
            ctrl = self.buffers["control"]
            self.dispatch("collectMeshFrontiers", int(min(ctrl[1], pc)), c)
        if self.wall_count:  # gpu.py:544-545
            self.dispatch("collectWallContacts", self.n * self.wall_count, c)

    def friction(self, c):
        self.dispatch("clearContactStorage", max(self.n, self.hash_size), c)
        self.dispatch("resolveContacts", self.contact_capacity, c)
        self.dispatch("buildHistoryHash", self.contact_capacity, c)

    def forces(self, c, *, capture_kinematics=True, exhaustive=False):
        if self.viscous and capture_kinematics:
            self.dispatch("captureContactKinematics", self.n, c)
        self.neighbours(c)
        self.collect(c, exhaustive)
        self.friction(c)
        self.dispatch("gather", self.n, c)
        if self.wall_count:
            self.dispatch("gatherWallRows", self.n * self.wall_count, c)
        if self.spec.timestep_policy == "active-contact":
            self.dispatch("checkContactTimestep", self.n, c)

    def begin(self, c):
        if self.spec.timestep_policy == "active-contact":
            self.dispatch("checkContactTimestep", self.n, c)
        self.dispatch("beginStep", self.n, c)
        self.dispatch("advanceCell", 1, c)
        if self.wall_count:
            self.dispatch("advanceWalls", 1, c)
        self.dispatch("checkRebuild", self.n, c)

    def check_errors(self):
        ctrl = self.buffers["control"]
        if ctrl[15] != 0:
            raise RuntimeError("Arithmetic materialization mask must remain zero")
        if ctrl[0]:
            raise RejectedStep(ctrl[0])
        return ctrl.copy()

    def initialize(self):
        self.forces(self.config(dt=0))
        self.check_errors()
        self.history = True
        self.active = 1 - self.active

    def _snapshot(self):
        return (
            {k: v.copy() for k, v in self.buffers.items()},
            [{k: v.copy() for k, v in s.items()} for s in self.sides],
            self.active,
            self.history,
        )

    def _rollback(self, snap):
        buffers, sides, active, history = snap
        for k, v in buffers.items():
            self.buffers[k][...] = v
        for s, saved in zip(self.sides, sides):
            for k, v in saved.items():
                s[k][...] = v
        self.active, self.history = active, history

    def advance(self, steps, *, rate=(0, 0, 0), drag=0.0, exhaustive=False, wall_velocities=None):
        if type(steps) is not int or steps < 0:
            raise ValueError("Nonnegative integer step count required")
        if steps < 1:
            return
        snap = self._snapshot()
        self.buffers["cell"][1, :3] = np.asarray(rate, float) * self.time_unit
        if wall_velocities is not None:  # gpu.py:682-713
            old = self.buffers["wallVelocity"].copy()
            new = np.zeros((self.wall_count, 4), np.float32)
            new[:, :3] = np.asarray(wall_velocities, float) * self.time_unit / self.length_unit
            self.buffers["wallVelocity"][...] = new
            if any(p.get("normal_viscosity", 0) > 0 for p in self.spec.planes) and not np.array_equal(old, new):
                self.forces(self.config(dt=0, drag=drag))
                self.active = 1 - self.active
                self.history = True
            else:
                self.dispatch("refreshWallPower", self.n * self.wall_count, self.config(drag=drag))
        for _ in range(steps):
            c = self.config(drag=drag)
            self.begin(c)
            self.forces(c, exhaustive=exhaustive)
            self.dispatch("finishStep", self.n, c)
            self.active = 1 - self.active
            self.history = True
        try:
            self.check_errors()
        except RuntimeError:
            self._rollback(snap)
            raise
        self.step += steps

    # -- state ------------------------------------------------------------
    def state(self):
        n = self.n
        out = {}
        for name in STATE_NAMES:
            rows = 3 if name == "cell" else 2 if name == "cellLog" else n
            out[name] = self.buffers[name][:rows].copy()
        if self.viscous:
            for name in DAMPING_STATE:
                out[name] = self.buffers[name].copy()
        ctrl = self.check_errors()
        count = int(ctrl[2])
        side = self.sides[1 - self.active]
        out["contacts"] = count
        for name in ("meta", "slip", "normalArea"):
            out[name] = side[name][:count].copy()
        if self.wall_count:
            for name in WALL_STATE:
                out[name] = self.buffers[name].copy()
        return out

    def restore(self, state, step):
        for name in DAMPING_STATE:
            self.buffers[name][...] = state[name] if self.viscous else 0
        for name in STATE_NAMES:
            self.buffers[name][...] = np.asarray(state[name], self.buffers[name].dtype)
        if self.wall_count:
            for name in WALL_STATE:
                self.buffers[name][...] = np.asarray(state[name], np.float32)
        count = int(state["contacts"])
        if count < 0 or count > self.contact_capacity:
            raise ValueError("Checkpoint contact count is outside capacity")
        committed = self.sides[1]
        for name in ("meta", "slip", "normalArea"):
            values = np.asarray(state[name], np.uint32 if name == "meta" else np.float32)
            if values.shape != (count, 4):
                raise ValueError("Checkpoint contact history shape mismatch")
            committed[name][:count] = values
        ctrl = np.zeros(16, np.uint32)
        ctrl[2], ctrl[4] = count, 1
        self.buffers["control"][...] = ctrl
        self.active, self.history = 1, True
        c = self.config(dt=0)
        self.dispatch("clearContactStorage", max(self.n, self.hash_size), c)
        self.dispatch("buildHistoryHash", self.contact_capacity, c)
        self.check_errors()
        self.active = 0
        self.buffers["control"][...] = ctrl
        self.forces(self.config(dt=0), capture_kinematics=False)
        self.check_errors()
        self.active = 1
        self.step = step

    def diagnostic_rows(self):
        """Per-grain rows and their reduction in the reference tree order."""
        c = self.config()
        self.dispatch("diagnosticRows", self.n, c)
        self.dispatch("fabricRows", self.pair_capacity, c)
        rows = tree_reduce(self.buffers["diagnosticRows"].reshape(self.n, 8, 4), max_field=(4, 3))
        fabric = tree_reduce(self.buffers["fabricRows"].reshape(self.pair_capacity, 2, 4))
        return rows, fabric

    def diagnostics(self):
        """The reference's diagnostics dictionary (``gpu.py:788-891``) from
        the oracle's tree-reduced rows: stress tensors, p/q, strains, energies,
        contact counts, coordination, fabric and sliding fraction.  Periodic
        specimens (plane rows are :meth:`wall_rows`)."""
        data, fabric_data = self.diagnostic_rows()
        ctrl = self.check_errors()
        active_pairs = round(float(fabric_data[1, 2]))
        # FP32 rows divided in FP32, as the reference's numpy expression does.
        f = fabric_data
        fabric = np.array([[f[0, 0], f[0, 3], f[1, 0]], [f[0, 3], f[0, 1], f[1, 1]],
                           [f[1, 0], f[1, 1], f[0, 2]]]) / max(active_pairs, 1)
        cell = self.buffers["cell"][:3]
        box = cell[0, :3].astype(float) * self.length_unit
        volume = float(box.prod())
        energy = self.energy_unit
        contact = data[:3, :3].astype(float) * energy / volume
        kinetic = data[3:6, :3].astype(float) * energy / volume
        total = contact + kinetic
        sym = 0.5 * (total + total.T)
        solid = sum(self.library.shapes[int(i)].volume * s**3 for i, s in zip(self.ids, self.scales))
        initial = np.asarray(self.initial_cell, float)
        return {
            "step": self.step, "cell": box.tolist(), "stress": total.tolist(), "contact_stress": contact.tolist(),
            "kinetic_stress": kinetic.tolist(),
            "stress_antisymmetry": float(np.linalg.norm(total - total.T) / max(np.linalg.norm(total), 1e-30)),
            "p": float(np.trace(sym) / 3), "q": float(sym[2, 2] - 0.5 * (sym[0, 0] + sym[1, 1])),
            "axial_strain": float(1 - box[2] / initial[2]), "volumetric_strain": float(np.sum(1 - box / initial)),
            "volume_ratio": float(volume / np.prod(initial)), "log_strain": (-np.log(box / initial)).tolist(),
            "void_ratio": float(volume / solid - 1), "kinetic_energy": float(data[0, 3] * energy),
            "elastic_energy_proxy": float(data[1, 3] * energy),
            "unbalanced_force": float(data[2, 3] / max(data[3, 3], 1e-30)),
            "max_overlap_fraction": float(data[4, 3]),
            "friction_dissipation_last_step": float(data[5, 3] * energy),
            "candidate_pairs": int(ctrl[1]), "active_surface_contacts": int(ctrl[2]),
            "active_grain_pairs": active_pairs, "coordination": 2 * active_pairs / self.n,
            "fabric": fabric.tolist(), "sliding_fraction": float(ctrl[6] / max(ctrl[2], 1)),
            "cell_log_rate": (cell[1, :3] / self.time_unit).tolist(),
            "friction_dissipation": float(data[6, 0] * energy), "drag_dissipation": float(data[6, 1] * energy),
            "cell_work": float(data[6, 2] * energy), "wall_work": float(data[6, 3] * energy),
            "normal_contact_dissipation": float(data[7, 0] * energy),
            "normal_contact_power": float(data[7, 1] * energy / self.time_unit),
        }

    def wall_rows(self):
        """Per-wall (reaction | count, moment | power, work) rows reduced over
        the grains in the reference tree order (``diagnostic.slang:33-49``)."""
        rows = self.buffers["wallRows"].reshape(self.wall_count, self.n, 3, 4)
        return np.stack([wall_tree_reduce(rows[w]) for w in range(self.wall_count)])


def wall_tree_reduce(values):
    """``reduceWallRows``: 256-wide tree sums with the contact count in row 0's
    w carried as an integer."""
    values = np.array(values, np.float32)
    while len(values) > 1:
        n = len(values)
        groups = (n + 255) // 256
        out = np.zeros((groups, 3, 4), np.float32)
        for g in range(groups):
            block = np.zeros((256, 3, 4), np.float32)
            block[: min(256, n - 256 * g)] = values[256 * g : 256 * g + 256]
            counts = block[:, 0, 3].copy().view(np.uint32)
            block[:, 0, 3] = 0
            step = 128
            while step:
                block[:step] += block[step : 2 * step]
                counts[:step] += counts[step : 2 * step]
                step //= 2
            block[0, 0, 3] = counts[:1].view(np.float32)[0]
            out[g] = block[0]
        values = out
    return values[0]


def tree_reduce(values, max_field=None):
    """256-wide binary tree sums repeated to one row (``diagnostic.slang:3-28``).

    ``max_field=(row, component)`` reduces that field with max instead of sum.
    """
    values = np.asarray(values, np.float32)
    while len(values) > 1:
        n = len(values)
        groups = (n + 255) // 256
        out = np.zeros((groups,) + values.shape[1:], np.float32)
        for g in range(groups):
            block = np.zeros((256,) + values.shape[1:], np.float32)
            block[: min(256, n - 256 * g)] = values[256 * g : 256 * g + 256]
            step = 128
            while step:
                if max_field is not None:
                    r, k = max_field
                    m = np.maximum(block[:step, r, k], block[step : 2 * step, r, k])
                block[:step] += block[step : 2 * step]
                if max_field is not None:
                    block[:step, r, k] = m
                step //= 2
            out[g] = block[0]
        values = out
    return values[0]
