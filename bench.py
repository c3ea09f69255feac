"""Benchmark: grain-steps/s of the mesh-surface DEM step on one GB300.

Workloads (``--workload``):

``dense-10k`` (default, the headline): the 10,000-grain plain-method
    configuration.  64 seeded perturbed geodesic icospheres (1,280 triangles,
    642 Sobol nodes each), grain scales lognormal (median 1, sigma_ln 0.2) on
    a 0.5 mm nominal radius, a dense periodic packing prepared by affine
    compression and frictionless force descent on the GPU toward solid
    fraction 0.58 (the rough grains jam near 0.54 at overlaps under 9% of a
    diameter; the record states what was reached,
    sand_atlas_dem_gb300/data/packing-f8-10000.npz), then isotropic
    compression at 0.5/s with rho 2650, kn 1e12, kt 5e11, mu 0.5, normal
    viscosity for damping ratio 0.3 and dt one ulp below the reference's
    conservative bound.
``uneven-50k``: 50,000 grains from the uneven library (64 shapes, triangle
    counts log-uniform 320..5,120, axis ratios U(0.6, 1)): a dense periodic
    packing of 6,250 grains prepared like dense-10k's (affine compression and
    frictionless force descent toward solid fraction 0.58; the record states
    what was reached, sand_atlas_dem_gb300/data/packing-uneven-6250.npz),
    repeated 2 x 2 x 2, compressed at 0.5/s.
``lattice-50k``: 50,653 grains of the uneven library on a jittered cubic
    lattice at solid fraction 0.58 (about 127 contacts per grain: an
    overlapped stress case), compressed at 0.5/s.
``specimens-128``: 128 independent periodic specimens batched in one engine
    (one launch per phase, one graph per step), 512..4,096 grains each from
    the uneven library at solid fractions U(0.55, 0.60), each compressed at
    its own rate U(0.1, 1.0)/s.
``walled-10k``: 10,648 grains of the f8 library on a jittered cubic lattice
    (solid fraction 0.58) in a nonperiodic domain, boxed by six penalty planes
    that press the outer grains and move inward (the reference's wall stage).
``sdf-spheres-1k``: the SDF contact geometry on the reference's own benchmark
    case (``benchmark.py:162-253`` defaults): 1,000 analytical spheres
    (resolution 32, 512 nodes) on a simple cubic lattice at 1.99 radii,
    dt 1e-8.

Data are synthetic (seeded); the reference's Hostun assets are not used.

``value``  : device throughput, CUDA events on the engine stream around each
             graph-replayed step, L2 flushed (256 MiB write) before each step.
``amortized``: the workload's whole run after the headline steps (10,000
             steps for dense-10k, the plain-method configuration's length;
             2,000 otherwise), every step timed the same way, with the filter
             builds and neighbour rebuilds its motion caused, the step-time
             median, 99th percentile and maximum, and its kernel launches.
``gpu_launches``: kernel launches of the timed steps: each captured step runs
             its unconditional kernels; the neighbour-build and filter-build
             bodies are conditional graph nodes that run only on the steps
             whose device flag asks for them (counted from the device's
             rebuild and build counters).
``e2e``    : the public API a caller uses (``Engine.advance`` chunks of 10
             steps plus ``diagnostics()``), host wall clock, including the
             host<->device traffic of those calls (counted by the engine).
``--impl reference`` times the CPU oracle port of the reference CPU backend
on the host cores (``oracle/``), same workload and metric.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "grain-steps/s"
COMMON = dict(shapes=64, friction=0.5, damping_ratio=0.3,
              dtype_note="FP32 state with compensated residuals; FP64 minimum image")
WORKLOADS = {
    "sparse-1k": dict(COMMON, workload="sparse-periodic-1k-icosphere-f4", library="f4", grains=1000,
                      triangles_per_grain=320, nodes_per_grain=162, solid_fraction_target=0.35,
                      initial_velocity_sigma_m_s=0.05, max_overlap_fraction=0.1, strain_rate_per_s=0.0,
                      run_steps=2000),
    "dense-10k": dict(COMMON, workload="dense-periodic-10k-icosphere-f8", library="f8", grains=10_000,
                      triangles_per_grain=1280, nodes_per_grain=642, solid_fraction_target=0.58,
                      max_overlap_fraction=0.1, strain_rate_per_s=-0.5),
    "uneven-50k": dict(COMMON, workload="dense-periodic-50k-uneven", library="uneven", grains=50_000,
                       triangles_per_grain="320..5120", solid_fraction_target=0.58, max_overlap_fraction=0.1,
                       strain_rate_per_s=-0.5,
                       packing="force-descent packing of 6,250 grains (packing-uneven-6250.npz) tiled 2x2x2"),
    "lattice-50k": dict(COMMON, workload="lattice-periodic-50k-uneven", library="uneven", grains=37**3,
                        triangles_per_grain="320..5120", solid_fraction=0.58, max_overlap_fraction=0.5,
                        strain_rate_per_s=-0.5, packing="jittered cubic lattice (overlapped stress case)"),
    "specimens-128": dict(COMMON, workload="128-specimens-uneven", library="uneven", specimens=128,
                          grains_per_specimen="512..4096", solid_fraction="U(0.55, 0.60)",
                          strain_rate_per_s="-U(0.1, 1.0) per specimen", max_overlap_fraction=0.5,
                          packing="jittered cubic lattice per specimen"),
    "walled-10k": dict(COMMON, workload="walled-lattice-10k-f8", library="f8", grains=22**3,
                       triangles_per_grain=1280, nodes_per_grain=642, solid_fraction=0.58, max_overlap_fraction=0.5,
                       strain_rate_per_s=0.0, walls="6 box planes 0.02 diameters into the outer grains, "
                       "moving inward at 0.5/s of the box half-width, friction 0.3",
                       packing="jittered cubic lattice, nonperiodic"),
    "sdf-spheres-1k": dict(workload="sdf-spheres-1k-simple-cubic", library="sphere", grains=1000, shapes=1,
                           contact_geometry="sdf", sdf_resolution=32, nodes_per_grain=512,
                           packing="simple cubic at 1.99 radii", timestep_s=1e-8, max_overlap_fraction=0.01,
                           pairs_per_particle=8, contacts_per_particle=256, strain_rate_per_s=0.0),
}
DATA = ROOT / "sand_atlas_dem_gb300" / "data"
# DRAM bytes (read + write) of one reuse step's exact queries
# (k_nodeWalkKnown and k_nodeWalkStaged; k_nodeWalkSlow returns at once on a
# short list) from an ncu capture of the same workload
# (profiles/walk-dense-10k.md); None where not captured.
WALK_TRAFFIC = {"dense-10k": 40.03e6 + 0.48e6 + 9.26e6}
# work[] counters (csrc/dem_device.cuh): the stored node-filter results and
# the neighbour-list rebuilds.
W_FILTER_MARGIN, W_FILTER_BUILDS, W_FILTER_STEPS, W_CERTIFIED, W_REBUILDS, W_DORMANT = 8, 9, 10, 15, 17, 18
# Steps of the long window timed after the headline steps: the length of the
# workload's own run, so that the filter builds and neighbour rebuilds its
# motion causes are inside it.
WINDOW_STEPS = {"dense-10k": 10_000, "sparse-1k": 2_000, "uneven-50k": 2_000, "lattice-50k": 2_000,
                "specimens-128": 2_000,
                "walled-10k": 2_000, "sdf-spheres-1k": 2_000}


def log(*args):
    print(*args, file=sys.stderr, flush=True)


def cache_dir():
    path = Path(os.environ.get("SAND_DEM_GB300_CACHE", "/tmp/sand-dem-gb300-cache"))
    path.mkdir(parents=True, exist_ok=True)
    return path


def library(kind):
    from sand_atlas_dem_gb300.shapes import ShapeLibrary, analytic_sphere, synthetic_library

    if kind == "sphere":
        return ShapeLibrary([analytic_sphere(resolution=32, samples=512)])
    return synthetic_library(kind, 64)


def packing(lib, grains, phi, seed=42, kind="f8", name=None):
    """The prepared packing (committed record, else prepared here within a
    bounded time and cached)."""
    from sand_atlas_dem_gb300.workloads import descent_packing, load_packing, save_packing

    name = name or f"packing-{kind}-{grains}.npz"
    for path in (DATA / name, cache_dir() / name):
        if path.exists():
            return dict(load_packing(path), path=str(path))
    t = time.perf_counter()
    out = descent_packing(lib, grains, phi, seed=seed, max_seconds=600, log=lambda d: log("prepare", d))
    meta = dict(library=kind, grains=grains, solid_fraction=phi, seed=seed, evaluations=out["evaluations"],
                seconds=round(time.perf_counter() - t, 1), achieved_solid_fraction=out["phi"],
                max_overlap_fraction=out["overlap"], method="affine compression with frictionless force descent")
    save_packing(cache_dir() / name, out["engine"], out["ids"], out["scales"], meta)
    return dict(load_packing(cache_dir() / name), path=str(cache_dir() / name))


class Workload:
    """One benchmark workload: its library, how to build an initialized
    engine of a given class on it, and each specimen's compression rate."""

    def __init__(self, name, grains=None):
        from sand_atlas_dem_gb300.workloads import lattice_at, material_spec, specimen_set

        self.name = name
        self.config = dict(WORKLOADS[name])
        self.lib = library(self.config["library"])
        self.velocities = None
        if name == "sparse-1k":
            # The plain-method CPU configuration: a loose packing at solid
            # fraction 0.35 with random orientations and velocities N(0, 0.05 m/s).
            pack = packing(self.lib, self.config["grains"], self.config["solid_fraction_target"], kind="f4",
                           name="packing-f4-1000-phi035.npz")
            self.specimens = [(pack["positions"], pack["cell"], pack["ids"], pack["scales"])]
            self.rotations = pack["rotations"]
            rng = np.random.default_rng(42 + 2)
            self.velocities = rng.normal(0.0, self.config["initial_velocity_sigma_m_s"], (len(pack["ids"]), 3))
            self.rates = np.zeros((1, 3))
            self.config.update(packing_meta=pack["meta"],
                               solid_fraction=pack["meta"].get("achieved_solid_fraction"))
        elif name == "dense-10k":
            grains = grains or self.config["grains"]
            pack = packing(self.lib, grains, self.config["solid_fraction_target"])
            self.specimens = [(pack["positions"], pack["cell"], pack["ids"], pack["scales"])]
            self.rotations = pack["rotations"]
            self.rates = np.full((1, 3), self.config["strain_rate_per_s"])
            self.config.update(grains=grains, packing_meta=pack["meta"],
                               solid_fraction=pack["meta"].get("achieved_solid_fraction"))
        elif name == "sdf-spheres-1k":
            # The reference's own benchmark case (benchmark.py:162-253 defaults):
            # 1,000 analytical spheres on a simple cubic lattice at 1.99 radii.
            radius = self.lib.shapes[0].radius
            side = round(self.config["grains"] ** (1 / 3))
            spacing = 1.99 * radius
            idx = np.stack(np.meshgrid(*([np.arange(side)] * 3), indexing="ij"), -1).reshape(-1, 3)
            n = len(idx)
            self.specimens = [((idx + 0.5) * spacing, np.full(3, side * spacing), np.zeros(n, np.uint32),
                               np.ones(n))]
            self.rotations = np.tile(np.array([0, 0, 0, 1], np.float32), (n, 1))
            self.rates = np.zeros((1, 3))
        elif name == "walled-10k":
            from sand_atlas_dem_gb300.workloads import walled_lattice

            case = walled_lattice(self.lib, round(self.config["grains"] ** (1 / 3)), self.config["solid_fraction"])
            self.specimens = [(case["positions"], case["cell"], case["ids"], case["scales"])]
            self.rotations = case["rotations"]
            self.rates = np.zeros((1, 3))
            self.planes = case["planes"]
        elif name == "uneven-50k":
            # 50,000 grains: the committed 6,250-grain dense packing of the
            # uneven library, repeated 2 x 2 x 2 (a periodic packing of the
            # same solid fraction and contacts per grain).
            from sand_atlas_dem_gb300.workloads import load_packing, tile_packing

            pack = tile_packing(load_packing(DATA / "packing-uneven-6250.npz"))
            self.specimens = [(pack["positions"], pack["cell"], pack["ids"], pack["scales"])]
            self.rotations = pack["rotations"]
            self.rates = np.full((1, 3), self.config["strain_rate_per_s"])
            self.config.update(packing_meta=pack["meta"],
                               solid_fraction=pack["meta"].get("achieved_solid_fraction"))
        elif name == "lattice-50k":
            case = lattice_at(self.lib, round(self.config["grains"] ** (1 / 3)), self.config["solid_fraction"],
                              seed=5)
            self.specimens = [(case["positions"], case["cell"], case["ids"], case["scales"])]
            self.rotations = case["rotations"]
            self.rates = np.full((1, 3), self.config["strain_rate_per_s"])
        else:
            self.specimens, self.rotations, rates = specimen_set(self.lib, self.config["specimens"])
            self.rates = -np.repeat(rates[:, None], 3, axis=1)
            self.config.update(grains=int(sum(len(s[0]) for s in self.specimens)),
                               specimen_grains=[len(s[0]) for s in self.specimens])
        ids = np.concatenate([s[2] for s in self.specimens])
        scales = np.concatenate([s[3] for s in self.specimens])
        # Lattices have at most 26 neighbours in range: 16 pairs per grain
        # leave room, and the engine grows on overflow.
        pairs = {} if name in ("dense-10k", "sparse-1k", "uneven-50k") else dict(pairs_per_particle=16)
        if name == "sdf-spheres-1k":
            from sand_atlas_dem_gb300.spec import Experiment

            self.spec = Experiment(particles=len(ids), contact_geometry="sdf", timestep=self.config["timestep_s"],
                                   pairs_per_particle=self.config["pairs_per_particle"],
                                   contacts_per_particle=self.config["contacts_per_particle"],
                                   max_overlap_fraction=self.config["max_overlap_fraction"])
        elif name == "walled-10k":
            self.spec = material_spec(self.lib, ids, scales, max_overlap_fraction=self.config["max_overlap_fraction"],
                                      periodic=False, planes=self.planes, boundary_box=list(range(6)), **pairs)
        else:
            self.spec = material_spec(self.lib, ids, scales,
                                      max_overlap_fraction=self.config["max_overlap_fraction"], **pairs)
        self.grains = len(ids)

    def engine(self, cls, specimens=None, **kwargs):
        """An initialized engine from rest on all (or the listed) specimens."""
        chosen = list(range(len(self.specimens))) if specimens is None else list(specimens)
        offsets = np.cumsum([0] + [len(s[0]) for s in self.specimens])
        if len(chosen) == 1:
            s = self.specimens[chosen[0]]
            e = cls(self.lib, self.spec_for(chosen), s[0], s[1], s[2], s[3], **kwargs)
        else:
            e = cls.batch(self.lib, self.spec_for(chosen), [self.specimens[k] for k in chosen], **kwargs)
        rotations = np.concatenate([self.rotations[offsets[k]:offsets[k + 1]] for k in chosen])
        rotations = np.ascontiguousarray(rotations, np.float32)
        uploads = {"rotation": rotations}
        if self.velocities is not None:
            v = np.zeros((e.n, 4), np.float32)
            v[:, :3] = np.concatenate([self.velocities[offsets[k]:offsets[k + 1]] for k in chosen]) \
                * e.time_unit / e.length_unit
            uploads["velocity"] = v
        for name, array in uploads.items():
            buffer = e.buffers[name]
            if isinstance(buffer, np.ndarray):
                buffer[...] = array
            else:
                buffer.copy_from_numpy(array)
        e.initialize()
        return e

    def spec_for(self, chosen):
        from dataclasses import replace

        return replace(self.spec, particles=int(sum(len(self.specimens[k][0]) for k in chosen)))

    def rate(self, chosen=None):
        rows = self.rates if chosen is None else self.rates[list(chosen)]
        return tuple(rows[0]) if len(rows) == 1 else rows


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                 f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[3:7]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(n, pairs, contacts, items, nodes, survivors, kept, rebuild, library_bytes, dormant=0):
    """Per-step algorithmic HBM bytes of the whole step and of the node query.

    Step: 516 B/grain + 264 B/pair + 272 B/contact + 88 B/grain on rebuild
    steps + the packed library once.  Node query (filter, survivor list,
    prefilter and exact walks, one launch group): each (directed pair, leaf)
    item reads its record, pair, source plane and leaf range and writes its
    survivor and hit masks and counts (88 B); each node considered reads its
    sample index and sample (20 B); each survivor of the one-dot test is
    listed and read back, and its keep flag written and scanned (24 B); each
    exact query reads its list entry, item record, pair, branch, sample and
    both grains' rotation and body, and a hit writes its record (132 B); a
    dormant slot of a stored list (its node proven out of reach until the
    next build) reads its 8-byte certificate word and is not queried; the
    packed library is read once (it stays in L2).
    """
    step = 516 * n + 264 * pairs + 272 * contacts + 88 * n * rebuild + library_bytes
    query = 88 * items + 20 * nodes + 24 * survivors + 132 * kept + library_bytes
    walk = 132 * (kept - dormant) + 8 * dormant + library_bytes
    return step, query, walk


def launches(e, steps, rebuilds, builds):
    """Kernel launches of ``steps`` graph-replayed steps: the ones every step
    runs, plus the neighbour-build body on rebuild steps and the filter-build
    body on filter-build steps."""
    lib, h = e.lib, e._native
    return (lib.sdg_engine_kernels_per_step(h) * steps + lib.sdg_engine_branch_kernels(h, 0) * rebuilds
            + lib.sdg_engine_branch_kernels(h, 1) * builds)


def counters(e):
    work = e.read("work", np.uint32, (64,))
    return int(work[W_REBUILDS]), int(work[W_FILTER_BUILDS]), int(work[W_CERTIFIED]), int(work[W_DORMANT])


def long_window(e, w, steps, flush):
    """The workload's whole run (``steps`` steps), each step timed on the
    device with L2 flushed before it: the amortized throughput over every
    filter build and neighbour rebuild the run's motion causes."""
    before = counters(e)
    ms = np.asarray(timed_steps(e, steps, flush))
    after = counters(e)
    rebuilds, builds = after[0] - before[0], after[1] - before[1]
    return {"steps": steps, "value": w.grains * steps / (ms.sum() / 1e3), "unit": "grain-steps/s",
            "ms_per_step": float(ms.mean()), "ms_median": float(np.median(ms)),
            "ms_p99": float(np.percentile(ms, 99)), "ms_max": float(ms.max()),
            "neighbour_rebuilds": rebuilds, "filter_builds": builds,
            "certified_queries_per_step": (after[2] - before[2]) / steps,
            "dormant_slots_at_end": after[3],
            "gpu_launches": launches(e, steps, rebuilds, builds),
            "l2": "flushed before each step (256 MiB write)"}


def timed_steps(e, steps, flush):
    """Device milliseconds of each of ``steps`` graph-replayed steps, L2 flushed before each."""
    import torch

    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    e.synchronize()
    for k in range(steps):
        with torch.cuda.stream(e.stream):
            flush.fill_(k & 0xFF)
            events[k][0].record(e.stream)
        e.run_steps(1)
        with torch.cuda.stream(e.stream):
            events[k][1].record(e.stream)
    e.synchronize()
    return [a.elapsed_time(b) for a, b in events]


def set_rates(e, w):
    """Write each specimen's strain-rate row into the cell (graph replay reads it)."""
    rows = 3 * e.specimens
    cell = e.read("cell", np.float32, (rows, 4))
    cell[1::3, :3] = np.asarray(w.rates) * e.time_unit
    e.buffers["cell"].copy_from_numpy(cell)


def run_gb300(args, cpu=True):
    import torch

    from sand_atlas_dem_gb300.engine import Engine

    w = Workload(args.workload, args.grains)
    e = w.engine(Engine, use_graph=not args.no_graph)
    rate = w.rate()
    # Warm-up (graph capture happens in the first call).
    e.advance(max(3, args.warmup), rate=rate)
    set_rates(e, w)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=e.device)
    ctrl0 = e.check_errors()
    work0 = e.read("work", np.uint32, (64,))
    window_steps = args.window if args.window is not None else WINDOW_STEPS[w.name]
    with ClockSampler() as clocks:
        step_ms = timed_steps(e, args.steps, flush)
        work1 = e.read("work", np.uint32, (64,))
        window = long_window(e, w, window_steps, flush) if window_steps else None
    ctrl = e.check_errors()
    timed_rebuilds = int(work1[W_REBUILDS] - work0[W_REBUILDS])
    timed_builds = int(work1[W_FILTER_BUILDS] - work0[W_FILTER_BUILDS])
    filter_cache = {"margin": e.filter_margin,
                    "adapted_margin": float(work1[W_FILTER_MARGIN:W_FILTER_MARGIN + 1].view(np.float32)[0]),
                    "builds_in_timed_steps": timed_builds,
                    "neighbour_rebuilds_in_timed_steps": timed_rebuilds,
                    "timed_steps": int(work1[W_FILTER_STEPS] - work0[W_FILTER_STEPS]),
                    "certified_queries_per_step": float(work1[W_CERTIFIED] - work0[W_CERTIFIED]) / args.steps,
                    "dormant_slots": int(work1[W_DORMANT])}
    device_s = sum(step_ms) / 1e3
    value = w.grains * args.steps / device_s
    kernel_count = launches(e, args.steps, timed_rebuilds, timed_builds)
    # Phase profile (cold L2 each), for the roofline of the dominant launch group.
    phases = []
    for _ in range(3):
        with torch.cuda.stream(e.stream):
            flush.fill_(1)
        phases.append(e.profile_phases())
    e.check_errors()
    phase_ms = {k: float(np.median([p[k] for p in phases])) for k in phases[0]}
    work = e.read("work", np.uint32, (64,))
    items, survivors, kept = int(work[0]), int(work[2]), int(work[3])
    pairs, contacts = int(ctrl[1]), int(ctrl[2])
    leaf_nodes = e.layout.geometry["meshClusterRanges"][:, 1]
    cand = e.read("candidates", np.uint32, (e.candidate_capacity, 2))[:items]
    nodes = int(leaf_nodes[cand[:, 1]].sum()) if items else 0
    lib_bytes = sum(a.nbytes for k, a in e.layout.geometry.items() if k.startswith("mesh") or k == "sample")
    dormant = filter_cache["dormant_slots"]
    step_bytes, query_bytes, walk_bytes = algorithmic_bytes(w.grains, pairs, contacts, items, nodes, survivors,
                                                            kept, 0, lib_bytes, dormant)
    kernel_name = ("k_nodeWalkKnown + k_nodeWalkStaged/k_nodeWalkSlow (exact queries: certified triangles, "
                   "then full BVH walks)"
                   if e.filter_margin > 0 and e.culler is None else "k_nodeWalk (exact BVH queries, one thread per kept node)")
    group_name = "k_nodeFilter, k_survivorList, k_survivorPrefilter, k_walkList, k_nodeWalk + scans"
    if e.sdf:
        # SDF emit (k_sdfEmit, one warp per pair), counted at its minimum:
        # every node of both grains read once (its sample, 16 B), the 8 grid
        # values of each contact node's cell (32 B) and 52 B written per
        # contact; the count pass reads the samples once more.
        node_count = pairs * 2 * w.config["nodes_per_grain"]
        walk_bytes = 16 * node_count + (32 + 52) * contacts + sum(e.layout.geometry[k].nbytes for k in ("distance", "sample"))
        query_bytes = walk_bytes + 16 * node_count + 32 * contacts
        step_bytes = 516 * w.grains + 264 * pairs + 272 * contacts + query_bytes
        kernel_name = "k_sdfEmit (SDF node queries and contact writes, one warp per pair)"
        group_name = "k_sdfCount, contact scan, k_sdfEmit"
    hbm, peak_kind = peaks()
    top = max(phase_ms, key=phase_ms.get)
    query_ms = phase_ms["node_filter"] + phase_ms["node_query"] + (phase_ms["pair_cull"] if e.sdf else 0.0)
    query_gbs = query_bytes / (query_ms / 1e3) / 1e9
    # The dominant kernel, k_nodeWalk, is the whole "node_query" phase (one launch).
    walk_gbs = walk_bytes / (phase_ms["node_query"] / 1e3) / 1e9
    # End to end through the public API: advance() chunks plus diagnostics().
    chunk = 10
    chunks = max(1, args.steps // chunk)
    e2e_s = 0.0
    h2d0, d2h0 = e.h2d_bytes, e.d2h_bytes
    for _ in range(chunks):
        with torch.cuda.stream(e.stream):
            flush.fill_(2)
        e.synchronize()
        t = time.perf_counter()
        e.advance(chunk, rate=rate)
        e.diagnostics()
        e2e_s += time.perf_counter() - t
    e2e = w.grains * chunk * chunks / e2e_s
    h2d = (e.h2d_bytes - h2d0) / (chunk * chunks)
    d2h = (e.d2h_bytes - d2h0) / (chunk * chunks)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "grain-steps/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * device_s / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": dict(w.config, l2="flushed before each timed step (256 MiB write)",
                       pairs=pairs, contacts=contacts, node_query_items=items, node_queries=nodes,
                       plane_survivors=survivors, exact_queries=kept, timestep_s=e.spec.timestep,
                       phase_ms=phase_ms, filter_cache=filter_cache,
                       dominant_phase=top, tuning=dict(e.tuning)),
        "e2e": {"value": e2e, "unit": "grain-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "api": f"Engine.advance({chunk}) + Engine.diagnostics() per chunk"},
        "gpu_launches": int(kernel_count),
        "kernels_per_step": {"every_step": int(e.lib.sdg_engine_kernels_per_step(e._native)),
                             "neighbour_build_body": int(e.lib.sdg_engine_branch_kernels(e._native, 0)),
                             "filter_build_body": int(e.lib.sdg_engine_branch_kernels(e._native, 1))},
        "amortized": window,
        "roofline": {
            "bound": "hbm",
            "kernel": kernel_name,
            "achieved": walk_gbs,
            "peak": hbm,
            "peak_source": peak_kind,
            "unit": "GB/s",
            "frac": walk_gbs / hbm,
            "traffic": WALK_TRAFFIC.get(w.name),
            "algorithmic_bytes": walk_bytes,
            "kernel_ms": phase_ms["node_query"],
            "launch_group": group_name,
            "launch_group_algorithmic_bytes": query_bytes,
            "launch_group_ms": query_ms,
            "launch_group_achieved_gbs": query_gbs,
            "step_algorithmic_bytes": step_bytes,
            "step_achieved_gbs": step_bytes / (device_s / args.steps) / 1e9,
        },
        "clocks": clocks.summary(),
    }
    if not args.no_plain and not e.sdf:  # the SDF geometry has no filters to compare
        line["plain_gpu_path"] = plain_comparison(w, args, flush)
    if not args.no_culler and not e.sdf:
        line["learned_culler"] = culler_comparison(w, args, flush)
    if "run_steps" in w.config and cpu and not args.no_cpu_baseline:
        line["full_run"] = full_run(w, args)
    if cpu and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args)
    if ctrl0[0] or ctrl[0]:
        line["solver_flags"] = int(ctrl[0])
    return line


def full_run(w, args):
    """The whole run of the configuration (``run_steps`` steps) from the
    prepared start: on the GPU through the public API (one
    ``Engine.advance`` call and ``diagnostics()``, host wall clock, host
    copies included) and on the CPU oracle with every host thread; and how far
    apart the two end states are."""
    from oracle.engine import OracleEngine
    from sand_atlas_dem_gb300.engine import Engine

    steps = w.config["run_steps"]
    g = w.engine(Engine)
    g.synchronize()
    t = time.perf_counter()
    g.advance(steps, rate=w.rate())
    g.diagnostics()
    gpu_s = time.perf_counter() - t
    o = w.engine(OracleEngine, threads=args.cpu_threads)
    t = time.perf_counter()
    o.advance(steps, rate=w.rate())
    cpu_s = time.perf_counter() - t
    sg, so = g.state(), o.state()
    box = so["cell"][0, :3].astype(float)
    d = (sg["position"][:, :3].astype(float) + sg["positionRemainder"][:, :3]) \
        - (so["position"][:, :3].astype(float) + so["positionRemainder"][:, :3])
    d -= np.round(d / box) * box
    diameters = g.layout.body[:, 3].astype(float)
    qg, qo = sg["rotation"].astype(float), so["rotation"].astype(float)
    sign = np.where(np.einsum("ij,ij->i", qg, qo) < 0, -1.0, 1.0)
    return {"steps": steps, "grain_steps": w.grains * steps,
            "gpu_e2e_s": gpu_s, "gpu_e2e_value": w.grains * steps / gpu_s,
            "cpu_oracle_s": cpu_s, "cpu_oracle_value": w.grains * steps / cpu_s, "cpu_threads": o.threads,
            "gpu_over_cpu": cpu_s / gpu_s,
            "same_contact_keys_at_end": bool(sg["contacts"] == so["contacts"]
                                             and np.array_equal(sg["meta"], so["meta"])),
            "contacts_at_end": int(sg["contacts"]),
            "max_centre_deviation_diameters": float((np.linalg.norm(d, axis=1) / diameters).max()),
            "max_quaternion_component_deviation": float(np.abs(sign[:, None] * qg - qo).max())}


def plain_comparison(w, args, flush):
    """The plain GPU path against each acceleration, from one start state.

    ``plain`` runs the reference's own conservative filters every step (no
    distance-bound grid, no stored filter results); ``grid`` adds the
    certified distance-bound grid; ``stored_filters`` adds only the stored
    node-filter results; ``accelerated`` is the headline configuration (both).
    Every engine runs the same warm-up and timed steps (L2 flushed before
    each); contacts and forces must be bit-identical to ``plain``.
    """
    import torch

    from sand_atlas_dem_gb300.engine import Engine

    rate = w.rate()
    configs = {"plain": dict(distance_grid=False, filter_margin=0.0),
               "grid": dict(distance_grid=True, filter_margin=0.0),
               "stored_filters": dict(distance_grid=False),
               "accelerated": dict()}
    steps = min(args.steps, 50)
    out, states = {}, {}
    for name, settings in configs.items():
        e = w.engine(Engine, **settings)
        e.advance(max(3, args.warmup), rate=rate)
        set_rates(e, w)
        ms = timed_steps(e, steps, flush)
        phases = e.profile_phases()
        states[name] = e.state()
        out[name] = dict(value=w.grains * steps / (sum(ms) / 1e3), ms_per_step=sum(ms) / steps,
                         collector_ms=phases["pair_cull"] + phases["node_filter"] + phases["node_query"],
                         filter_margin=e.filter_margin, distance_grid=e.distance_grid)
        del e
        torch.cuda.empty_cache()
    base = states["plain"]
    for name in configs:
        out[name]["bitwise_equal_to_plain"] = all(
            v.tobytes() == states[name][k].tobytes() for k, v in base.items() if isinstance(v, np.ndarray))
    result = dict(steps=steps, **out)
    result["speedup_over_plain"] = {k: out[k]["value"] / out["plain"]["value"] for k in configs if k != "plain"}
    return result


def culler_comparison(w, args, flush):
    """Exact step against the learned-cull step from one start state: on the
    accelerated path (distance-bound grid and stored filter results; with the
    culler the exact-query list is rebuilt every step, since the network's
    calibrated decisions are taken per step) and on the plain path (the
    reference's filters alone).

    The culler is trained (2^20 shell points and 2^18 interior points per
    shape, 2,000 Adam steps) and calibrated on the GPU and attached to the
    culled engines; every engine runs the same timed steps.  Missed contacts
    = exact contacts absent from the culled run; forces are compared bit for
    bit.
    """
    import gc

    import torch

    from sand_atlas_dem_gb300.culler import LearnedCuller
    from sand_atlas_dem_gb300.engine import Engine

    rate = w.rate()
    reference_filters = dict(distance_grid=False, filter_margin=0.0)
    configs = {"plain": {}, "culled": {}, "plain_no_grid": reference_filters, "culled_no_grid": reference_filters}
    # One engine at a time (besides the one the culler samples its shapes
    # through): a batched workload's engines take tens of GB each.
    t = time.perf_counter()
    trainer = w.engine(Engine, **reference_filters)
    c = LearnedCuller(trainer, points=1 << 20, steps=2000, batch=8192)
    c.train()
    c.calibrate()
    train_s = time.perf_counter() - t
    out = {}
    steps = min(args.steps, 50)
    for name, settings in configs.items():
        e = w.engine(Engine, **settings)
        if name.startswith("culled"):
            c.attach(e)
        e.advance(max(3, args.warmup), rate=rate)
        set_rates(e, w)
        e.buffers["cullerStats"].copy_from_numpy(np.zeros(4, np.uint32))
        ms = timed_steps(e, steps, flush)
        phases = e.profile_phases()
        stats = e.read("cullerStats", np.uint32, (4,))
        out[name] = dict(value=w.grains * steps / (sum(ms) / 1e3), ms_per_step=sum(ms) / steps,
                         node_query_ms=phases["node_filter"] + phases["node_query"],
                         tested=int(stats[0]), culled=int(stats[1]), state=e.state())
        del e
        gc.collect()
        torch.cuda.empty_cache()
    result = dict(steps=steps, training_s=round(train_s, 1), margins_mean=float(np.mean(c.margins)),
                  cell_margins_mean=float(np.mean(c.cell_margins)), loss_over_weight=c.over,
                  validation_cull_rate=c.cull_rate())
    for grid in ("", "_no_grid"):
        p, q = out["plain" + grid], out["culled" + grid]
        sp, sc = p.pop("state"), q.pop("state")
        keys_p = {tuple(m) for m in sp["meta"][:, :3].tolist()}
        keys_c = {tuple(m) for m in sc["meta"][:, :3].tolist()}
        force_p = sp["force"][:, :3].astype(float)
        err = float(np.abs(sc["force"][:, :3] - force_p).max() / max(np.abs(force_p).max(), 1e-30))
        result["accelerated_path" if not grid else "reference_filters"] = dict(
            plain_value=p["value"], culled_value=q["value"], speedup=q["value"] / p["value"],
            plain_node_query_ms=p["node_query_ms"], culled_node_query_ms=q["node_query_ms"],
            tested_nodes=q["tested"], culled_nodes=q["culled"],
            cull_rate_of_exact_queries=q["culled"] / max(q["tested"], 1),
            missed_contacts=len(keys_p - keys_c), extra_contacts=len(keys_c - keys_p),
            forces_bitwise_equal=bool(sp["force"].tobytes() == sc["force"].tobytes()),
            force_max_relative_error=err)
    result["accelerated_speedup_over_reference_filters"] = out["plain"]["value"] / out["plain_no_grid"]["value"]
    result["culled_speedup_over_plain_path"] = out["culled"]["value"] / out["plain_no_grid"]["value"]
    return result


def cpu_sample(w):
    """Specimens the CPU oracle times: all of a single-specimen workload, the
    first eight specimens (one at a time: the oracle has no batching) of a
    batched one."""
    return [[0]] if len(w.specimens) == 1 else [[k] for k in range(8)]


def cpu_baseline(w, args, budget_s=15.0, max_steps=200):
    """Oracle port of the reference CPU backend on this host's cores: whole
    steps of the workload (or of its sampled specimens), repeated until about
    ``budget_s`` seconds of CPU work (at least 3 steps)."""
    from oracle.engine import OracleEngine

    grains, seconds, threads, steps = 0, 0.0, 1, 0
    engines = [(w.engine(OracleEngine, chosen, threads=args.cpu_threads), chosen) for chosen in cpu_sample(w)]
    while steps < max_steps and (steps < 3 or seconds < budget_s):
        for e, chosen in engines:
            threads = e.threads
            t = time.perf_counter()
            e.advance(1, rate=w.rate(chosen))
            seconds += time.perf_counter() - t
            grains += e.n
        steps += 1
    what = "the whole workload" if len(w.specimens) == 1 else f"specimens 0-7 ({grains // steps} grains)"
    line = {"value": grains / seconds, "unit": "grain-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full steps of {what}, {seconds:.2f} s"}
    if threads > 1:
        # The same oracle on one worker (the reference CPU backend's serial
        # collector), a shorter sample: at least one step of each specimen.
        del engines
        one = [(w.engine(OracleEngine, chosen, threads=1), chosen) for chosen in cpu_sample(w)]
        grains1, seconds1, steps1 = 0, 0.0, 0
        while steps1 < 1 or (seconds1 < budget_s / 3 and steps1 < max_steps):
            for e, chosen in one:
                t = time.perf_counter()
                e.advance(1, rate=w.rate(chosen))
                seconds1 += time.perf_counter() - t
                grains1 += e.n
            steps1 += 1
        line["single_worker"] = {"value": grains1 / seconds1, "unit": "grain-steps/s", "cores": 1,
                                 "sample": f"{steps1} full steps of {what}, {seconds1:.2f} s"}
    return line


def run_reference(args):
    from oracle.engine import OracleEngine

    w = Workload(args.workload, args.grains)
    grains, seconds, threads = 0, 0.0, 1
    for chosen in cpu_sample(w):
        e = w.engine(OracleEngine, chosen, threads=args.cpu_threads)
        threads = e.threads
        rate = w.rate(chosen)
        if args.warmup > 0:
            e.advance(1, rate=rate)
        t = time.perf_counter()
        e.advance(args.steps, rate=rate)
        seconds += time.perf_counter() - t
        grains += e.n * args.steps
    value = grains / seconds
    return {
        "metric": METRIC, "value": value, "unit": "grain-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * seconds / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(w.config), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "grain-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps after {min(args.warmup, 1)} warm-up step, "
                                   f"{len(cpu_sample(w))} specimen(s)"},
        "e2e": {"value": value, "unit": "grain-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }

# Mesh-packing workload (the reference's startup, mesh.pack_meshes): not a
# timestep workload, so it has its own line.
PACK_WORKLOAD = "pack-53"
PACK_CONFIG = dict(workload="pack-53-shapes-1M-nodes", shapes=53, distinct_grains=8, triangles_per_shape=32_000,
                   nodes_per_shape=1 << 20, leaf_nodes=64, leaf_triangles=4,
                   note="the reference profiles its startup at 53 shape roots and 2.4 million cluster-tree nodes")


def tree_bytes(counts, leaf, key_bytes):
    """Algorithmic DRAM bytes of one tree build: every level reads the key
    (and box) of each item still in a node, and the stable sort of an internal
    node reads and writes each item's index (4 + 4 bytes)."""
    from sand_atlas_dem_gb300.trees import tree_levels

    return sum(in_nodes * key_bytes + internal * 8 for in_nodes, internal, _, _ in tree_levels(counts, leaf))


def run_packing(args, reference=False):
    """Packs the 53-shape library: on the GPU (trees built by
    sdg_median_trees, host parts on a thread pool) against the reference's
    recursion on the host (packing.host_median_trees, byte-identical to
    mesh.pack_meshes), timed on a bounded sample of one shape."""
    from sand_atlas_dem_gb300.packing import pack_library
    from sand_atlas_dem_gb300.shapes import ShapeLibrary
    from sand_atlas_dem_gb300.workloads import packing_library

    t = time.perf_counter()
    lib = packing_library(shapes=args.pack_shapes)
    log("packing library generated in", round(time.perf_counter() - t, 1), "s")
    nodes = sum(len(s.samples) for s in lib.shapes)
    triangles = sum(len(s.faces) for s in lib.shapes)
    config = dict(PACK_CONFIG, shapes=len(lib.shapes), nodes=nodes, triangles=triangles)
    unit = "sample nodes/s"

    def host_sample():
        one = ShapeLibrary(lib.shapes[:1])
        t0 = time.perf_counter()
        pack_library(one, 1e-3)
        dt = time.perf_counter() - t0
        return {"value": len(one.shapes[0].samples) / dt, "unit": unit, "cores": 1, "kind": "port",
                "sample": f"one shape ({len(one.shapes[0].samples)} nodes, {len(one.shapes[0].faces)} triangles) "
                          f"packed by the reference's recursion on the host in {dt:.2f} s"}

    if reference:
        base = host_sample()
        return {"metric": "mesh packing throughput", "value": base["value"], "unit": unit, "impl": "reference",
                "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": True, "data": "synthetic",
                "dtype": "f32", "config": config, "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    import torch

    from sand_atlas_dem_gb300.trees import device_median_trees, tree_launches

    timing = {}

    def trees(items, leaf):
        t0 = {}
        out = device_median_trees(items, leaf, timing=t0)
        timing[leaf] = t0
        return out

    for _ in range(max(1, args.warmup)):
        pack_library(ShapeLibrary(lib.shapes[:2]), 1e-3, trees=trees)
    runs, device = [], []
    steps = max(1, min(args.steps, 5))
    with ClockSampler() as clocks:
        for _ in range(steps):
            t0 = time.perf_counter()
            packed = pack_library(lib, 1e-3, trees=trees)
            runs.append(time.perf_counter() - t0)
            device.append((timing[64]["device_ms"], timing[4]["device_ms"],
                           timing[64]["wall_ms"] + timing[4]["wall_ms"]))
    # The per-shape host stage alone (hull, pseudonormals, checks; thread pool).
    from concurrent.futures import ThreadPoolExecutor

    from sand_atlas_dem_gb300.packing import _prepare

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=min(len(lib.shapes), os.cpu_count() or 1)) as pool:
        list(pool.map(lambda shape: _prepare(shape, 1e-3), lib.shapes))
    prepare_s = time.perf_counter() - t0
    wall = float(np.median(runs))
    cluster_ms = float(np.median([d[0] for d in device]))
    bvh_ms = float(np.median([d[1] for d in device]))
    counts_nodes = [len(s.samples) for s in lib.shapes]
    counts_tri = [len(s.faces) for s in lib.shapes]
    alg = tree_bytes(counts_nodes, 64, 16)
    peak, peak_kind = peaks()
    achieved = alg / (cluster_ms * 1e-3) / 1e9
    line = {
        "metric": "mesh packing throughput", "value": nodes / ((cluster_ms + bvh_ms) * 1e-3), "unit": unit,
        "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup), "ms_per_step": 1e3 * wall,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config,
        "value_note": "value: nodes / device time of both tree builds (cluster tree and triangle BVH); "
                      "e2e: nodes / wall time of the whole pack_library call (host parts, copies, trees)",
        "e2e": {"value": nodes / wall, "unit": unit,
                "h2d_bytes_per_step": 16 * (nodes + 3 * triangles), "d2h_bytes_per_step": None},
        "trees_device_ms": {"cluster_tree": cluster_ms, "triangle_bvh": bvh_ms},
        "pack_wall_s": runs,
        "pack_parts_s": {"shape_preparation": prepare_s,
                         "tree_builder_calls": float(np.median([d[2] for d in device])) / 1e3,
                         "host_threads": os.cpu_count()},
        "roofline": {"bound": "hbm", "kernel": "cluster-tree build (all levels)", "achieved": achieved,
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": alg, "traffic": None},
        "layout_nodes": int(len(packed["meshClusterRanges"])), "layout_bvh_nodes": int(len(packed["meshLinks"])),
        "clocks": clocks.summary(),
        "gpu_launches": steps * (tree_launches(counts_nodes, 64) + tree_launches(counts_tri, 4)),
    }
    # Per item its row (4 B); per tree node its record and two bound rows (48 B).
    line["e2e"]["d2h_bytes_per_step"] = int(4 * nodes + 4 * triangles + 48 * (len(packed["meshClusterRanges"])
                                                                            + len(packed["meshLinks"])))
    if args.no_cpu_baseline:
        line["cpu_baseline"] = None
    else:
        line["cpu_baseline"] = host_sample()
        line["speedup_over_host"] = {"device_trees": line["value"] / line["cpu_baseline"]["value"],
                                     "e2e": line["e2e"]["value"] / line["cpu_baseline"]["value"]}
    return line



def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    p.add_argument("--workload", default="dense-10k", choices=tuple(WORKLOADS) + (PACK_WORKLOAD,))
    p.add_argument("--grains", type=int, default=None, help="dense-10k only: grains of the packing record")
    p.add_argument("--cpu-threads", type=int, default=os.cpu_count() or 1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--prepare-only", action="store_true")
    p.add_argument("--no-culler", action="store_true",
                   help="skip the learned-culler comparison (training the per-shape networks and timing the "
                        "culled steps)")
    p.add_argument("--no-graph", action="store_true",
                   help="launch each step's kernels one by one instead of replaying the captured graph "
                        "(for per-kernel profilers, which do not list the kernels of conditional graph nodes; "
                        "the neighbour-build and filter-build kernels then launch and return at once on the "
                        "steps that skip them)")
    p.add_argument("--no-plain", action="store_true", help="skip the plain-path comparison")
    p.add_argument("--pack-shapes", type=int, default=53,
                   help="pack-53 only: shapes of the packing library (53 = the reference's profiled startup)")
    p.add_argument("--window", type=int, default=None,
                   help="steps of the long amortized window (default: the workload's run length; 0 skips it)")
    args = p.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.workload == PACK_WORKLOAD:
        if rank == 0:
            print(json.dumps(run_packing(args, reference=args.impl == "reference")), flush=True)
        return
    if args.impl == "reference":
        if args.steps > 20:
            args.steps = 20  # a bounded CPU sample: each oracle step of 10k grains takes a fraction of a second
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if args.gpus > 1 or int(os.environ.get("WORLD_SIZE", "1")) > 1:
        # Independent replicas: every rank runs the same workload on its own
        # GPU; only the timings are exchanged, after the timed region.
        import torch
        import torch.distributed as dist

        from sand_atlas_dem_gb300.replicas import aggregate

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        dist.barrier()
        line = run_gb300(args, cpu=rank == 0)
        grains = line["config"]["grains"]
        job = aggregate(grains * args.steps, line["ms_per_step"] * args.steps / 1e3, device="cuda")
        if rank == 0:
            line["n_gpus"] = job["ranks"]
            line["ms_per_step"] = 1e3 * job["seconds"] / args.steps
            line["value"] = job["value"]
            line["scaling"] = "weak"
            line["config"]["parallelism"] = f"{job['ranks']} independent specimen replicas"
            print(json.dumps(line), flush=True)
        dist.destroy_process_group()
        return
    if args.prepare_only:
        w = Workload(args.workload, args.grains)
        print(json.dumps({"prepared": True, "grains": w.grains}))
        return
    print(json.dumps(run_gb300(args)), flush=True)


if __name__ == "__main__":
    main()
