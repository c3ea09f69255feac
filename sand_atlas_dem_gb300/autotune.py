"""Launch-shape autotuner for the persistent phases (no reference counterpart).

The persistent phases spread work items over a grid of CTAs: the node
filter (one warp per (directed pair, leaf) item), the exact query (one
thread per surviving node), the pair set-up and leaf
cull (one warp per directed pair), the contact emit and contact law, and the
gather (one warp per grain).  How many CTAs per SM, and how many warps per
node-query CTA (which sets its shared-memory tile when the learned culler is
on), decide occupancy against latency; the best choice depends on the
workload (grains, contacts per grain, triangle counts) and on whether the
culler runs.  None of these choices changes which work is done or the order
in which any sum is accumulated, so every choice gives bit-identical results.

:func:`tune` times each phase with CUDA events (``Engine.profile_phases``)
for each candidate of its parameter in turn (coordinate descent, phases are
independent), keeps the fastest, and rolls the engine back (its transactional backup)
so that the trial steps leave no trace.  Results can be kept in a JSON cache keyed by the
device and the workload signature.
"""

import json
import statistics
from pathlib import Path

from .engine import TUNING_KEYS

SPACE = {
    "query_warps": (8, 4),
    "query_blocks_per_sm": (2, 4, 8, 16),
    "cull_blocks_per_sm": (2, 4, 8, 16),
    "contact_blocks_per_sm": (2, 4, 8, 16),
    "gather_warps_per_sm": (16, 32, 64),
    "walk_blocks_per_sm": (2, 4, 8, 16),
}
PHASES = {
    "query_warps": ("node_filter",),
    "query_blocks_per_sm": ("node_filter",),
    "cull_blocks_per_sm": ("pair_cull",),
    "contact_blocks_per_sm": ("node_filter", "contact_emit", "friction_and_history"),
    "gather_warps_per_sm": ("force_reduction",),
    "walk_blocks_per_sm": ("node_query",),
}
assert set(SPACE) == set(TUNING_KEYS) == set(PHASES)


def signature(engine):
    """Workload key: device, grains, shapes, triangles and nodes, culler."""
    import torch

    shapes = engine.library.shapes
    return json.dumps(dict(
        device=torch.cuda.get_device_name(engine.device),
        grains=int(engine.n),
        specimens=int(engine.specimens),
        triangles=int(sum(len(s.faces) for s in shapes)),
        nodes=int(sum(len(s.samples) for s in shapes)),
        shapes=len(shapes),
        culler=engine.culler is not None,
    ), sort_keys=True)


def _load(cache):
    if cache and Path(cache).expanduser().exists():
        return json.loads(Path(cache).expanduser().read_text())
    return {}


def tune(engine, *, repeats=3, cache=None, log=None):
    """Pick the launch shapes for ``engine`` and install them in ``engine.tuning``.

    Returns ``(choice, table)``: the chosen values and, per parameter, the
    median milliseconds of its phases for each candidate.
    """
    key = signature(engine)
    known = _load(cache)
    if key in known:
        engine.tuning = dict(known[key]["choice"])
        return engine.tuning, known[key]["table"]
    # The engine's own rollback copy (the one a rejected chunk restores) puts
    # every buffer back byte for byte after the trial steps.
    engine._backup()
    active, history, step = engine.active, engine.history, engine.step
    choice = {k: 0 for k in TUNING_KEYS}
    table = {}
    engine.profile_phases()  # warm-up: graphs, caches, first-touch
    for name, candidates in SPACE.items():
        times = {}
        for value in candidates:
            engine.tuning = dict(choice, **{name: value})
            samples = []
            for _ in range(repeats):
                ms = engine.profile_phases()
                samples.append(sum(ms[p] for p in PHASES[name]))
            times[value] = statistics.median(samples)
        best = min(times, key=times.get)
        choice[name] = best
        table[name] = {str(v): round(t, 5) for v, t in times.items()}
        if log:
            log(dict(parameter=name, chosen=best, ms=table[name]))
    engine.active, engine.history = active, history
    engine._backup(restore=True)
    engine.synchronize()
    engine.step = step
    engine.tuning = dict(choice)
    if cache:
        known[key] = dict(choice=choice, table=table)
        path = Path(cache).expanduser()
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(known, indent=1, sort_keys=True))
    return engine.tuning, table


def default_choice():
    """The built-in shapes (what 0 selects in the launchers)."""
    return dict(query_warps=8, query_blocks_per_sm=8, cull_blocks_per_sm=8, contact_blocks_per_sm=8,
                gather_warps_per_sm=64, walk_blocks_per_sm=8)


__all__ = ["SPACE", "PHASES", "signature", "tune", "default_choice"]
