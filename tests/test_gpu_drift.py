"""Drift over a 1,000-step horizon: CUDA step against the CPU oracle.

The per-step gate is 1e-5 relative (the CUDA and libm transcendentals of the
integrator may differ in the last place, and the difference is carried
forward).  Over 1,000 steps of a dense, compressing, frictional lattice the
first test records, every 100 steps, the largest centre deviation (in units of the
grain's equivalent diameter), the largest quaternion component deviation,
and whether
the contact key sets are still identical, and prints the table.  The FP64
closed-form horizon (2,000 steps of the elastic release oscillator against
the analytic solution) is ``test_known_answers.py``.  The second test states
the drift against the FP64 oracle (the oracle's kernels built in double
precision) on the plain-method configuration.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu


def centres(state):
    return state["position"][:, :3].astype(float) + state["positionRemainder"][:, :3].astype(float)


def test_thousand_step_horizon_against_oracle(gpu_library):
    library, spec, case = lattice_case(viscosity=4e5, speed=0.05)
    o = build(OracleEngine, library, spec, case, threads=8)
    g = build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    diameters = g.layout.body[:, 3].astype(float)
    rows = []
    for _ in range(10):
        o.advance(100, rate=(-0.5, -0.5, -0.5))
        g.advance(100, rate=(-0.5, -0.5, -0.5))
        so, sg = o.state(), g.state()
        # Centres in units of the median diameter: wrap differences across the seam.
        box = so["cell"][0, :3].astype(float)
        d = centres(sg) - centres(so)
        d -= np.round(d / box) * box
        shift = np.linalg.norm(d, axis=1) / diameters
        qg, qo = sg["rotation"].astype(float), so["rotation"].astype(float)
        sign = np.where(np.einsum("ij,ij->i", qg, qo) < 0, -1.0, 1.0)
        rotation = np.abs(sign[:, None] * qg - qo).max()
        same_keys = so["contacts"] == sg["contacts"] and np.array_equal(sg["meta"], so["meta"])
        rows.append(dict(step=g.step, centre_over_diameter=float(shift.max()), rotation_component=float(rotation),
                         contacts=int(sg["contacts"]), same_contact_keys=bool(same_keys)))
    print(json.dumps(rows))
    assert g.step == o.step == 1000
    assert all(r["contacts"] > 0 for r in rows)
    assert all(r["same_contact_keys"] for r in rows), [r["step"] for r in rows if not r["same_contact_keys"]]
    # Drift bound over the horizon (a statement, not the per-step gate).
    assert max(r["centre_over_diameter"] for r in rows) < 1e-4
    assert max(r["rotation_component"] for r in rows) < 1e-4


SPARSE = Path(__file__).resolve().parent.parent / "sand_atlas_dem_gb300" / "data" / "packing-f4-1000-phi035.npz"


def kinetic_energy(state, body, inv_inertia):
    """Translational and rotational kinetic energy (normalized units) of a
    state: m v^2 / 2 and L . (I^-1 L) / 2 with I^-1 taken to the world frame."""
    v = state["velocity"][:, :3].astype(float) + state["velocityRemainder"][:, :3]
    m = body[:, 1].astype(float)
    q = state["rotation"].astype(float)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    rot = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)
    L = state["momentum"][:, :3].astype(float) + state["momentumRemainder"][:, :3]
    local = np.einsum("nji,nj->ni", rot, L)
    inv = inv_inertia[:, :3].astype(float).reshape(-1, 3, 3)
    return 0.5 * float((m * (v * v).sum(1)).sum()) + 0.5 * float(np.einsum("ni,nij,nj->", local, inv, local))


def test_thousand_steps_against_the_fp64_oracle(gpu_library):
    """Drift of the FP32 GPU step against the FP64 oracle (the same kernels
    in double precision) over 1,000 steps of the plain-method configuration:
    1,000 grains of the 320-triangle library at solid fraction 0.35, random
    orientations, velocities N(0, 0.05 m/s), damping ratio 0.3, mu 0.5.  The
    FP32 oracle's own drift from FP64 is the yardstick: the GPU may drift no
    more than a few times as far (its integrator's sin/cos/exp differ from
    libm in the last place).  Centre deviations in equivalent diameters,
    quaternion components, kinetic energy relative."""
    from sand_atlas_dem_gb300.shapes import synthetic_library
    from sand_atlas_dem_gb300.workloads import load_packing, material_spec

    pack = load_packing(SPARSE)
    library = synthetic_library("f4", 64)
    spec = material_spec(library, pack["ids"], pack["scales"], max_overlap_fraction=0.1)
    velocities = np.random.default_rng(44).normal(0.0, 0.05, (len(pack["ids"]), 3))
    case = dict(positions=pack["positions"], cell=pack["cell"], ids=pack["ids"], scales=pack["scales"],
                rotations=pack["rotations"], velocities=velocities)
    g = build(Engine, library, spec, case)
    o32 = build(OracleEngine, library, spec, case, threads=16)
    o64 = build(OracleEngine, library, spec, case, threads=16, precision="fp64")
    for e in (g, o32, o64):
        e.initialize()
    diameters = g.layout.body[:, 3].astype(float)
    inv_inertia = o64.layout.invI
    rows = []
    for _ in range(10):
        for e in (g, o32, o64):
            e.advance(100)
        sg, s32, s64 = g.state(), o32.state(), o64.state()
        box = s64["cell"][0, :3].astype(float)

        def deviation(s):
            d = centres(s) - centres(s64)
            d -= np.round(d / box) * box
            q, q64 = s["rotation"].astype(float), s64["rotation"].astype(float)
            sign = np.where(np.einsum("ij,ij->i", q, q64) < 0, -1.0, 1.0)
            return float((np.linalg.norm(d, axis=1) / diameters).max()), float(np.abs(sign[:, None] * q - q64).max())

        e64 = kinetic_energy(s64, o64.layout.body, inv_inertia)
        gpu_c, gpu_q = deviation(sg)
        cpu_c, cpu_q = deviation(s32)
        rows.append(dict(step=g.step, contacts=int(s64["contacts"]),
                         gpu_centre=gpu_c, gpu_rotation=gpu_q,
                         gpu_energy=abs(kinetic_energy(sg, g.layout.body, inv_inertia) - e64) / e64,
                         fp32_oracle_centre=cpu_c, fp32_oracle_rotation=cpu_q,
                         fp32_oracle_energy=abs(kinetic_energy(s32, o32.layout.body, inv_inertia) - e64) / e64,
                         same_keys_as_fp64=bool(sg["contacts"] == s64["contacts"]
                                                and np.array_equal(sg["meta"], s64["meta"]))))
    print(json.dumps(rows))
    assert g.step == o64.step == 1000
    assert rows[-1]["contacts"] > 0
    for r in rows:
        assert r["gpu_centre"] <= max(10 * r["fp32_oracle_centre"], 1e-7) and r["gpu_centre"] < 1e-5, r
        assert r["gpu_rotation"] <= max(10 * r["fp32_oracle_rotation"], 1e-6), r
        assert r["gpu_energy"] <= max(10 * r["fp32_oracle_energy"], 1e-5), r
