"""Drift over a 1,000-step horizon: CUDA step against the CPU oracle.

The per-step gate is 1e-5 relative (the CUDA and libm transcendentals of the
integrator may differ in the last place, and the difference is carried
forward).  Over 1,000 steps of a dense, compressing, frictional lattice the
test records, every 100 steps, the largest centre deviation (in units of the
grain's equivalent diameter), the largest quaternion component deviation,
and whether
the contact key sets are still identical, and prints the table.  The FP64
closed-form horizon (2,000 steps of the elastic release oscillator against
the analytic solution) is ``test_known_answers.py``.
"""

import json

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
