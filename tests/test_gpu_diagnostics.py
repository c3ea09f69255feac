"""The diagnostics dictionary (``gpu.py:746-891``) against the oracle's.

Stress tensors, p and q, strains, energies, dissipations, contact and pair
counts, coordination, fabric and sliding fraction, on a frictional, viscous,
compressing multi-grain lattice.  At the zero-timestep initialization the
per-grain rows and their 256-wide tree reductions are bit-identical, so every
value agrees to float64 rounding of the host's assembly; after timesteps each value is within 1e-5 of the largest
magnitude of its kind (the per-step state tolerance) and the counts are equal.
"""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu
COUNTS = ("step", "candidate_pairs", "active_surface_contacts", "active_grain_pairs")


def compare(go, oo, rel):
    for key, want in oo.items():
        got = go[key]
        if key in COUNTS:
            assert got == want, key
            continue
        a, b = np.asarray(got, np.float64), np.asarray(want, np.float64)
        if rel == 0:
            # The device rows are FP32 and identical; the host assembles them
            # in float64, where only the solid volume's summation order
            # differs (a last-place difference of the void ratio).
            assert np.allclose(a, b, rtol=1e-13, atol=0), (key, got, want)
            continue
        # Differences of large sums are compared on the scale of the sums:
        # q on p's, the antisymmetry (already relative) absolutely, the
        # unbalanced force (net over total contact force) at 1e-3 of itself.
        scale = {"q": abs(oo["p"]), "stress_antisymmetry": 1.0}.get(key, np.abs(b).max())
        tol = 1e-3 if key == "unbalanced_force" else rel
        assert np.abs(a - b).max() <= tol * max(scale, 1e-300), (key, got, want)


def test_diagnostics_match_oracle(gpu_library):
    library, spec, case = lattice_case(side=6, viscosity=4e5, speed=0.05)
    o = build(OracleEngine, library, spec, case, threads=8)
    g = build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    first = o.diagnostics()
    assert first["active_surface_contacts"] > 0 and first["active_grain_pairs"] > 100
    compare(g.diagnostics(), first, 0)
    for _ in range(3):
        o.advance(2, rate=(-0.5, -0.3, -0.1))
        g.advance(2, rate=(-0.5, -0.3, -0.1))
        oo = o.diagnostics()
        compare(g.diagnostics(), oo, 1e-5)
    assert oo["sliding_fraction"] > 0 and oo["normal_contact_dissipation"] > 0 and oo["p"] > 0
