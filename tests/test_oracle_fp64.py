"""The FP64 drift oracle: the oracle's kernels built in double precision.

On a contact-rich lattice it collects the same contacts as the FP32
restatement, its forces agree to FP32 rounding, and over 200 steps the two
stay within the FP32 drift of one another.  The FP64 build passes the
reference's closed-form cube force (``tests/test_cpu_solver.py:176-199``) at
the reference's tolerance.
"""

import numpy as np

from oracle.engine import OracleEngine
from tests.specimens import build, cube_pair, lattice_case


def centres(s):
    return s["position"][:, :3].astype(float) + s["positionRemainder"][:, :3]


def test_fp64_oracle_follows_the_fp32_restatement():
    library, spec, case = lattice_case(viscosity=4e5, speed=0.05)
    o32 = build(OracleEngine, library, spec, case, threads=4)
    o64 = build(OracleEngine, library, spec, case, threads=4, precision="fp64")
    for e in (o32, o64):
        e.initialize()
    s32, s64 = o32.state(), o64.state()
    assert s64["position"].dtype == np.float64
    assert s32["contacts"] == s64["contacts"] > 0
    np.testing.assert_array_equal(s32["meta"], s64["meta"])
    scale = np.abs(s64["force"][:, :3]).max()
    assert np.abs(s32["force"][:, :3] - s64["force"][:, :3]).max() < 1e-5 * scale
    for _ in range(2):
        for e in (o32, o64):
            e.advance(100, rate=(-0.5, -0.5, -0.5))
    s32, s64 = o32.state(), o64.state()
    np.testing.assert_array_equal(s32["meta"], s64["meta"])
    assert np.abs(centres(s32) - centres(s64)).max() < 1e-7  # diameters, after 200 steps
    assert np.abs(s32["rotation"] - s64["rotation"]).max() < 1e-6


def test_fp64_oracle_exact_cube_force():
    e = cube_pair(lambda *a, **k: OracleEngine(*a, precision="fp64", **k))
    e.initialize()
    force = e.buffers["force"][:2, :3] * e.force_unit
    # The reference's tolerance: the geometry enters as FP32-rounded
    # normalized nodes and vertices in both builds.
    np.testing.assert_allclose(force[0], [-0.001, 0.0, 0.0], rtol=2e-4, atol=1e-9)
    np.testing.assert_allclose(force[1], [0.001, 0.0, 0.0], rtol=2e-4, atol=1e-9)
