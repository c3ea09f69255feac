"""Stored node-filter results against the filters run every step.

With a filter margin, the leaf cull, the node filter and the node prefilter
store their results built with every test grown by the margin, and later
steps reuse them while no grain has moved that far relative to a partner
(only the exact queries run).  Contacts, forces and the whole state must stay
bit-identical to an engine that runs the filters every step (margin 0),
whether the stored results are reused, rebuilt after motion beyond the
margin, or checked again after a restart.
"""

import numpy as np
import pytest

from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu
W_FILTER_MARGIN, W_FILTER_BUILDS, W_FILTER_STEPS, W_CERTIFIED, W_DORMANT = 8, 9, 10, 15, 18
RATE = (-0.5, -0.5, -0.5)


def counters(e):
    work = e.read("work", np.uint32, (64,))
    return int(work[W_FILTER_BUILDS]), int(work[W_FILTER_STEPS])


def assert_same(a, b):
    sa, sb = a.state(), b.state()
    assert sa["contacts"] == sb["contacts"] > 0
    for key, value in sa.items():
        if isinstance(value, np.ndarray):
            assert value.tobytes() == sb[key].tobytes(), key


def engines(margin, speed=0.05, **case_args):
    library, spec, case = lattice_case(viscosity=4e5, speed=speed, **case_args)
    plain = build(Engine, library, spec, case, filter_margin=0.0)
    stored = build(Engine, library, spec, case, filter_margin=margin)
    for e in (plain, stored):
        e.initialize()
    return plain, stored


def turned(state, grain, angle):
    """State with one grain turned by `angle` about z and renormalized."""
    out = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in state.items()}
    q = out["rotation"][grain, :4].astype(np.float64)
    h = 0.5 * angle
    r = np.array([0.0, 0.0, np.sin(h), np.cos(h)])
    v = r[3] * q[:3] + q[3] * r[:3] + np.cross(r[:3], q[:3])
    w = r[3] * q[3] - r[:3] @ q[:3]
    turned_q = np.append(v, w)
    out["rotation"][grain, :4] = turned_q / np.linalg.norm(turned_q)
    out["rotationRemainder"][grain] = 0.0
    return out


def test_reused_results_are_bit_identical(gpu_library):
    plain, stored = engines(1e-3)
    for chunk in (1, 5, 20):
        for e in (plain, stored):
            e.advance(chunk, rate=RATE)
        assert_same(plain, stored)
    builds, steps = counters(stored)
    assert steps == 27  # the initialization and 26 steps
    assert 1 <= builds <= 2, builds  # built at the start, reused since
    assert counters(plain) == (0, 27)
    # Most exact queries of the reuse steps were answered by a walk
    # certificate, and some stored slots were dormant (their nodes proven out
    # of reach until the next build) -- with the state bit-identical.
    work = stored.read("work", np.uint32, (64,))
    certified, kept, dormant = int(work[W_CERTIFIED]), int(work[3]), int(work[W_DORMANT])
    assert certified > 5 * kept, (certified, kept)
    assert 0 < dormant < kept, (dormant, kept)


def test_motion_beyond_the_margin_rebuilds(gpu_library):
    plain, stored = engines(1e-3)
    for e in (plain, stored):
        e.advance(2, rate=RATE)
    builds, _ = counters(stored)
    # A turn of 1e-7 rad moves no node near 1e-3 of the shape size: reused.
    small = turned(plain.state(), 0, 1e-7)
    for e in (plain, stored):
        e.restore(small, 2)
        e.advance(3, rate=RATE)
    assert_same(plain, stored)
    assert counters(stored)[0] == builds
    # A turn of 0.02 rad moves the grain's surface by about 1e-2 of its
    # size, beyond the margin: the next collector run builds again.
    large = turned(plain.state(), 0, 0.02)
    for e in (plain, stored):
        e.restore(large, 5)
    assert counters(stored)[0] == builds + 1
    for e in (plain, stored):
        e.advance(3, rate=RATE)
    assert_same(plain, stored)
    assert counters(stored)[0] == builds + 1


def test_margin_below_rounding_slack_builds_every_step(gpu_library):
    plain, stored = engines(1e-9)
    for e in (plain, stored):
        e.advance(4, rate=RATE)
    assert_same(plain, stored)
    assert counters(stored) == (5, 5)


def test_many_steps_with_rebuilds_stay_identical(gpu_library):
    """Fast grains (2 m/s: a few 1e-6 of a diameter per step) against a
    margin of 1e-4: builds and reuses alternate over a long run, and the
    margin grows toward 16 times the configured one as builds come early."""
    plain, stored = engines(1e-4, speed=2.0)
    for _ in range(4):
        for e in (plain, stored):
            e.advance(25, rate=RATE)
        assert_same(plain, stored)
    builds, steps = counters(stored)
    assert steps == 101
    assert 3 <= builds <= 90, builds
    margin = stored.read("work", np.uint32, (64,))[W_FILTER_MARGIN:W_FILTER_MARGIN + 1].view(np.float32)[0]
    assert 1e-4 < margin <= 16e-4 * (1 + 1e-6), margin


def test_margin_is_validated(gpu_library):
    library, spec, case = lattice_case()
    with pytest.raises(ValueError, match="filter margin"):
        build(Engine, library, spec, case, filter_margin=-1.0)
