"""CUDA step against the CPU oracle on identical seeded inputs.

Bit-exact gates: pair lists, contact keys (and their canonical order), contact
geometry, history slots and, at the zero-timestep initialization, forces.
After timesteps the integrator's transcendental functions (CUDA vs libm
sin/cos/exp) may differ in the last place, so state is compared at 1e-5
relative (the per-step force/torque/pose tolerance of the contract).
"""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu
REL = 1e-5


def committed(e, name, dtype=np.float32):
    count = int(e.check_errors()[2])
    side = e.sides[1 - e.active]
    if isinstance(side[name], np.ndarray):
        return side[name][:count]
    return e.m.read_prefix(side[name], 4 * count, dtype, shape=(count, 4))


def gpu_buffer(e, name, dtype, rows, width=4):
    return e.read(name, dtype, (rows, width))


def assert_close(a, b, rel=REL, what=""):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max() if a.size else 0.0
    assert err <= rel * scale, f"{what}: max error {err:.3e} vs scale {scale:.3e}"


@pytest.mark.parametrize("viscosity", [0.0, 4e5])
def test_initialize_bit_exact(gpu_library, viscosity):
    library, spec, case = lattice_case(viscosity=viscosity)
    o = build(OracleEngine, library, spec, case)
    g = build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    oc, gc = o.check_errors(), g.check_errors()
    assert oc[1] == gc[1] and oc[2] == gc[2] and oc[1] > 0 and oc[2] > 0
    pairs = int(oc[1])
    np.testing.assert_array_equal(gpu_buffer(g, "pairs", np.uint32, pairs, 2), o.buffers["pairs"][:pairs])
    count = int(oc[2])
    for name in ("meta", "normalArea"):
        dtype = np.uint32 if name == "meta" else np.float32
        assert committed(g, name, dtype).tobytes() == committed(o, name, dtype).tobytes(), name
    for name in ("pointDepth", "contactForce"):
        assert gpu_buffer(g, name, np.float32, count).tobytes() == o.buffers[name][:count].tobytes(), name
    n = spec.particles
    for name in ("force", "torque", "particleStress", "particleDiagnostic", "accumulated"):
        rows = 3 * n if name == "particleStress" else n
        assert gpu_buffer(g, name, np.float32, rows).tobytes() == o.buffers[name][:rows].tobytes(), name


@pytest.mark.parametrize("policy", ["conservative", "active-contact"])
def test_steps_match_oracle(gpu_library, policy):
    library, spec, case = lattice_case(policy=policy, viscosity=4e5)
    o = build(OracleEngine, library, spec, case)
    g = build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    for chunk in (1, 2, 3):
        o.advance(chunk, rate=(-0.5, -0.5, -0.5))
        g.advance(chunk, rate=(-0.5, -0.5, -0.5))
        so, sg = o.state(), g.state()
        assert so["contacts"] == sg["contacts"]
        np.testing.assert_array_equal(sg["meta"], so["meta"])
        for name in ("position", "velocity", "rotation", "momentum", "force", "torque", "slip",
                     "normalArea", "accumulated"):
            assert_close(sg[name], so[name], what=name)


def test_restore_collects_identically(gpu_library):
    """Per-phase gate from identical state: restore the GPU's own state into
    both engines; pair lists, contact keys and history slots must agree."""
    library, spec, case = lattice_case()
    g = build(Engine, library, spec, case)
    g.initialize()
    g.advance(4)
    state = g.state()
    o = build(OracleEngine, library, spec, case)
    g2 = build(Engine, library, spec, case)
    o.restore(state, 4)
    g2.restore(state, 4)
    so, sg = o.state(), g2.state()
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    assert sg["slip"].tobytes() == so["slip"].tobytes()
    assert sg["force"].tobytes() == so["force"].tobytes()


def test_graph_replay_is_bitwise_reproducible(gpu_library):
    library, spec, case = lattice_case()
    states = []
    for use_graph in (True, True, False):
        g = build(Engine, library, spec, case, use_graph=use_graph)
        g.initialize()
        g.advance(5, rate=(-0.5, -0.5, -0.5))
        states.append(g.state())
    for s in states[1:]:
        for k, v in states[0].items():
            if isinstance(v, np.ndarray):
                assert v.tobytes() == s[k].tobytes(), k


@pytest.mark.parametrize("side,spacing", [(8, 0.985), (10, 1.05)])
def test_multibin_specimen_matches_oracle(gpu_library, side, spacing):
    """Several bins per axis, periodic wrap across bin boundaries."""
    library, spec, case = lattice_case(side=side, spacing=spacing, viscosity=4e5, speed=0.05)
    o = build(OracleEngine, library, spec, case, threads=8)
    g = build(Engine, library, spec, case)
    assert g.bins.min() >= 3
    o.initialize()
    g.initialize()
    for _ in range(3):
        o.advance(2, rate=(-0.5, -0.5, -0.5))
        g.advance(2, rate=(-0.5, -0.5, -0.5))
        so, sg = o.state(), g.state()
        assert so["contacts"] == sg["contacts"]
        np.testing.assert_array_equal(sg["meta"], so["meta"])
        for name in ("position", "velocity", "force", "torque", "slip"):
            assert_close(sg[name], so[name], what=name)


def test_graph_branches_skip_only_idle_work(gpu_library):
    """The captured step holds the neighbour build and the filter build as
    conditional bodies keyed on their device flags.  Over a run in which both
    rebuild on some steps and not on others (fast grains), replayed graphs,
    plain launches and the oracle agree: bitwise between the two launch
    modes; identical contact keys and poses within the step tolerance
    against the oracle."""
    library, spec, case = lattice_case(viscosity=4e5, speed=50.0)
    o = build(OracleEngine, library, spec, case, threads=8)
    engines = [build(Engine, library, spec, case, use_graph=flag) for flag in (True, False)]
    o.initialize()
    for e in engines:
        e.initialize()
    for _ in range(4):
        o.advance(100, rate=(-0.5, -0.5, -0.5))
        for e in engines:
            e.advance(100, rate=(-0.5, -0.5, -0.5))
    work = [e.read("work", np.uint32, (64,)) for e in engines]
    rebuilds, builds = int(work[0][17]), int(work[0][9])
    assert 2 <= rebuilds < 200 and 2 <= builds < 200, (rebuilds, builds)
    assert work[0].tobytes() == work[1].tobytes()
    sg, sp, so = engines[0].state(), engines[1].state(), o.state()
    for key, value in sg.items():
        if isinstance(value, np.ndarray):
            assert value.tobytes() == sp[key].tobytes(), key
    # 400 fast steps carry the last-place differences of the integrator's
    # transcendentals forward (the per-step gate is the tests above): the
    # contact keys stay identical and the poses agree to the step tolerance.
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    for name in ("position", "velocity", "rotation"):
        assert_close(sg[name], so[name], what=name)
    lib = engines[0].lib
    assert lib.sdg_engine_kernels_per_step(engines[0]._native) > 0
    assert lib.sdg_engine_branch_kernels(engines[0]._native, 0) >= 10
    assert lib.sdg_engine_branch_kernels(engines[0]._native, 1) >= 10


@pytest.mark.parametrize("pairs_per_particle", [8, 32])
def test_both_cell_list_paths_give_the_reference_pairs(gpu_library, pairs_per_particle):
    """The neighbour build sorts the grains into bins by an LSD radix sort
    whose scratch lives in the pair-by-second-grain array; where that array is
    too small for it (8 pairs a grain here: 512 words against the sort's 513)
    the atomic bin fill with a rank sort per bin runs instead.  Both give the
    oracle's pair list, pair for pair and in order."""
    from dataclasses import replace

    library, spec, case = lattice_case(spacing=1.05)
    spec = replace(spec, pairs_per_particle=pairs_per_particle)
    o = build(OracleEngine, library, spec, case)
    g = build(Engine, library, spec, case)
    o.initialize()
    g.initialize()
    oc, gc = o.check_errors(), g.check_errors()
    pairs = int(oc[1])
    assert gc[1] == pairs > 0
    np.testing.assert_array_equal(gpu_buffer(g, "pairs", np.uint32, pairs, 2), o.buffers["pairs"][:pairs])
    n = spec.particles
    np.testing.assert_array_equal(gpu_buffer(g, "pairOffsets", np.uint32, n, 1), o.buffers["pairOffsets"][:n].reshape(n, 1))
