"""Packing preparation on the GPU engine and on the CPU oracle, side by side.

The force-descent preparation (affine compression, FIRE on the centres,
Jacobi rotation steps; ``workloads.descent_packing``) evaluates the
zero-timestep contact forces and torques hundreds of times and moves every
grain by them.  Driven by the GPU engine and by the oracle from the same
seed, the two runs take the same number of force evaluations and end in
the same packing, bit for bit: every one of those force passes agreed.
(The committed 1,000-grain solid-fraction-0.35 record took 2,857 passes and
came out identical on both as well.)
"""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from sand_atlas_dem_gb300.workloads import descent_packing
from tests.specimens import small_library

pytestmark = pytest.mark.gpu


def test_descent_packing_is_identical_on_gpu_and_oracle(gpu_library):
    library = small_library()
    runs = []
    for cls in (Engine, lambda *a, **k: OracleEngine(*a, threads=8, **k)):
        out = descent_packing(library, 125, 0.3, seed=7, overlap=0.01, engine_cls=cls)
        state = out["engine"].state()
        runs.append((out["evaluations"], out["phi"], out["overlap"], state))
    (eg, pg, og, sg), (eo, po, oo, so) = runs
    assert eg == eo > 50 and pg == po and og == oo
    for name in ("position", "positionRemainder", "rotation", "cell"):
        assert sg[name].tobytes() == so[name].tobytes(), name
    assert sg["contacts"] == so["contacts"] > 0
    np.testing.assert_array_equal(sg["meta"], so["meta"])
