"""A GPU engine's checkpoint written in the reference's HDF5 format and
restarted in a fresh GPU engine and in the CPU oracle."""

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300 import checkpoint
from sand_atlas_dem_gb300.engine import Engine
from tests.specimens import build, lattice_case

pytestmark = pytest.mark.gpu


def test_gpu_checkpoint_restarts_on_gpu_and_oracle(gpu_library, tmp_path):
    library, spec, case = lattice_case(viscosity=4e5)
    g = build(Engine, library, spec, case)
    g.initialize()
    g.advance(4, rate=(-0.5, -0.5, -0.5))
    path = tmp_path / "gb300.h5"
    checkpoint.save_checkpoint(path, g)
    attrs, state = checkpoint.load_checkpoint(path)
    assert attrs["backend"] == "gb300" and attrs["step"] == 4 and attrs["format"] == "sand-dem-checkpoint/5"
    restarted, oracle = build(Engine, library, spec, case), build(OracleEngine, library, spec, case)
    checkpoint.resume(restarted, path)
    checkpoint.resume(oracle, path)
    a, o = restarted.state(), oracle.state()
    np.testing.assert_array_equal(a["meta"], o["meta"])
    assert a["force"].tobytes() == o["force"].tobytes() and a["slip"].tobytes() == o["slip"].tobytes()
    g.advance(3, rate=(-0.5, -0.5, -0.5))
    restarted.advance(3, rate=(-0.5, -0.5, -0.5))
    x, y = g.state(), restarted.state()
    np.testing.assert_array_equal(x["meta"], y["meta"])
    for name in ("position", "velocity", "force", "slip"):
        np.testing.assert_allclose(y[name], x[name], rtol=2e-6, atol=1e-9, err_msg=name)
