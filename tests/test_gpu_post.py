"""Vorticity magnitude and Q-criterion on the GPU against the oracle
restatement, on periodic and wall grids, after steps and after a restart
from dump files (the post-processor's use)."""
import importlib

import numpy as np
import pytest

from test_oracle_pin import _case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tgv12", "wall", "shear"])
def test_gpu_vorticity_q_matches_oracle(gpu_pkg, cases, oracle, name):
    cfg, ic = _case(cases, name)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(3)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    p.run(3)
    v, q = s.vorticity_q()
    vr, qr = p.vorticity_q()
    assert np.abs(v - vr).max() <= 1e-12 * np.abs(vr).max()
    assert np.abs(q - qr).max() <= 1e-12 * np.abs(qr).max()


def test_gpu_vorticity_q_from_dump(gpu_pkg, cases, tmp_path):
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    cfg, ic = cases.tgv(16, precision=_abi.FP32_MIXED)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(2)
    v0, q0 = s.vorticity_q()
    s.dump_solution(str(tmp_path) + "/")
    t = gpu_pkg.Solver(cfg)
    t.load_solution(str(tmp_path) + "/", 2, 0.0)
    v1, q1 = t.vorticity_q()
    assert np.array_equal(v0, v1) and np.array_equal(q0, q1)
