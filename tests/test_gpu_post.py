"""Vorticity magnitude and Q-criterion on the GPU against the reference's
own post-processor (tests/golden/ref_postprocess.npz, its 512 x 256 x 128
grid), against the oracle restatement on periodic and wall grids, after
steps and after a restart from dump files (the post-processor's use)."""
import importlib

import numpy as np
import pytest

from conftest import load_golden

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


def test_gpu_vorticity_q_matches_reference_postprocessor(gpu_pkg, cases):
    """cs3d_vorticity_q on the post-processor's grid and state (PostProcess.cpp:
    44-79, 190-310) against the reference program's own FP64 output, 1e-12
    relative to each field's largest value."""
    g = load_golden("ref_postprocess.npz")
    cfg, q = cases.postprocess_grid()
    s = gpu_pkg.Solver(cfg)
    one, zero = np.ones(q[0].shape), np.zeros(q[0].shape)
    s.set_initial_conditions(one, one, zero, zero, zero)
    s.set_conserved(q)
    vort, qc = s.vorticity_q()
    s.close()
    idx = g["idx"]
    ev = np.abs(vort.reshape(-1)[idx] - g["vort"]).max() / float(g["vort_max"])
    eq = np.abs(qc.reshape(-1)[idx] - g["qcrit"]).max() / float(g["qcrit_max"])
    assert ev <= 1e-12 and eq <= 1e-12, (ev, eq)
