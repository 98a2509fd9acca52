"""On-device diagnostics against the reference: calcTurbulenceQuantities and
shearLayerInfoCalc after two steps and the stages of a third (before the
post-step sponge update, as the reference's postStep orders them), compared
with the reference's own outputs (tests/golden/ref_diagnostics.npz) and the
oracle restatement."""
import numpy as np
import pytest

from conftest import load_golden
from test_oracle_pin import DIAG_CASES, _diag_case, _stages_then, diag_compare

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", DIAG_CASES)
def test_gpu_diagnostics_match_reference(gpu_pkg, cases, oracle, name):
    g = load_golden("ref_diagnostics.npz")
    cfg, ic = _diag_case(cases, name)
    s = gpu_pkg.Solver(cfg)
    s.set_option(gpu_pkg.OPT_STORE_DIAGNOSTICS, 1)
    s.set_initial_conditions(*ic)
    _stages_then(s, cfg)
    turb = s.turbulence_quantities()
    info = s.shear_layer_info()
    diag_compare(turb, info, g, name, 1e-10)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    _stages_then(p, cfg)
    assert np.abs(info - p.shear_layer_info()).max() <= 1e-12 * np.abs(info).max()


def test_gpu_shear_info_mixed_tracks_fp64(gpu_pkg, cases):
    import importlib
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    out = []
    for prec in (_abi.FP64, _abi.FP32_MIXED):
        cfg, ic = cases.shear_layer(32, 24, 16, precision=prec)
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.run(10)
        out.append(s.shear_layer_info())
    for k in (0, 1, 6, 7):
        assert np.abs(out[1][k] - out[0][k]).max() <= 1e-5 * np.abs(out[0][k]).max(), k
