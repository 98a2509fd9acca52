"""AeroOptics::computeAO on the GPU: against the reference's own OPL arrays
after unfiltered steps (where its rho2 is the state) and against the oracle
restatement on filtered steps (density of the state q1)."""
import numpy as np
import pytest

from conftest import load_golden, rel_err
from test_oracle_pin import AERO_CASES, aero_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", AERO_CASES)
def test_gpu_aero_optics_matches_reference(gpu_pkg, cases, name):
    g = load_golden("ref_aero.npz")
    cfg, ic = aero_case(cases, name)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(3)
    assert rel_err(s.aero_optics(5, 70.0), g[name]) <= 1e-13


def test_gpu_aero_optics_filtered_and_angles(gpu_pkg, cases, oracle):
    cfg, ic = cases.tgv(16)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(4)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    p.run(4)
    for na, ma in ((5, 70.0), (3, 45.0), (9, 80.0)):
        assert rel_err(s.aero_optics(na, ma), p.aero_optics(na, ma)) <= 1e-13, (na, ma)
    with pytest.raises(gpu_pkg.CS3DError):
        s.aero_optics(1, 70.0)
    with pytest.raises(gpu_pkg.CS3DError):
        s.aero_optics(5, 90.0)
