"""FP64 parity of the GPU path against the oracle at the workload sizes the
benchmark names, not just on small grids: the Taylor-Green vortex 64^3 for
100 RK4 steps (CFL 0.5, alphaF 0.49, filter every step), the Taylor-Green
vortex 128^3 (the benchmark's grid) for 10 steps, and the temporal shear
layer at its full 256 x 128 x 42 size for 5 TVD-RK3 steps (walls, sponge band,
one filtered step).  Bar: relative max-norm per conserved field <= 1e-12
(momenta against the largest momentum component), the time step and the
simulated time to 1e-13 relative.  Reference path: RK4.hpp:120-170,
TVDRK3.hpp:98-139, CSolver_AWS.cpp:507-551, 829-1504, 1682-1893."""
import importlib

import numpy as np
import pytest

from conftest import state_errors

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _run_both(gpu_pkg, oracle, cfg, ic, nsteps):
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    r = oracle.OraclePort(cfg)
    r.set_initial_conditions(*ic)
    s.run(nsteps)
    r.run(nsteps)
    s.sync()
    q = s.conserved()
    dt, t, ts = s.scalars()
    rdt, rt, rts = r.scalars()
    s.close()
    qr = r.conserved()
    return q, qr, (dt, t, ts), (rdt, rt, rts)


def _check(q, qr, sc, rsc, label):
    assert np.isfinite(q).all(), label
    errs = state_errors(q, qr)
    assert max(errs) <= TOL, (label, errs)
    assert sc[2] == rsc[2], (label, sc, rsc)
    assert abs(sc[0] - rsc[0]) <= 1e-13 * abs(rsc[0]), (label, sc, rsc)
    assert abs(sc[1] - rsc[1]) <= 1e-13 * abs(rsc[1]), (label, sc, rsc)
    return errs


def test_tgv64_100_steps_fp64(gpu_pkg, oracle, cases):
    """The Taylor-Green vortex 64^3, 100 RK4 steps, FP64."""
    cfg, ic = cases.tgv(64)
    q, qr, sc, rsc = _run_both(gpu_pkg, oracle, cfg, ic, 100)
    _check(q, qr, sc, rsc, "tgv64x100")


def test_tgv128_10_steps_fp64(gpu_pkg, oracle, cases):
    """The Taylor-Green vortex 128^3 (the benchmark's grid), 10 RK4 steps, FP64."""
    cfg, ic = cases.tgv(128)
    q, qr, sc, rsc = _run_both(gpu_pkg, oracle, cfg, ic, 10)
    _check(q, qr, sc, rsc, "tgv128x10")


def test_shear_layer_full_size_fp64(gpu_pkg, oracle, cases):
    """The temporal shear layer 256 x 128 x 42, 5 TVD-RK3 steps, FP64: y
    walls, the 15% sponge band and the filter on step 5."""
    abi = importlib.import_module("3dcompactsolver_gb300._abi")
    cfg, ic = cases.shear_layer(256, 128, 42, precision=abi.FP64)
    q, qr, sc, rsc = _run_both(gpu_pkg, oracle, cfg, ic, 5)
    _check(q, qr, sc, rsc, "shear256x128x42x5")
