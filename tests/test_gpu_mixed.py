"""The FP32-mixed form: kinetic-energy error against the FP64 form, and
stability on every workload shape."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ke(q):
    return float(0.5 * np.sum((q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]))


def test_tgv_mixed_ke_error(gpu_pkg, cases):
    """TGV 32^3, 40 RK4 steps: |KE_mixed - KE_fp64| / KE_fp64 < 1e-6."""
    abi = importlib.import_module("3dcompactsolver_gb300._abi")
    out = {}
    for prec in (abi.FP64, abi.FP32_MIXED):
        cfg, ic = cases.tgv(32, precision=prec)
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.run(40)
        s.sync()
        out[prec] = s.conserved()
        s.close()
    ke64, ke32 = _ke(out[abi.FP64]), _ke(out[abi.FP32_MIXED])
    assert abs(ke32 - ke64) / ke64 < 1e-6, (ke32, ke64)
    for f in range(5):
        d = np.abs(out[abi.FP32_MIXED][f] - out[abi.FP64][f]).max() / np.abs(out[abi.FP64][f]).max()
        assert d < 1e-4, (f, d)


def test_tgv_mixed_ke_drift(gpu_pkg, cases):
    """TGV 32^3, 300 RK4 steps at one fixed time step, filter every step: the
    mixed form's kinetic energy stays within 5e-7 of the FP64 form's.  An FP32
    filter applied as F itself (rather than v + (F - I) v) loses about 4e-8 of
    the energy per step and fails this by far."""
    abi = importlib.import_module("3dcompactsolver_gb300._abi")
    cfg, ic = cases.tgv(32)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.step()
    dt = s.scalars()[0]
    s.close()
    ke = {}
    for prec in (abi.FP64, abi.FP32_MIXED):
        cfg, _ = cases.tgv(32, precision=prec)
        cfg.dt_fixed = dt
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.run(300)
        ke[prec] = _ke(s.conserved())
        s.close()
    assert abs(ke[abi.FP32_MIXED] - ke[abi.FP64]) / ke[abi.FP64] < 5e-7, ke


@pytest.mark.parametrize("name", ["wall_moving_sponge", "shear", "hit"])
def test_mixed_tracks_fp64(gpu_pkg, cases, name):
    abi = importlib.import_module("3dcompactsolver_gb300._abi")
    mk = {
        "wall_moving_sponge": lambda p: cases.wall_box((20, 16, 12), moving=True, sponge=True, precision=p),
        "shear": lambda p: cases.shear_layer(32, 24, 16, precision=p),
        "hit": lambda p: cases.hit(32, precision=p),
    }[name]
    out = {}
    for prec in (abi.FP64, abi.FP32_MIXED):
        cfg, ic = mk(prec)
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.run(15)
        s.sync()
        out[prec] = s.conserved()
        s.close()
    for f in range(5):
        a, b = out[abi.FP32_MIXED][f], out[abi.FP64][f]
        assert np.isfinite(a).all()
        d = np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)
        assert d < 1e-4, (name, f, d)


def test_mixed_rk4_accumulator_mid_step(gpu_pkg, cases):
    """The mixed RK4 form accumulates q2 += a_s dq in FP64 on every stage
    (RK4.hpp:35-118): read between stages, the RK accumulator q2 (fields
    10..14) is q1 + sum a_i dq_i up to the FP32 rounding of each product
    a_i dq_i, and a value written there between stages is what the next stage
    adds to."""
    cfg, ic = cases.tgv(16, precision=gpu_pkg.FP32_MIXED)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(2)
    s.set_option(gpu_pkg.OPT_STORE_INCREMENTS, 1)
    q1 = s.conserved()
    s.pre_step()
    acc = np.zeros_like(q1)
    for st, b in ((1, 1 / 6), (2, 1 / 3), (3, 1 / 3)):
        s.sub_step(st, 0)
        dq = np.stack([s.get(15 + f) for f in range(5)])
        acc += b * dq
        q2 = np.stack([s.get(10 + f) for f in range(5)])
        for f in range(5):
            tol = 2e-7 * np.abs(acc[f]).max() + 1e-15 * np.abs(q1[f]).max()
            assert np.abs(q2[f] - (q1[f] + acc[f])).max() <= tol, (st, f)
    # a write to the accumulator between stages reaches the last stage
    shift = 1e-3
    q2w = q2[0] + shift
    s.set(10, q2w)
    s.sub_step(4, 0)
    dq4 = s.get(15)
    q2n = s.get(10)
    tol = 2e-7 * np.abs(dq4).max() + 1e-15 * np.abs(q2w).max()
    assert np.abs(q2n - (q2w + dq4 / 6)).max() <= tol
    s.close()
