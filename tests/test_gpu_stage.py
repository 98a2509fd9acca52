"""Full time steps of the GPU path (plain FP64 form) against the
reference's own outputs (tests/golden/ref_*.npz) and against the oracle,
for every boundary kind and both integrators."""
import importlib

import numpy as np
import pytest

from conftest import load_golden, rel_err, state_errors

pytestmark = pytest.mark.gpu
TOL = 1e-12  # relative max-norm per conserved field, FP64 form


def _cases(cases):
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    return {
        "tgv12": lambda: cases.tgv(12),
        "wall": lambda: cases.wall_box((12, 10, 9)),
        "wall_moving_sponge": lambda: cases.wall_box((12, 10, 9), moving=True, sponge=True),
        "wall_tvdrk3": lambda: cases.wall_box((12, 10, 9), rk=_abi.TVDRK3),
        "shear": lambda: cases.shear_layer(16, 12, 10, precision=_abi.FP64),
    }


@pytest.mark.parametrize("name", ["tgv12", "wall", "wall_moving_sponge", "wall_tvdrk3", "shear"])
def test_steps_match_reference_outputs(gpu_pkg, cases, name):
    g = load_golden(f"ref_{name}.npz")
    cfg, ic = _cases(cases)[name]()
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(int(g["nsteps"]))
    s.sync()
    q = s.conserved()
    dt, t, ts = s.scalars()
    assert ts == int(g["timeStep"])
    assert abs(dt - float(g["dt"])) <= 1e-13 * float(g["dt"])
    errs = state_errors(q, g["q1"])
    assert max(errs) <= TOL, (name, errs)


@pytest.mark.parametrize("name,nsteps", [("tgv12", 30), ("wall", 20), ("wall_moving_sponge", 20),
                                         ("wall_tvdrk3", 20), ("shear", 20)])
def test_many_steps_match_oracle(gpu_pkg, oracle, cases, name, nsteps):
    cfg, ic = _cases(cases)[name]()
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    r = oracle.OraclePort(cfg)
    r.set_initial_conditions(*ic)
    s.run(nsteps)
    r.run(nsteps)
    s.sync()
    errs = state_errors(s.conserved(), r.conserved())
    assert max(errs) <= TOL, (name, errs)


@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 20, 18), (33, 17, 9)])
def test_tgv_ragged_shapes_match_oracle(gpu_pkg, oracle, cases, shape):
    """Non-cubic, odd and non-multiple-of-tile shapes."""
    cfg, ic = cases.tgv(shape[0])
    Nx, Ny, Nz = shape
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    cfg = _abi.make_config(shape, (2.0, 1.7, 1.3), alphaF=0.48, mu_ref=1e-3, CFL=0.5)
    rng = np.random.default_rng(7)
    z, y, x = np.meshgrid(np.linspace(0, 1.3, Nz), np.linspace(0, 1.7, Ny), np.linspace(0, 2, Nx),
                          indexing="ij")
    rho = 1 + 0.05 * np.sin(3 * x + 2 * y) * np.cos(z)
    U = 0.2 * np.sin(2 * y) + 0.01 * rng.standard_normal(x.shape)
    V = 0.1 * np.cos(x + z)
    W = 0.1 * np.sin(x - y)
    p = np.full(x.shape, 1 / 1.4)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(rho, p, U, V, W)
    r = oracle.OraclePort(cfg)
    r.set_initial_conditions(rho, p, U, V, W)
    s.run(10)
    r.run(10)
    s.sync()
    errs = state_errors(s.conserved(), r.conserved())
    assert max(errs) <= TOL, errs


def test_stage_increments_match_oracle(gpu_pkg, oracle, cases):
    """dt*RHS of the first stage (rhok2..rhoEk2, CSolver_AWS.cpp:1246-1504)
    including the wall and sponge fix-ups."""
    cfg, ic = cases.wall_box((14, 12, 10), moving=True, sponge=True)
    s = gpu_pkg.Solver(cfg)
    s.set_option(gpu_pkg.OPT_STORE_INCREMENTS, 1)
    s.set_initial_conditions(*ic)
    r = oracle.OraclePort(cfg)
    r.set_initial_conditions(*ic)
    s.pre_step(); r.pre_step()
    s.sub_step(1, False); r.sub_step(1, False)
    s.sync()
    for f, nm in enumerate(("rhok2", "rhoUk2", "rhoVk2", "rhoWk2", "rhoEk2")):
        a = s.get(15 + f)
        b = r.get(nm)
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(b).max(), 1e-300), nm
        assert np.array_equal(a == 0.0, b == 0.0), nm  # the same points are zeroed


def test_deterministic(gpu_pkg, cases):
    cfg, ic = cases.tgv(16)
    out = []
    for _ in range(2):
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.run(3)
        s.sync()
        out.append(s.conserved())
        s.close()
    assert np.array_equal(out[0], out[1])


def test_nan_in_state_is_reported(gpu_pkg, cases):
    """Fault injected on the host: a NaN written into the state makes
    cs3d_sync return CS3D_ERR_NAN; the context stays usable."""
    cfg, ic = cases.tgv(12)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    q = s.get(0)
    q[3, 4, 5] = np.nan
    s.set(0, q)
    s.step()
    with pytest.raises(gpu_pkg.CS3DError) as e:
        s.sync()
    assert e.value.code == 4
    s2 = gpu_pkg.Solver(cfg)  # the device is still fine
    s2.set_initial_conditions(*ic)
    s2.step()
    s2.sync()


def test_call_order_errors(gpu_pkg, cases):
    cfg, ic = cases.tgv(12)
    s = gpu_pkg.Solver(cfg)
    with pytest.raises(gpu_pkg.CS3DError) as e:
        s.step()
    assert e.value.code == 6
    s.set_initial_conditions(*ic)
    with pytest.raises(gpu_pkg.CS3DError) as e:
        s.sub_step(1, False)
    assert e.value.code == 6
    with pytest.raises(gpu_pkg.CS3DError) as e:
        s.tgv_quantities()
    assert e.value.code == 6


@pytest.mark.parametrize("mixed", [False, True])
def test_bulk_conserved_matches_per_field(gpu_pkg, cases, mixed):
    """cs3d_set_conserved / cs3d_get_conserved move the five conserved fields
    as cs3d_set_field / cs3d_get_field do, FP32 shadow included: a step after
    either is bit-identical."""
    prec = gpu_pkg.FP32_MIXED if mixed else gpu_pkg.FP64
    cfg, ic = cases.tgv(16, precision=prec)
    a = gpu_pkg.Solver(cfg)
    a.set_initial_conditions(*ic)
    a.run(2)
    q = a.conserved()
    assert all(np.array_equal(q[f], a.get(f)) for f in range(5))
    rng = np.random.default_rng(9)
    q = q * (1.0 + 1e-3 * rng.standard_normal(q.shape))
    b = gpu_pkg.Solver(cfg)
    b.set_initial_conditions(*ic)
    b.run(2)
    a.set_conserved(q)
    for f in range(5):
        b.set(f, q[f])
    assert np.array_equal(a.conserved(), q)
    a.step()
    b.step()
    assert np.array_equal(a.conserved(), b.conserved())
