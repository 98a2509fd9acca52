"""Pins the oracle (the C restatement in oracle/cs3d_oracle.c) to the
reference: against the reference's own outputs committed in tests/golden
(made by tests/golden/make_golden.py from the reference sources), against the
reference's committed Taylor-Green trajectories, and -- where the reference
harness is built (oracle/_ref) -- bit for bit against the live reference."""
import os
import platform

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, rel_err

CASE_NAMES = ["tgv12", "wall", "wall_moving_sponge", "wall_tvdrk3", "shear"]


def _case(cases, name):
    import importlib
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    table = {
        "tgv12": lambda: cases.tgv(12),
        "wall": lambda: cases.wall_box((12, 10, 9)),
        "wall_moving_sponge": lambda: cases.wall_box((12, 10, 9), moving=True, sponge=True),
        "wall_tvdrk3": lambda: cases.wall_box((12, 10, 9), rk=_abi.TVDRK3),
        "shear": lambda: cases.shear_layer(16, 12, 10, precision=_abi.FP64),
    }
    return table[name]()


@pytest.mark.parametrize("name", CASE_NAMES)
def test_port_matches_reference_outputs(oracle, cases, name):
    g = load_golden(f"ref_{name}.npz")
    cfg, ic = _case(cases, name)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    p.run(int(g["nsteps"]))
    q = p.conserved()
    dt, t, ts = p.scalars()
    assert ts == int(g["timeStep"])
    assert abs(dt - float(g["dt"])) <= 1e-14 * abs(float(g["dt"]))
    assert abs(t - float(g["time"])) <= 1e-14 * max(abs(float(g["time"])), 1e-300)
    # bit-identical on the machine that made the fixtures (x86-64 glibc); other
    # libm builds may differ in the last place of pow/sqrt
    tol = 0.0 if platform.machine() == "x86_64" else 1e-13
    for f in range(5):
        assert rel_err(q[f], g["q1"][f]) <= tol, (name, f, rel_err(q[f], g["q1"][f]))


def test_port_line_operators_match_reference(oracle):
    g = load_golden("ref_lineops.npz")
    L = g["L"]
    aF = float(g["alphaF"])
    i = 0
    while f"in{i}" in g:
        kind, d, bc, nx, ny, nz = [int(v) for v in g[f"meta{i}"]]
        n3 = (nx, ny, nz)
        N = n3[d]
        dh = (1.0 / (N - 1.0)) * L[d]
        out = oracle.line_op_port(kind, bc, N, dh, aF, g[f"in{i}"])
        assert rel_err(out, g[f"out{i}"]) <= 1e-15, (kind, d, bc, n3)
        i += 1
    assert i >= 20


def _tgv_rows(N):
    return np.loadtxt(os.path.join(GOLDEN, f"taylorgreen_run{N}_head.txt"))


def test_port_reproduces_taylorgreen_run64(oracle, cases):
    """taylorgreen_vortex/taylorgreen_run64: CFL 0.5, filterStep 2,
    alphaF 0.495, mu_ref 1.4625e-5, p = 100 + ... (3DCompact.cpp_N64)."""
    rows = _tgv_rows(64)
    cfg, ic = cases.tgv(64, CFL=0.5, alphaF=0.495, filter_step=2, legacy_p=100.0, mu_ref=0.000014625)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    for s in range(len(rows)):
        p.step()
        q = p.tgv_quantities()
        gold = rows[s]
        assert abs(q[0] - gold[0]) <= 1e-14 * max(abs(gold[0]), 1.0)
        for c in (1, 2, 3, 4, 5):  # KE, dissipation, enstrophy, 2mu-enstrophy, mean mu
            assert abs(q[c] - gold[c]) <= 1e-12 * abs(gold[c]), (s, c, q[c], gold[c])
        assert abs(q[6] - gold[6]) <= 1e-10 * abs(gold[6])  # rms dilatation: a tiny quantity


@pytest.mark.parametrize("name", ["wall_moving_sponge", "shear"])
def test_port_bit_identical_to_live_reference(oracle, cases, name):
    if not oracle.ref_available():
        pytest.skip("reference harness not built here (no reference checkout)")
    cfg, ic = _case(cases, name)
    p = oracle.OraclePort(cfg)
    r = oracle.RefSolver(cfg)
    p.set_initial_conditions(*ic)
    r.set_initial_conditions(*ic)
    for _ in range(2):
        p.step()
        r.step()
    for nm in ("rho1", "rhoU1", "rhoV1", "rhoW1", "rhoE1", "U", "T", "mu", "Ux", "Wyz", "Tzz"):
        assert np.array_equal(p.get(nm), r.get(nm)), nm


DIAG_CASES = ["tgv12", "hit12", "shear", "wall_moving_sponge"]


def _diag_case(cases, name):
    if name == "hit12":
        return cases.hit(12, seed=3, k0=3.0)
    return _case(cases, name)


def diag_compare(turb, info, g, name, tol):
    """turbdata row and shear-layer profiles against the reference's (rows the
    reference does not write are NaN in the fixture)."""
    ref = g[f"{name}_turb"]
    for i, (a, b) in enumerate(zip(turb, ref)):
        assert abs(a - b) <= tol * abs(b) + 1e-300, (name, "turb", i, a, b)
    ref = g[f"{name}_shear"]
    vvar = np.nanmax(np.abs(ref[7:10]))
    for k in range(ref.shape[0]):
        if np.isnan(ref[k]).all():
            continue
        # velocity means against the velocity scale and velocity (co)variances
        # against the largest variance: for the Taylor-Green vortex the plane
        # means and the covariances are rounding noise about zero
        nat = np.sqrt(vvar) if 1 <= k <= 3 else (vvar if 7 <= k <= 9 or k >= 12 else 0.0)
        scale = max(np.abs(ref[k]).max(), nat, 1e-300)
        # a variance about a mean m picks up 2 sqrt(var) * (state rounding, ~1e-13 m)
        atol = 0.0
        if 6 <= k <= 11 and not np.isnan(ref[k - 6]).all():
            atol = 2.0 * np.sqrt(np.abs(ref[k]).max()) * 1e-13 * np.abs(ref[k - 6]).max()
        assert np.abs(info[k] - ref[k]).max() <= tol * scale + atol, (name, "shear", k)


def _stages_then(sv, cfg):
    import importlib
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    nst = 3 if cfg.rk == _abi.TVDRK3 else 4
    sv.run(2)
    sv.pre_step()
    for st in range(1, nst + 1):
        sv.sub_step(st, st == nst)


@pytest.mark.parametrize("name", DIAG_CASES)
def test_port_diagnostics_match_reference(oracle, cases, name):
    """calcTurbulenceQuantities and shearLayerInfoCalc: the restatement against
    the reference's own output files (tests/golden/ref_diagnostics.npz); sums in
    another order, so not bit for bit."""
    g = load_golden("ref_diagnostics.npz")
    cfg, ic = _diag_case(cases, name)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    _stages_then(p, cfg)
    info = p.shear_layer_info()
    # the reference writes uwprime = u'w' + v'w' and vwprime = 0 (CSolver_AWS.cpp:2317-2318)
    sc = np.abs(info[7:10]).max()  # covariances are measured against the velocity variances
    assert np.abs(info[13] - (info[15] + info[16])).max() <= 1e-12 * sc
    assert not info[14].any()
    diag_compare(p.turbulence_quantities(), info, g, name, 1e-11)


def test_reference_dump_format(oracle, cases):
    """dumpSolution's format, read from the reference itself: five raw FP64
    files of q1 in XYZ order, no header, named <field>.out.<step>."""
    if not oracle.ref_available():
        pytest.skip("reference harness not built here")
    cfg, ic = _case(cases, "wall")
    r = oracle.RefSolver(cfg)
    r.set_initial_conditions(*ic)
    for _ in range(3):
        r.step()
    files = r.dump_solution()
    names = ["rho", "rhoU", "rhoV", "rhoW", "rhoE"]
    assert sorted(files) == sorted(f"{n}.out.3" for n in names)
    for f, n in enumerate(names):
        data = np.frombuffer(files[f"{n}.out.3"], dtype="<f8")
        assert data.size == cfg.npts
        assert np.array_equal(data, r.get(["rho1", "rhoU1", "rhoV1", "rhoW1", "rhoE1"][f]).reshape(-1))


AERO_CASES = ["shear", "tgv12_nofilter"]


def aero_case(cases, name):
    import importlib
    _abi = importlib.import_module("3dcompactsolver_gb300._abi")
    if name == "shear":
        return cases.shear_layer(16, 12, 10, precision=_abi.FP64)
    if name == "tgv12_nofilter":
        return cases.tgv(12, filter_step=1000)
    return cases.tgv(12)


@pytest.mark.parametrize("name", AERO_CASES)
def test_port_aero_optics_matches_reference(oracle, cases, name):
    """AeroOptics::computeAO after 3 steps without filtering (where the
    reference's rho2 is the state): the restatement bit for bit on x86-64."""
    g = load_golden("ref_aero.npz")
    cfg, ic = aero_case(cases, name)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    p.run(3)
    tol = 0.0 if platform.machine() == "x86_64" else 1e-14
    assert rel_err(p.aero_optics(5, 70.0), g[name]) <= tol
