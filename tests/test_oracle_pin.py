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


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libref3d_strict.so")),
                    reason="reference harness not built here (no reference checkout)")
@pytest.mark.parametrize("name", ["wall_moving_sponge", "shear"])
def test_port_bit_identical_to_live_reference(oracle, cases, name):
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
