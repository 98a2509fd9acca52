"""Regenerate the golden fixtures of tests/golden from the reference.

Needs the reference checkout (oracle/Makefile's REF, or $CS3D_REFERENCE)
and the reference harness built by `make -C oracle ref`.  Writes:

  taylorgreen_run64_head.txt   rows 1-5 of taylorgreen_vortex/taylorgreen_run64/taylorgreen.out
  taylorgreen_run128_head.txt  rows 1-3 of taylorgreen_vortex/taylorgreen_run128/taylorgreen.out
  ref_<case>.npz               q1 after 3 steps of the reference's own CSolver_AWS + RK4/TVDRK3
                               (oracle/_ref, strict build), with dt, time and timeStep
  ref_diagnostics.npz          the reference's calcTurbulenceQuantities row and shearLayerInfoCalc
                               profiles after 2 steps + the stages of a third (before postStep's sponge)
  ref_aero.npz                 the reference's AeroOptics::computeAO OPL after 3 unfiltered steps
  ref_lineops.npz              the reference's calc1stDerivField / calc2ndDerivField /
                               filterField on seeded random fields

Run:  python tests/golden/make_golden.py
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

REF = oracle.reference_dir()
if REF is None:
    raise SystemExit("make_golden.py: no reference checkout (set REF in oracle/Makefile or $CS3D_REFERENCE)")
cases = importlib.import_module("3dcompactsolver_gb300.cases")
_abi = importlib.import_module("3dcompactsolver_gb300._abi")

# Small cases: every boundary kind, both integrators, sponge faces and bands.
CASES = {
    "tgv12": lambda: cases.tgv(12),
    "wall": lambda: cases.wall_box((12, 10, 9)),
    "wall_moving_sponge": lambda: cases.wall_box((12, 10, 9), moving=True, sponge=True),
    "wall_tvdrk3": lambda: cases.wall_box((12, 10, 9), rk=_abi.TVDRK3),
    "shear": lambda: cases.shear_layer(16, 12, 10, precision=_abi.FP64),
}
NSTEPS = 3
DIAG_EXTRA = {"hit12": lambda: cases.hit(12, seed=3, k0=3.0)}
DIAG_CASES = ["tgv12", "hit12", "shear", "wall_moving_sponge"]
AERO_CASES = {"shear": lambda: cases.shear_layer(16, 12, 10, precision=_abi.FP64),
              "tgv12_nofilter": lambda: cases.tgv(12, filter_step=1000)}

# single operators: (kind, dir, bc_type, (Nx, Ny, Nz))
LINEOPS = [(k, d, bc, n) for k in (1, 2, 3) for d in (0, 1, 2) for bc in (0, 1)
           for n in [(12, 10, 9)]] + [(k, 0, bc, (37, 3, 2)) for k in (1, 2, 3) for bc in (0, 1)]


def main():
    for N, rows in ((64, 5), (128, 3)):
        src = os.path.join(REF, f"taylorgreen_vortex/taylorgreen_run{N}/taylorgreen.out")
        with open(src) as f:
            lines = [next(f) for _ in range(rows)]
        with open(os.path.join(HERE, f"taylorgreen_run{N}_head.txt"), "w") as f:
            f.writelines(lines)
    oracle.build(ref=True)
    for name, mk in CASES.items():
        cfg, ic = mk()
        r = oracle.RefSolver(cfg)
        r.set_initial_conditions(*ic)
        for _ in range(NSTEPS):
            r.step()
        dt, t, ts = r.scalars()
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), q1=r.conserved(), dt=dt, time=t,
                            timeStep=ts, nsteps=NSTEPS)
    # the reference's calcTurbulenceQuantities and shearLayerInfoCalc after two
    # steps and the stages of a third, before its post-step (the order of
    # CSolver_AWS::postStep, CSolver_AWS.cpp:2930-2938)
    diag = {}
    for name in DIAG_CASES:
        cfg, ic = CASES[name]() if name in CASES else DIAG_EXTRA[name]()
        r = oracle.RefSolver(cfg)
        r.set_initial_conditions(*ic)
        r.run(2)
        r.pre_step()
        nst = 3 if cfg.rk == _abi.TVDRK3 else 4
        for st in range(1, nst + 1):
            r.sub_step(st, st == nst)
        diag[f"{name}_turb"] = r.turbulence_quantities()
        diag[f"{name}_shear"] = r.shear_layer_info()
    np.savez_compressed(os.path.join(HERE, "ref_diagnostics.npz"), **diag)
    # the reference's AeroOptics::computeAO (5 angles up to 70 degrees) after 3
    # steps without filtering, where its rho2 holds the state
    aero = {}
    for name, mk in AERO_CASES.items():
        cfg, ic = mk()
        r = oracle.RefSolver(cfg)
        r.set_initial_conditions(*ic)
        for _ in range(3):
            r.step()
        aero[name], _ = r.aero_optics(5, 70.0)
    np.savez_compressed(os.path.join(HERE, "ref_aero.npz"), **aero)
    rng = np.random.default_rng(2024)
    out = {}
    for idx, (kind, d, bc, n) in enumerate(LINEOPS):
        Nd = n[d]
        nl = n[0] * n[1] * n[2] // Nd
        x = rng.standard_normal((nl, Nd)) + np.sin(np.linspace(0, 3, Nd))[None, :]
        L = (3.0, 2.5, 2.0)
        y = oracle.line_op_ref(kind, d, bc, n, L, 0.47, x)
        out[f"in{idx}"] = x
        out[f"out{idx}"] = y
        out[f"meta{idx}"] = np.array([kind, d, bc, n[0], n[1], n[2]])
    out["L"] = np.array([3.0, 2.5, 2.0])
    out["alphaF"] = np.array(0.47)
    np.savez_compressed(os.path.join(HERE, "ref_lineops.npz"), **out)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
