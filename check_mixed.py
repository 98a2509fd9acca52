"""Kinetic-energy and dissipation error of the FP32-mixed form against the
FP64 form, per workload.

    python check_mixed.py [--workloads tgv128,hit256,shear]

Both forms run the same initial state with CFL time steps.  Every `every`
steps the diagnostics of calcTaylorGreenQuantities (CSolver_AWS.cpp:
2175-2257) are taken on the device: KE = sum rho |u|^2 / 2 / npts, the
dissipation -dKE/dt (central differences over the samples) and the
2mu-enstrophy integral.  Prints one JSON line per workload with the largest
relative errors of the mixed series against the FP64 series (KE relative to
KE, the dissipation measures relative to their largest FP64 value).
"""
import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
cs3d = importlib.import_module("3dcompactsolver_gb300")
cases = importlib.import_module("3dcompactsolver_gb300.cases")

WORKLOADS = {
    "tgv128": (lambda p: cases.tgv(128, precision=p), 1000, 10),
    "tgv64": (lambda p: cases.tgv(64, precision=p), 100, 5),
    "hit256": (lambda p: cases.hit(256, seed=0, precision=p), 200, 10),
    "shear": (lambda p: cases.shear_layer(precision=p), 1000, 10),
}


def series(make, precision, steps, every):
    cfg, ic = make(precision)
    s = cs3d.Solver(cfg)
    s.set_option(cs3d.OPT_STORE_DIAGNOSTICS, 1)
    s.set_initial_conditions(*ic)
    rows = []
    t0 = time.perf_counter()
    for k in range(steps // every):
        s.run(every)
        q = s.tgv_quantities()
        rows.append([q[0], q[1] / cfg.npts, q[4] / cfg.npts])
    s.sync()
    el = time.perf_counter() - t0
    s.close()
    return np.array(rows), el


def compare(name, steps=None, every=None):
    make, n, ev = WORKLOADS[name]
    steps = steps or n
    every = every or ev
    a, t64 = series(make, cs3d.FP64, steps, every)
    b, t32 = series(make, cs3d.FP32_MIXED, steps, every)
    ke_err = np.abs(b[:, 1] - a[:, 1]) / np.abs(a[:, 1])
    # -dKE/dt by central differences over the samples (each run its own times)
    da = -(a[2:, 1] - a[:-2, 1]) / (a[2:, 0] - a[:-2, 0])
    db = -(b[2:, 1] - b[:-2, 1]) / (b[2:, 0] - b[:-2, 0])
    diss_err = np.abs(db - da) / np.abs(da).max()
    ens_err = np.abs(b[:, 2] - a[:, 2]) / np.abs(a[:, 2]).max()
    return {"workload": name, "steps": steps, "sample_every": every,
            "time_fp64": float(a[-1, 0]), "time_mixed": float(b[-1, 0]),
            "ke_final": float(a[-1, 1]), "ke_rel_err_max": float(ke_err.max()),
            "ke_rel_err_final": float(ke_err[-1]),
            "dissipation_rel_err_max": float(diss_err.max()),
            "ens2mu_rel_err_max": float(ens_err.max()),
            "wall_s": {"fp64": t64, "mixed": t32}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workloads", default="tgv128,hit256,shear")
    ap.add_argument("--steps", type=int, default=0)
    args = ap.parse_args(argv)
    out = []
    for w in args.workloads.split(","):
        r = compare(w, steps=args.steps or None)
        print(json.dumps(r), flush=True)
        out.append(r)
    return out


if __name__ == "__main__":
    main()
