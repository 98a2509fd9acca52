"""Regenerate tests/golden/ref_postprocess.npz: the vorticity magnitude and
Q-criterion of the reference's own post-processor.

Needs the reference checkout (oracle/Makefile's REF, or $CS3D_REFERENCE).
PostProcess.cpp, Derivatives.cpp, VisitWriter.cpp and Utils.cpp are compiled
from where they lie (strict flags, as the oracle's parity build), with
Utils.cpp's getRange renamed so that pp_capture.cpp's getRange captures every
field PostProcess.cpp reports at full FP64 precision.  The program runs
unmodified in a scratch directory on the state of cases.postprocess_grid(),
written as the text files it reads (PostProcess.cpp:101-183, 512 x 256 x 128
values each, "%.17g" so the parse is exact).  The fixture keeps the outputs
at 8192 seeded points and on three whole y-lines (the wall closures).

    python tests/golden/make_postprocess_golden.py
"""
import importlib
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

REF = oracle.reference_dir()
if REF is None:
    raise SystemExit("make_postprocess_golden.py: no reference checkout (set REF in oracle/Makefile or $CS3D_REFERENCE)")
cases = importlib.import_module("3dcompactsolver_gb300.cases")
FLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp", "-std=c++11", "-w"]
SUBDIR = "ShearLayer/A3_FullDomain_k6nocurl_10oversqrt3percpert"  # PostProcess.cpp:103-175
LINES = [(0, 0), (300, 77), (511, 127)]  # (i, k) of the y-lines kept whole


def sample_indices(cfg):
    rng = np.random.default_rng(20261204)
    n = cfg.Nx * cfg.Ny * cfg.Nz
    pts = rng.choice(n, size=8192, replace=False)
    lines = [k * cfg.Nx * cfg.Ny + np.arange(cfg.Ny) * cfg.Nx + i for i, k in LINES]
    return np.sort(np.unique(np.concatenate([pts] + lines)))


def main():
    cfg, q = cases.postprocess_grid()
    work = tempfile.mkdtemp(prefix="cs3d_pp_")
    try:
        utils_o = os.path.join(work, "Utils.o")
        subprocess.run(["g++"] + FLAGS + ["-DgetRange=ref_getRange", "-I" + REF, "-c",
                                          os.path.join(REF, "Utils.cpp"), "-o", utils_o], check=True)
        exe = os.path.join(work, "postprocess")
        subprocess.run(["g++"] + FLAGS + ["-I" + REF] +
                       [os.path.join(REF, f) for f in ("PostProcess.cpp", "Derivatives.cpp", "VisitWriter.cpp")] +
                       [os.path.join(HERE, "pp_capture.cpp"), utils_o, "-o", exe, "-lm"], check=True)
        d = os.path.join(work, SUBDIR)
        os.makedirs(d)
        t0 = time.time()
        for f, name in enumerate(("rho", "rhoU", "rhoV", "rhoW", "rhoE")):
            q[f].reshape(-1).tofile(os.path.join(d, f"{name}.out.5000"), sep="\n", format="%.17g")
        print(f"inputs written in {time.time() - t0:.0f} s", flush=True)
        t0 = time.time()
        r = subprocess.run([exe], cwd=work, capture_output=True, text=True)
        print(f"post-processor ran in {time.time() - t0:.0f} s, rc {r.returncode}", flush=True)
        if r.returncode != 0:
            raise SystemExit(r.stdout[-2000:] + r.stderr[-2000:])
        vort = np.fromfile(os.path.join(work, "VORTMAG.f64"))
        qcrit = np.fromfile(os.path.join(work, "QCRIT.f64"))
        # the post-processor read back exactly the state we wrote
        rho = np.fromfile(os.path.join(work, "RHO.f64"))
        assert np.array_equal(rho, q[0].reshape(-1))
    finally:
        shutil.rmtree(work, ignore_errors=True)
    idx = sample_indices(cfg)
    np.savez_compressed(os.path.join(HERE, "ref_postprocess.npz"), idx=idx, vort=vort[idx], qcrit=qcrit[idx],
                        vort_max=np.abs(vort).max(), qcrit_max=np.abs(qcrit).max(),
                        lines=np.array(LINES))
    print("wrote ref_postprocess.npz:", idx.size, "points; |vort| max", np.abs(vort).max(),
          "|Q| max", np.abs(qcrit).max())


if __name__ == "__main__":
    main()
