"""The C++ host layer (3dcompactsolver_gb300/host) drives the GPU path the
way the reference's main() drives CSolver_AWS; its result equals the C ABI
driven from Python."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cpp_driver_matches_python_api(gpu_pkg, cases, tmp_path):
    exe = tmp_path / "tgv_main"
    cmd = ["g++", "-O2", "-std=c++14", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "3dcompactsolver_gb300", "host"),
           os.path.join(ROOT, "3dcompactsolver_gb300", "host", "tgv_main.cpp"), "-o", str(exe),
           "-L" + os.path.dirname(gpu_pkg.LIB_PATH), "-lcs3d_gb300",
           "-Wl,-rpath," + os.path.dirname(gpu_pkg.LIB_PATH)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe), "24", "4", "0"], capture_output=True, text=True, check=True).stdout
    ke_cpp = float(out.split("KE")[1])
    cfg, ic = cases.tgv(24)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(4)
    q = s.conserved()
    ke = float(0.5 * np.sum((q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]))
    assert abs(ke_cpp - ke) <= 1e-12 * ke, (ke_cpp, ke)
