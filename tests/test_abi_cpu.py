"""The C ABI without a GPU: every function declared in include/cs3d.h is
exported by the library, configurations are validated before any device
work, the C++ host layer compiles against the header, and the workload
generators produce what they claim."""
import ctypes
import importlib
import math
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    hdr = open(os.path.join(ROOT, "include", "cs3d.h")).read()
    return sorted(set(re.findall(r"\b(cs3d_[a-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol(gpu_pkg):
    lib = ctypes.CDLL(gpu_pkg.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_config_validation_without_device(gpu_pkg):
    cases = importlib.import_module("3dcompactsolver_gb300.cases")
    cfg, _ = cases.tgv(16)
    bad = [
        (cfg.copy(Nx=6), 2),                                     # too short for the filter
        (cfg.copy(filter_step=0), 1),
        (cfg.copy(rk=7), 1),
        (cfg.copy(precision=3), 1),
        (cfg.copy(Lx=0.0), 1),
        (cfg.copy(CFL=0.0), 1),
    ]
    for c, code in bad:
        with pytest.raises(gpu_pkg.CS3DError) as e:
            gpu_pkg.Solver(c)
        assert e.value.code == code, (e.value.code, str(e.value))
    c = cfg.copy()
    c.bc_type[1] = 5
    with pytest.raises(gpu_pkg.CS3DError) as e:
        gpu_pkg.Solver(c)
    assert e.value.code == 1


def test_operator_handle_validation_without_device(gpu_pkg):
    """cs3d_op_create checks its direction's line length, L and BC type (and
    nothing of the other directions) before looking for a device."""
    cfg = gpu_pkg.make_config((16, 3, 2), (1.0, 1.0, 1.0))
    for c, d, code in [(cfg.copy(Nx=6), 0, 2), (cfg.copy(Lx=0.0), 0, 1), (cfg, 3, 1)]:
        with pytest.raises(gpu_pkg.CS3DError) as e:
            gpu_pkg.Operator(c, d)
        assert e.value.code == code, (e.value.code, str(e.value))
    c = cfg.copy()
    c.bc_type[0] = 4
    with pytest.raises(gpu_pkg.CS3DError) as e:
        gpu_pkg.Operator(c, 0)
    assert e.value.code == 1
    with pytest.raises(gpu_pkg.CS3DError) as e:
        gpu_pkg.Operator(cfg, 1)  # Ny = 3: too short for the compact closures
    assert e.value.code == 2


def test_valid_config_reports_missing_device(gpu_pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cases = importlib.import_module("3dcompactsolver_gb300.cases")
    cfg, _ = cases.tgv(16)
    with pytest.raises(gpu_pkg.CS3DError) as e:
        gpu_pkg.Solver(cfg)
    assert e.value.code == 7


def test_cpp_host_layer_compiles(gpu_pkg, tmp_path):
    exe = tmp_path / "tgv_main"
    cmd = ["g++", "-O1", "-std=c++14", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "3dcompactsolver_gb300", "host"),
           os.path.join(ROOT, "3dcompactsolver_gb300", "host", "tgv_main.cpp"), "-o", str(exe),
           "-L" + os.path.dirname(gpu_pkg.LIB_PATH), "-lcs3d_gb300",
           "-Wl,-rpath," + os.path.dirname(gpu_pkg.LIB_PATH)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_hit_field_is_solenoidal_at_target_mach(cases):
    cfg, (rho, p, U, V, W) = cases.hit(32, seed=3)
    n = 32
    k = np.fft.fftfreq(n, d=1.0 / n)
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    div = KX * np.fft.fftn(U) + KY * np.fft.fftn(V) + KZ * np.fft.fftn(W)
    assert np.abs(div).max() < 1e-9 * np.abs(np.fft.fftn(U)).max()
    mt = math.sqrt(float(np.mean(U * U + V * V + W * W))) / math.sqrt(1.4 * p.mean() / 1.0)
    assert abs(mt - 0.3) < 1e-12


def test_tgv_matches_reference_driver_formulas(cases):
    cfg, (rho, p, U, V, W) = cases.tgv(16, legacy_p=100.0)
    L = 2 * math.pi - 2 * math.pi / 16
    x = (3 / 15.0) * L
    y = (5 / 15.0) * L
    z = (7 / 15.0) * L
    assert abs(U[7, 5, 3] - math.sin(x) * math.cos(y) * math.cos(z)) < 1e-15
    assert abs(p[7, 5, 3] - (100 + (1 / 16) * (math.cos(2 * x) + math.cos(2 * y)) * (math.cos(2 * z) + 2))) < 1e-13
