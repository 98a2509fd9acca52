"""The drop-in binding (3dcompactsolver_gb300/host/cs3d_ref_binding.hpp)
compiled against the reference's own headers, read in place from the
reference checkout: CSolver_GB300 derives from the reference's
AbstractCSolver, RK4_GB300 / TVDRK3_GB300 from its RK4 / TVDRK3 and override
only updateConservedData(), and the reference's unmodified
executeSolverLoop() (RK4.hpp:120-170, TVDRK3.hpp:98-139) drives the C ABI.

* against a call-recording test double of the C ABI (tests/binding/
  mock_cs3d.c): the sequence of C-ABI calls the reference's loops issue;
* against the real libcs3d_gb300.so: on a machine without a GPU the solver's
  constructor reports CS3D_ERR_NODEV through cs3d_ref::Error; with a GPU
  the run completes.
Skipped where no reference checkout exists (the GPU machines have none)."""
import os
import subprocess

import pytest

from conftest import ROOT

BIND = os.path.join(ROOT, "tests", "binding")
INC = [os.path.join(ROOT, "include"), os.path.join(ROOT, "3dcompactsolver_gb300", "host")]


@pytest.fixture(scope="module")
def ref_dir(oracle):
    d = oracle.reference_dir()
    if d is None:
        pytest.skip("no reference checkout here")
    return d


def _compile(ref, out, extra):
    cmd = (["g++", "-std=c++11", "-O1", "-w", "-I" + ref] + ["-I" + i for i in INC] +
           [os.path.join(BIND, "ref_loop_main.cpp"), os.path.join(ref, "Utils.cpp"), "-o", out] + extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _calls(stdout):
    return [ln[5:] for ln in stdout.splitlines() if ln.startswith("CALL ")]


@pytest.fixture(scope="module")
def mock_exe(ref_dir, tmp_path_factory):
    d = tmp_path_factory.mktemp("bind")
    obj = str(d / "mock_cs3d.o")
    r = subprocess.run(["gcc", "-std=c99", "-c", "-I" + INC[0], os.path.join(BIND, "mock_cs3d.c"), "-o", obj],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = str(d / "ref_loop_mock")
    _compile(ref_dir, exe, [obj])
    return exe


@pytest.mark.parametrize("rk,nst", [(0, 4), (1, 3)])
def test_reference_loop_issues_the_stage_calls(mock_exe, rk, nst):
    steps = 3
    r = subprocess.run([mock_exe, "16", str(steps), str(rk)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    calls = _calls(r.stdout)
    assert calls[0] == f"create 16 16 16 rk {rk} filter_step 1"
    assert calls[1].startswith("set_initial_conditions 1.000000")
    assert calls[2] == "get_field 0..14"          # host mirrors after setInitialConditions
    body = calls[3:]
    per_step = ["pre_step"] + [f"sub_step {s} {int(s == nst)}" for s in range(1, nst + 1)] + \
               ["post_step", "get_field 0..14"]  # checkStep = 1: mirrors every step
    expect = per_step * steps
    expect[-1:] = ["get_field 0..14", "get_field 0..14"]  # the end of the run syncs once more
    assert body[:len(expect)] == expect, body
    # the operator-only handle for Derivatives_GB300, then teardown
    assert body[len(expect):] == ["op_create dir 0 bc 0", "op_apply_host 1", "destroy", "op_destroy"]
    assert f"steps {steps} " in r.stdout


def test_rk_mismatch_is_reported(ref_dir, tmp_path, mock_exe):
    """A solver built for RK4 driven by the TVD-RK3 loop is refused (the
    stage count would not match) rather than computed wrongly."""
    src = tmp_path / "mismatch.cpp"
    src.write_text('#include "cs3d_ref_binding.hpp"\n'
                   'int main() { Domain d(8, 8, 8, 1, 1, 1);\n'
                   '  TimeStepping ts(TimeStepping::CONST_CFL, 0.5, 2, 1e300, 1, 1, 1 << 30);\n'
                   '  BC bc(BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC, BC::PERIODIC_SOLVE, BC::PERIODIC,\n'
                   '        BC::PERIODIC, BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC);\n'
                   '  cs3d_ref::CSolver_GB300 cs(&d, &bc, &ts, 0.49, 1e-3, 16, false, CS3D_RK4);\n'
                   '  cs.writeDumps = false;\n'
                   '  cs3d_ref::TVDRK3_GB300 rk(&cs);\n'
                   '  try { rk.executeSolverLoop(); } catch (const cs3d_ref::Error &e) { return e.code; }\n'
                   '  return 0; }\n')
    obj = os.path.join(os.path.dirname(mock_exe), "mock_cs3d.o")
    exe = str(tmp_path / "mismatch")
    cmd = (["g++", "-std=c++11", "-w", "-I" + ref_dir] + ["-I" + i for i in INC] +
           [str(src), os.path.join(ref_dir, "Utils.cpp"), obj, "-o", exe])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 6  # CS3D_ERR_STATE


def test_binding_links_the_library(ref_dir, gpu_pkg, tmp_path):
    import torch
    exe = str(tmp_path / "ref_loop_lib")
    libdir = os.path.dirname(gpu_pkg.LIB_PATH)
    _compile(ref_dir, exe, ["-L" + libdir, "-lcs3d_gb300", "-Wl,-rpath," + libdir])
    r = subprocess.run([exe, "16", "2", "0"], capture_output=True, text=True, timeout=300)
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        assert "steps 2 " in r.stdout
    else:
        assert r.returncode == 7, (r.returncode, r.stderr)  # CS3D_ERR_NODEV
        assert "no CUDA device" in r.stderr
