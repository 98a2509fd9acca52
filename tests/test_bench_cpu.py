"""bench.py pieces that need no GPU: the per-kernel byte model behind the
roofline numbers, and the reference arm's JSON line (the oracle on the host
cores, the requested warm-up steps)."""
import importlib
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    return importlib.import_module("bench")


def test_byte_model(bench):
    bpp = bench.kernel_bytes_per_point
    # mixed form, RK4: FP32 work arrays and stage-input shadow, FP64 q2
    # accumulated on every stage
    assert bpp("sweep_x", 4, 4) == 84
    assert bpp("sweep_y", 4, 4) == 104
    assert bpp("sweep_z", 4, 4) == pytest.approx(100 + (100 + 120 + 120 + 100) / 4.0)
    assert bpp("filter", 4, 4) == pytest.approx(220.0 / 3.0)
    assert bpp("cfl", 4, 4) == 20.0
    # plain FP64 form
    assert bpp("sweep_x", 8, 4) == 168
    assert bpp("sweep_z", 8, 4) == pytest.approx(330.0)
    assert bpp("filter", 8, 4) == 80.0
    # TVD-RK3 keeps the FP64 accumulation (plus the FP32 shadow in the mixed form)
    assert bpp("sweep_z", 4, 3) == pytest.approx(100 + 20 + (80 + 120 + 120) / 3.0)
    assert bpp("other", 4, 4) == 0.0


def test_flop_model(bench):
    fpp = bench.kernel_flops_per_point
    assert bench.SOLVE_FLOPS_D == 17 and bench.SOLVE_FLOPS_F == 25
    assert fpp("sweep_x", 4) == 263
    assert fpp("sweep_y", 4) == 293
    assert fpp("sweep_z", 4) == pytest.approx(460.5)
    assert fpp("filter", 4) == 125
    # a whole RK4 stage with the filter every step: about 1100 operations per point
    stage = sum(fpp(k, 4) for k in ("sweep_x", "sweep_y", "sweep_z")) + (3 * fpp("filter", 4) + fpp("cfl", 4)) / 4
    assert 1000 < stage < 1200


def test_reference_arm_line():
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "4"))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "tgv64", "--steps", "1", "--warmup", "2"],
                       capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["steps"] == 1 and line["warmup"] == 2
    assert line["value"] > 0 and line["unit"] == "Mpts/s per RK stage"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    # the same config object as the GPU arm prints for this workload
    cfg = line["config"]
    assert set(cfg) == {"workload", "npts", "rk_stages", "l2", "parallelism"}
    assert cfg["npts"] == 64 ** 3 and cfg["rk_stages"] == 4 and cfg["parallelism"] == "1 GPU"
