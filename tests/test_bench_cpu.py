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
    # mixed form, RK4: FP32 work arrays and shadow, FP32 increment sum
    assert bpp("sweep_x", 4, 4) == 84
    assert bpp("sweep_y", 4, 4) == 104
    assert bpp("sweep_z", 4, 4) == pytest.approx(180.0)
    assert bpp("filter", 4, 4) == pytest.approx(220.0 / 3.0)
    assert bpp("cfl", 4, 4) == 20.0
    # plain FP64 form
    assert bpp("sweep_x", 8, 4) == 168
    assert bpp("sweep_z", 8, 4) == pytest.approx(330.0)
    assert bpp("filter", 8, 4) == 80.0
    # TVD-RK3 keeps the FP64 accumulation (plus the FP32 shadow in the mixed form)
    assert bpp("sweep_z", 4, 3) == pytest.approx(100 + 20 + (80 + 120 + 120) / 3.0)
    assert bpp("other", 4, 4) == 0.0


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
