"""Known-answer trajectory: the reference's committed Taylor-Green output
taylorgreen_vortex/taylorgreen_run64/taylorgreen.out (rows 1-5, in
tests/golden), reproduced by the GPU path through cs3d_tgv_quantities."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_gpu_reproduces_taylorgreen_run64(gpu_pkg, cases):
    rows = np.loadtxt(os.path.join(GOLDEN, "taylorgreen_run64_head.txt"))
    cfg, ic = cases.tgv(64, CFL=0.5, alphaF=0.495, filter_step=2, legacy_p=100.0, mu_ref=0.000014625)
    s = gpu_pkg.Solver(cfg)
    s.set_option(gpu_pkg.OPT_STORE_DIAGNOSTICS, 1)
    s.set_initial_conditions(*ic)
    for k in range(len(rows)):
        s.step()
        q = s.tgv_quantities()
        g = rows[k]
        assert abs(q[0] - g[0]) <= 1e-13 * max(abs(g[0]), 1.0), (k, q[0], g[0])
        for c in (1, 2, 3, 4, 5):
            assert abs(q[c] - g[c]) <= 1e-11 * abs(g[c]), (k, c, q[c], g[c])
        assert abs(q[6] - g[6]) <= 1e-8 * abs(g[6])
