"""The post-processor's vorticity and Q-criterion (PostProcess.cpp:190-310),
restated in the oracle: against the analytic values of the Taylor-Green
initial field, and against the reference's own post-processor run on its own
512 x 256 x 128 grid (tests/golden/ref_postprocess.npz, made by
tests/golden/make_postprocess_golden.py from the unmodified program)."""
import numpy as np

from conftest import load_golden


def test_oracle_vorticity_q_taylor_green(oracle, cases):
    N = 32
    cfg, ic = cases.tgv(N)
    p = oracle.OraclePort(cfg)
    p.set_initial_conditions(*ic)
    vort, q = p.vorticity_q()
    x = np.array([i * cfg.Lx / (N - 1) for i in range(N)])
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    sx, cx, sy, cy, sz, cz = np.sin(X), np.cos(X), np.sin(Y), np.cos(Y), np.sin(Z), np.cos(Z)
    g = np.zeros((3, 3) + X.shape)  # g[c][e] = d u_c / d x_e
    g[0, 0], g[0, 1], g[0, 2] = cx * cy * cz, -sx * sy * cz, -sx * cy * sz
    g[1, 0], g[1, 1], g[1, 2] = sx * sy * cz, -cx * cy * cz, cx * sy * sz
    w = np.stack([g[2, 1] - g[1, 2], g[0, 2] - g[2, 0], g[1, 0] - g[0, 1]])
    S = 0.5 * (g + g.transpose(1, 0, 2, 3, 4))
    W = 0.5 * (g - g.transpose(1, 0, 2, 3, 4))
    q_exact = 0.5 * (W ** 2).sum(axis=(0, 1)) - 0.5 * (S ** 2).sum(axis=(0, 1))
    assert np.abs(vort - np.sqrt((w ** 2).sum(axis=0))).max() <= 1e-5
    assert np.abs(q - q_exact).max() <= 1e-5 * np.abs(q_exact).max()


def test_oracle_vorticity_q_matches_reference_postprocessor(oracle, cases):
    """The restatement on the post-processor's grid and state: the same
    numbers as the reference program's vortMag and qCrit, FP64 in full."""
    g = load_golden("ref_postprocess.npz")
    cfg, q = cases.postprocess_grid()
    p = oracle.OraclePort(cfg)
    for f, name in enumerate(("rho1", "rhoU1", "rhoV1", "rhoW1", "rhoE1")):
        p.set(name, q[f])
    vort, qc = p.vorticity_q()
    idx = g["idx"]
    ev = np.abs(vort.reshape(-1)[idx] - g["vort"]).max() / float(g["vort_max"])
    eq = np.abs(qc.reshape(-1)[idx] - g["qcrit"]).max() / float(g["qcrit_max"])
    assert ev <= 1e-14 and eq <= 1e-14, (ev, eq)
