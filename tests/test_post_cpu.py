"""The post-processor's vorticity and Q-criterion (PostProcess.cpp:190-310),
restated in the oracle: against the analytic values of the Taylor-Green
initial field.  The reference's post-processor is a stand-alone program with
fixed input paths and a text reader that cannot read its own binary dumps, so
it is pinned through its operators (the line operators, bit for bit in
test_oracle_pin.py) and this known answer."""
import numpy as np


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
