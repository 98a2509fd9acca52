"""Single compact operators on the GPU (cs3d_deriv1 / cs3d_deriv2 /
cs3d_filter, the replacements of Derivatives::calc1stDerivField,
calc2ndDerivField and Filter::filterField) against the reference's own
outputs (tests/golden/ref_lineops.npz) and against the oracle."""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-13  # FP64: the GPU uses precomputed reciprocals and fused multiply-adds


def _run(gpu_pkg, kind, d, bc, n3, L3, aF, lines):
    """Apply operator kind along direction d.  A solver handle needs at
    least 8 points in every direction, so other directions are widened and
    the extra lines padded with zeros."""
    import torch
    p = gpu_pkg
    bt = [p.PERIODIC_SOLVE] * 3
    bt[d] = bc
    n3 = tuple(n if (i == d or n >= 8) else 8 for i, n in enumerate(n3))
    N = n3[d]
    nl = n3[0] * n3[1] * n3[2] // N
    lines = np.asarray(lines, dtype=np.float64).reshape(-1, N)
    given = lines.shape[0]
    if given < nl:
        lines = np.concatenate([lines, np.zeros((nl - given, N))])
    cfg = p.make_config(n3, L3, bc_type=tuple(bt), alphaF=aF)
    s = p.Solver(cfg)
    x = torch.from_numpy(np.ascontiguousarray(lines, dtype=np.float64)).cuda()
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    s.line_op(kind, d, x.data_ptr(), y.data_ptr())
    s.sync()
    out = y.cpu().numpy()[:given]
    s.close()
    return out


def test_lineops_match_reference_fixtures(gpu_pkg):
    g = load_golden("ref_lineops.npz")
    L = tuple(float(v) for v in g["L"])
    aF = float(g["alphaF"])
    i = 0
    while f"in{i}" in g:
        kind, d, bc, nx, ny, nz = [int(v) for v in g[f"meta{i}"]]
        out = _run(gpu_pkg, kind, d, bc, (nx, ny, nz), L, aF, g[f"in{i}"])
        assert rel_err(out, g[f"out{i}"]) <= TOL, (i, kind, d, bc, rel_err(out, g[f"out{i}"]))
        i += 1


@pytest.mark.parametrize("N", [8, 9, 33, 64, 128, 256])
@pytest.mark.parametrize("kind", [1, 2, 3])
@pytest.mark.parametrize("bc", [0, 1])
def test_lineops_match_oracle(gpu_pkg, oracle, N, kind, bc):
    rng = np.random.default_rng(N * 10 + kind * 3 + bc)
    n3 = (N, 8, 8)
    L3 = (2.0 * np.pi * (1 - 1.0 / N), 1.0, 1.0)
    lines = rng.standard_normal((64, N)) + 3.0
    out = _run(gpu_pkg, kind, 0, bc, n3, L3, 0.49, lines)
    dh = (1.0 / (N - 1.0)) * L3[0]
    ref = oracle.line_op_port(kind, bc, N, dh, 0.49, lines)
    assert rel_err(out, ref) <= TOL


def test_derivative_of_sine_is_cosine(gpu_pkg):
    """Known answer: the 6th-order compact derivative of sin on a periodic
    grid of 64 points is cos to ~1e-9."""
    N = 64
    L = 2 * np.pi * (1 - 1.0 / N)
    x = np.array([(i / (N - 1.0)) * L for i in range(N)])
    lines = np.tile(np.sin(x), (4, 1))
    out = _run(gpu_pkg, 1, 0, 0, (N, 2, 2), (L, 1.0, 1.0), 0.49, lines)
    assert np.abs(out - np.cos(x)[None, :]).max() < 1e-8
    out2 = _run(gpu_pkg, 2, 0, 0, (N, 2, 2), (L, 1.0, 1.0), 0.49, lines)
    assert np.abs(out2 + np.sin(x)[None, :]).max() < 1e-7


def test_wall_closure_exact_on_cubic(gpu_pkg):
    """The wall closures are exact for low-order polynomials: d/dx of a cubic."""
    N = 20
    L = 1.0
    x = np.array([(i / (N - 1.0)) * L for i in range(N)])
    f = 1 + 2 * x - x ** 2 + 0.5 * x ** 3
    out = _run(gpu_pkg, 1, 0, 1, (N, 2, 2), (L, 1.0, 1.0), 0.49, np.tile(f, (4, 1)))
    assert np.abs(out - (2 - 2 * x + 1.5 * x ** 2)[None, :]).max() < 1e-10


def test_operator_handle_matches_reference_fixtures(gpu_pkg):
    """The operator-only handle (cs3d_op_apply_host, host arrays as the
    reference's calc1stDerivField / calc2ndDerivField / filterField take them,
    and cs3d_op_apply on device arrays) on the exact grids of the reference
    fixtures -- no widening of the other directions."""
    import torch
    g = load_golden("ref_lineops.npz")
    L = tuple(float(v) for v in g["L"])
    aF = float(g["alphaF"])
    i = 0
    while f"in{i}" in g:
        kind, d, bc, nx, ny, nz = [int(v) for v in g[f"meta{i}"]]
        bt = [gpu_pkg.PERIODIC_SOLVE] * 3
        bt[d] = bc
        cfg = gpu_pkg.make_config((nx, ny, nz), L, bc_type=tuple(bt), alphaF=aF)
        op = gpu_pkg.Operator(cfg, d)
        lines = np.asarray(g[f"in{i}"], dtype=np.float64).reshape(-1)
        ref = np.asarray(g[f"out{i}"]).reshape(-1)
        assert lines.size == nx * ny * nz
        out = op.apply_host(kind, lines)
        assert rel_err(out, ref) <= TOL, (i, kind, d, bc, rel_err(out, ref))
        x = torch.from_numpy(lines).cuda()
        y = torch.empty_like(x)
        torch.cuda.synchronize()
        op.apply(kind, x.data_ptr(), y.data_ptr())
        torch.cuda.ExternalStream(op.stream()).synchronize()
        assert np.array_equal(y.cpu().numpy(), out), i
        op.close()
        i += 1
    assert i >= 20
