"""The discrete adjoint through the C ABI, against finite differences of the
FP64 forward (the same product path, fixed time step).

* R(q) evaluated from the stored pointwise inputs equals the fused stage's
  right-hand side (dq/dt of stage 1);
* <w, J v> by central differences of R equals <J^T w, v> (adjoint test of
  one stage, random noise in every field);
* the gradient of the final mean kinetic energy with respect to the initial
  velocity equals central differences of the forward on seeded random
  directions, filtered every step and every second step;
* the checkpoint interval does not change the gradient, and the solver is
  back at its recorded final state afterwards;
* the backward from the tapes kept by the segment replay equals, bit for
  bit, the one that recomputes each step's stages;
* the same for TVD-RK3 steps (differences, segment storage, the mixed
  adjoint against the FP64 one).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tgv_fixed_dt(gpu_pkg, cases, N, **kw):
    cfg, ic = cases.tgv(N, **kw)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.step()
    dt = s.scalars()[0]
    s.close()
    cfg.dt_fixed = dt
    return cfg, ic


def _state(gpu_pkg, cases, N=16, steps=3, seed=0):
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N)
    rng = np.random.default_rng(seed)
    rho0, p0, U0, V0, W0 = ic
    W0 = 0.1 * np.sin(np.arange(N)[:, None, None] * 2 * np.pi / N + rng.uniform(0, 6.28)) * np.ones_like(U0)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(rho0, p0 * (1 + 0.01 * rng.standard_normal(U0.shape)), U0, V0, W0)
    s.run(steps)
    return s, cfg, s.conserved()


def test_rhs_eval_matches_fused_stage(gpu_pkg, cases):
    s, cfg, q = _state(gpu_pkg, cases)
    R = s.rhs_eval(q)
    s.set_option(gpu_pkg.OPT_STORE_INCREMENTS, 1)
    s.pre_step()
    s.sub_step(1, 0)
    dt = s.scalars()[0]
    dq = np.stack([s.get(15 + f) for f in range(5)])
    for f in range(5):
        scale = np.abs(dq[f]).max()
        assert np.abs(dt * R[f] - dq[f]).max() <= 1e-11 * scale, f


def test_rhs_vjp_adjoint_identity(gpu_pkg, cases):
    s, cfg, q = _state(gpu_pkg, cases, seed=1)
    rng = np.random.default_rng(7)
    scale = np.abs(q).reshape(5, -1).max(axis=1)[:, None, None, None]
    v = 1e-2 * scale * rng.standard_normal(q.shape)
    w = rng.standard_normal(q.shape)
    eps = 1e-4
    jv = (s.rhs_eval(q + eps * v) - s.rhs_eval(q - eps * v)) / (2 * eps)
    lhs = float(np.sum(w * jv))
    rhs = float(np.sum(s.rhs_vjp(q, w) * v))
    assert abs(lhs - rhs) <= 1e-7 * abs(lhs), (lhs, rhs)


def _mean_ke(q):
    return float(np.mean(0.5 * (q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]))


def _forward_J(gpu_pkg, cfg, ic, nsteps):
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(nsteps)
    J = _mean_ke(s.conserved())
    s.close()
    return J


@pytest.mark.parametrize("filter_step,every,rk", [(1, 4, "rk4"), (2, 0, "rk4"), (2, 4, "tvdrk3")])
def test_adjoint_matches_finite_differences(gpu_pkg, cases, filter_step, every, rk):
    N, nsteps = 16, 6
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N, filter_step=filter_step,
                            rk=gpu_pkg.TVDRK3_KIND if rk == "tvdrk3" else gpu_pkg.RK4_KIND)
    rho0, p0, U0, V0, W0 = ic
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.adjoint_record(nsteps, every)
    qN = s.conserved()
    grad, J = s.adjoint_backward(gpu_pkg.ADJ_KE_MEAN)
    assert abs(J - _mean_ke(qN)) <= 1e-14 * J
    gU, gV, gW = gpu_pkg.ic_velocity_gradient(grad, rho0, U0, V0, W0)
    rng = np.random.default_rng(100 + filter_step)
    eps = 1e-5
    for d in range(3):
        dU, dV, dW = (rng.standard_normal(U0.shape) for _ in range(3))
        adj = float(np.sum(gU * dU + gV * dV + gW * dW))
        Jp = _forward_J(gpu_pkg, cfg, (rho0, p0, U0 + eps * dU, V0 + eps * dV, W0 + eps * dW), nsteps)
        Jm = _forward_J(gpu_pkg, cfg, (rho0, p0, U0 - eps * dU, V0 - eps * dV, W0 - eps * dW), nsteps)
        fd = (Jp - Jm) / (2 * eps)
        assert abs(adj - fd) <= 1e-6 * abs(fd), (d, adj, fd)


def test_adjoint_checkpointing_and_restore(gpu_pkg, cases):
    N, nsteps = 16, 5
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N)
    grads = []
    for every in (1, 2, 5):
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.adjoint_record(nsteps, every)
        qN = s.conserved()
        g, _ = s.adjoint_backward(gpu_pkg.ADJ_KE_MEAN)
        grads.append(g)
        assert np.array_equal(s.conserved(), qN)
        assert s.scalars()[2] == nsteps
        s.step()
        ref = gpu_pkg.Solver(cfg)
        ref.set_initial_conditions(*ic)
        ref.run(nsteps + 1)
        assert np.array_equal(s.conserved(), ref.conserved())
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


@pytest.mark.parametrize("mixed,rk", [(False, "rk4"), (True, "rk4"), (False, "tvdrk3"), (True, "tvdrk3")])
def test_adjoint_segment_storage_equals_recompute(gpu_pkg, cases, mixed, rk):
    """The backward from the tapes and stage inputs kept by the segment replay
    gives the same bits as the per-step recompute of each step's stages
    (OPT_ADJ_RECOMPUTE): 7 steps in segments of 3 (one ragged), filter every
    second step, FP64 and FP32-mixed handles, RK4 and TVD-RK3."""
    N, nsteps = 16, 7
    rkc = gpu_pkg.TVDRK3_KIND if rk == "tvdrk3" else gpu_pkg.RK4_KIND
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N, filter_step=2, rk=rkc)
    if mixed:
        dt = cfg.dt_fixed
        cfg, _ = cases.tgv(N, filter_step=2, precision=gpu_pkg.FP32_MIXED, rk=rkc)
        cfg.dt_fixed = dt
    out = []
    for recompute in (0, 1):
        s = gpu_pkg.Solver(cfg)
        s.set_initial_conditions(*ic)
        s.set_option(gpu_pkg.OPT_ADJ_RECOMPUTE, recompute)
        s.adjoint_record(nsteps, 3)
        qN = s.conserved()
        g, J = s.adjoint_backward(gpu_pkg.ADJ_KE_MEAN)
        assert np.array_equal(s.conserved(), qN)
        out.append((g, J))
        s.close()
    assert np.isfinite(out[0][0]).all() and np.abs(out[0][0]).max() > 0
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_adjoint_user_seed_is_linear(gpu_pkg, cases):
    N, nsteps = 12, 3
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.adjoint_record(nsteps)
    rng = np.random.default_rng(5)
    a = rng.standard_normal((5, N, N, N))
    b = rng.standard_normal((5, N, N, N))
    ga, _ = s.adjoint_backward(gpu_pkg.ADJ_SEED, a)
    gb, _ = s.adjoint_backward(gpu_pkg.ADJ_SEED, b)
    gab, _ = s.adjoint_backward(gpu_pkg.ADJ_SEED, 2.0 * a - b)
    assert np.abs(gab - (2.0 * ga - gb)).max() <= 1e-10 * np.abs(gab).max()


def test_adjoint_rejects_unsupported(gpu_pkg, cases):
    cfg, ic = cases.tgv(16)  # no fixed time step
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    with pytest.raises(gpu_pkg.CS3DError) as e:
        s.adjoint_record(2)
    assert e.value.code == 6
    cfg, ic = cases.wall_box()
    cfg.dt_fixed = 1e-3
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    with pytest.raises(gpu_pkg.CS3DError) as e:
        s.adjoint_record(2)
    assert e.value.code == 6


def _smooth(rng, N, kmax=4.0):
    """A seeded random field with its energy at wavenumbers up to about kmax."""
    k = np.fft.fftfreq(N, d=1.0 / N)
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    f = np.real(np.fft.ifftn(np.fft.fftn(rng.standard_normal((N, N, N))) *
                             np.exp(-(KX ** 2 + KY ** 2 + KZ ** 2) / (kmax * kmax))))
    return f / np.sqrt(np.mean(f * f))


def test_mixed_adjoint_tracks_fp64(gpu_pkg, cases):
    """The FP32-mixed adjoint (FP32 stage Jacobians at the mixed forward's
    stage inputs, FP64 adjoint state and RK combination) within 1e-6, the
    bound the adjoint is held to (TGV 24^3, 8 RK4 steps, filter every step):

    * its velocity gradient against the FP64 adjoint's, relative L2 norm;
    * its directional derivatives against central differences of the FP64
      forward on seeded smooth directions.  A directional derivative g.d is
      only as well determined as |g||d| / |g.d| allows (a direction nearly
      orthogonal to the gradient amplifies every rounding error, the FP64
      adjoint's too), so directions with |g.d| < |g||d| / 100 are drawn again;
      at least three directions are checked."""
    N, nsteps = 24, 8
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N)
    cfg_m, _ = cases.tgv(N, precision=gpu_pkg.FP32_MIXED)
    cfg_m.dt_fixed = cfg.dt_fixed
    grads = []
    for c in (cfg, cfg_m):
        s = gpu_pkg.Solver(c)
        s.set_initial_conditions(*ic)
        s.adjoint_record(nsteps, 3)
        g, _ = s.adjoint_backward(gpu_pkg.ADJ_KE_MEAN)
        grads.append(gpu_pkg.ic_velocity_gradient(g, ic[0], ic[2], ic[3], ic[4]))
        s.close()
    num = np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(grads[1], grads[0])))
    gnorm = np.sqrt(sum(np.sum(b * b) for b in grads[0]))
    assert num / gnorm <= 1e-6, num / gnorm
    rng = np.random.default_rng(11)
    rho0, p0, U0, V0, W0 = ic
    eps = 1e-5
    checked = 0
    for _ in range(12):
        dU, dV, dW = (_smooth(rng, N) for _ in range(3))
        a64 = float(np.sum(grads[0][0] * dU + grads[0][1] * dV + grads[0][2] * dW))
        dnorm = np.sqrt(np.sum(dU * dU) + np.sum(dV * dV) + np.sum(dW * dW))
        if abs(a64) < gnorm * dnorm / 100:
            continue
        fd = (_forward_J(gpu_pkg, cfg, (rho0, p0, U0 + eps * dU, V0 + eps * dV, W0 + eps * dW), nsteps)
              - _forward_J(gpu_pkg, cfg, (rho0, p0, U0 - eps * dU, V0 - eps * dV, W0 - eps * dW), nsteps)) / (2 * eps)
        am = float(np.sum(grads[1][0] * dU + grads[1][1] * dV + grads[1][2] * dW))
        assert abs(a64 - fd) <= 1e-8 * abs(fd), (a64, fd)
        assert abs(am - fd) <= 1e-6 * abs(fd), (am, fd, abs(am - fd) / abs(fd))
        checked += 1
        if checked == 3:
            break
    assert checked == 3


def test_mixed_rhs_vjp_tracks_fp64(gpu_pkg, cases):
    s, cfg, q = _state(gpu_pkg, cases, seed=2)
    cfg_m, _ = cases.tgv(16, precision=gpu_pkg.FP32_MIXED)
    m = gpu_pkg.Solver(cfg_m)
    m.set_initial_conditions(*[np.ones((16, 16, 16))] * 2 + [np.zeros((16, 16, 16))] * 3)
    rng = np.random.default_rng(3)
    w = rng.standard_normal(q.shape)
    a = s.rhs_vjp(q, w)
    b = m.rhs_vjp(q, w)
    for f in range(5):
        assert np.abs(a[f] - b[f]).max() <= 2e-3 * np.abs(a[f]).max(), f


def test_mixed_tvdrk3_adjoint_tracks_fp64(gpu_pkg, cases):
    """TVD-RK3 (TVDRK3.hpp:38-96): the FP32-mixed adjoint's velocity gradient
    within 1e-6 of the FP64 adjoint's in relative L2 (TGV 24^3, 8 steps,
    filter every second step)."""
    N, nsteps = 24, 8
    cfg, ic = _tgv_fixed_dt(gpu_pkg, cases, N, filter_step=2, rk=gpu_pkg.TVDRK3_KIND)
    cfg_m, _ = cases.tgv(N, precision=gpu_pkg.FP32_MIXED, filter_step=2, rk=gpu_pkg.TVDRK3_KIND)
    cfg_m.dt_fixed = cfg.dt_fixed
    grads = []
    for c in (cfg, cfg_m):
        s = gpu_pkg.Solver(c)
        s.set_initial_conditions(*ic)
        s.adjoint_record(nsteps, 3)
        g, _ = s.adjoint_backward(gpu_pkg.ADJ_KE_MEAN)
        grads.append(gpu_pkg.ic_velocity_gradient(g, ic[0], ic[2], ic[3], ic[4]))
        s.close()
    num = np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(grads[1], grads[0])))
    gnorm = np.sqrt(sum(np.sum(b * b) for b in grads[0]))
    assert gnorm > 0 and num / gnorm <= 1e-6, num / gnorm
