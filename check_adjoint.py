"""Check the discrete adjoint on the Taylor-Green vortex.

    python check_adjoint.py --N 128 --steps 200 --dirs 16 [--rk tvdrk3]

J = volume-averaged kinetic energy after `steps` RK4 (or TVD-RK3) steps at a
fixed time step (the CFL 0.5 step of the initial state).  The gradient dJ/d(U0, V0, W0)
from cs3d_adjoint_backward (FP64 handle, and FP32-mixed handle) is compared
on `dirs` seeded random directions with central differences of the FP64
forward, and the mixed gradient with the FP64 gradient; each direction's
conditioning |g.d| / (|g| |d|) is reported with it.  Prints one JSON
line: per-direction relative errors, their maxima, and the time of the record
(forward with checkpoints) and of the backward sweep.
"""
import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
cs3d = importlib.import_module("3dcompactsolver_gb300")
cases = importlib.import_module("3dcompactsolver_gb300.cases")


def smooth_direction(rng, N, kmax=6.0):
    """A seeded random field with energy at wavenumbers up to about kmax."""
    k = np.fft.fftfreq(N, d=1.0 / N)
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    filt = np.exp(-(KX ** 2 + KY ** 2 + KZ ** 2) / (kmax * kmax))
    f = np.real(np.fft.ifftn(np.fft.fftn(rng.standard_normal((N, N, N))) * filt))
    return f / np.sqrt(np.mean(f * f))


def mean_ke(q):
    return float(np.mean(0.5 * (q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]))


def forward_J(cfg, ic, steps):
    s = cs3d.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.run(steps)
    J = mean_ke(s.conserved())
    s.close()
    return J


def adjoint(cfg, ic, steps, every):
    s = cs3d.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.sync()
    t0 = time.perf_counter()
    s.adjoint_record(steps, every)
    s.sync()
    t1 = time.perf_counter()
    grad, J = s.adjoint_backward(cs3d.ADJ_KE_MEAN)
    t2 = time.perf_counter()
    s.close()
    return grad, J, t1 - t0, t2 - t1


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--dirs", type=int, default=16)
    ap.add_argument("--every", type=int, default=0)
    ap.add_argument("--eps", type=float, default=1e-5)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--rk", default="rk4", choices=["rk4", "tvdrk3"])
    args = ap.parse_args(argv)
    N, steps = args.N, args.steps
    rk = cs3d.TVDRK3_KIND if args.rk == "tvdrk3" else cs3d.RK4_KIND
    cfg, ic = cases.tgv(N, rk=rk)
    s = cs3d.Solver(cfg)
    s.set_initial_conditions(*ic)
    s.step()
    dt = s.scalars()[0]
    s.close()
    cfg.dt_fixed = dt
    rho0, p0, U0, V0, W0 = ic
    out = {"workload": f"tgv{N}", "rk": args.rk, "steps": steps, "dt_fixed": dt, "dirs": args.dirs,
           "eps": args.eps}
    g64, J64, trec, tback = adjoint(cfg, ic, steps, args.every)
    out["J"] = J64
    out["fp64"] = {"record_s": trec, "backward_s": tback,
                   "backward_mpts_per_step_s": N ** 3 * steps / tback / 1e6}
    gU, gV, gW = cs3d.ic_velocity_gradient(g64, rho0, U0, V0, W0)
    gm = None
    if not args.no_mixed:
        cfg_m, _ = cases.tgv(N, precision=cs3d.FP32_MIXED, rk=rk)
        cfg_m.dt_fixed = dt
        gm_q, Jm, trec_m, tback_m = adjoint(cfg_m, ic, steps, args.every)
        out["mixed"] = {"record_s": trec_m, "backward_s": tback_m, "J": Jm,
                        "backward_mpts_per_step_s": N ** 3 * steps / tback_m / 1e6}
        gm = cs3d.ic_velocity_gradient(gm_q, rho0, U0, V0, W0)
        num = np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(gm, (gU, gV, gW))))
        den = np.sqrt(sum(np.sum(b * b) for b in (gU, gV, gW)))
        out["mixed"]["grad_rel_l2_vs_fp64"] = float(num / den)
    rng = np.random.default_rng(args.seed)
    e64, em, cond = [], [], []
    gnorm = np.sqrt(sum(np.sum(b * b) for b in (gU, gV, gW)))
    t0 = time.perf_counter()
    for d in range(args.dirs):
        dU, dV, dW = (smooth_direction(rng, N) for _ in range(3))
        eps = args.eps
        Jp = forward_J(cfg, (rho0, p0, U0 + eps * dU, V0 + eps * dV, W0 + eps * dW), steps)
        Jm_ = forward_J(cfg, (rho0, p0, U0 - eps * dU, V0 - eps * dV, W0 - eps * dW), steps)
        fd = (Jp - Jm_) / (2 * eps)
        a64 = float(np.sum(gU * dU + gV * dV + gW * dW))
        e64.append(abs(a64 - fd) / abs(fd))
        # |g.d| / (|g| |d|): how well the direction determines g.d
        cond.append(abs(a64) / (gnorm * np.sqrt(np.sum(dU * dU) + np.sum(dV * dV) + np.sum(dW * dW))))
        if gm is not None:
            am = float(np.sum(gm[0] * dU + gm[1] * dV + gm[2] * dW))
            em.append(abs(am - fd) / abs(fd))
    out["fd_s"] = time.perf_counter() - t0
    out["fp64"]["fd_rel_err"] = e64
    out["fp64"]["fd_rel_err_max"] = max(e64)
    out["direction_conditioning"] = cond
    if gm is not None:
        out["mixed"]["fd_rel_err"] = em
        out["mixed"]["fd_rel_err_max"] = max(em)
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
