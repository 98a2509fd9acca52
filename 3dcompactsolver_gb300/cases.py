"""Initial conditions and configurations of the workloads.

Each function returns (config, (rho0, p0, U0, V0, W0)) with fields as numpy
arrays of shape (Nz, Ny, Nx) -- the XYZ layout k*Nx*Ny + j*Nx + i of the
reference (Macros.hpp:8).  The grid is the reference's: x_i = i*L/(N-1)
(Domain.hpp:31-41), with L = 2*pi*(1 - 1/N) on periodic cubes so that the
period is exactly 2*pi.
"""
import math

import numpy as np

from . import _abi

GAMMA = 1.4


def grid(N, L):
    """Coordinates of the reference's Domain (Domain.hpp:31-41)."""
    return np.array([(float(i) / (float(N) - 1.0)) * L for i in range(N)])


def _mesh(cfg):
    x = grid(cfg.Nx, cfg.Lx)
    y = grid(cfg.Ny, cfg.Ly)
    z = grid(cfg.Nz, cfg.Lz)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return X, Y, Z


def tgv(N, precision=_abi.FP64, rk=_abi.RK4, CFL=0.5, alphaF=0.49, filter_step=1, mach=0.1,
        re=1600.0, legacy_p=None, mu_ref=None):
    """Taylor-Green vortex on the periodic cube [0, 2pi)^3.

    rho0 = 1; u = sin x cos y cos z; v = -cos x sin y cos z; w = 0;
    p = p0 + (1/16)(cos 2x + cos 2y)(cos 2z + 2) with p0 = 1/(gamma Ma^2);
    mu_ref from Re = 1600 at T0 = p0/(rho0 R)
    (taylorgreen_vortex/taylorgreen_run128/3DCompact.cpp:120-131).

    legacy_p=100 reproduces the committed trajectories of
    taylorgreen_run{64,128} (p = 100 + ... without the 1/gamma).
    """
    L = 2.0 * math.pi - (2.0 * math.pi / float(N))
    R = (1.0 / GAMMA)
    if legacy_p is None:
        p0 = 1.0 / (GAMMA * mach * mach)
    else:
        p0 = float(legacy_p)
    T0 = p0 / (1.0 * R)
    if mu_ref is None:
        mu_ref = 1.0 / (re * T0 ** 0.76)
    cfg = _abi.make_config(N, L, alphaF=alphaF, mu_ref=mu_ref, CFL=CFL, filter_step=filter_step,
                           rk=rk, precision=precision)
    X, Y, Z = _mesh(cfg)
    u0 = 1.0
    U0 = u0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    V0 = -u0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    W0 = np.zeros_like(X)
    rho0 = np.ones_like(X)
    p = (p0 + (1.0 / 16.0) * (np.cos(X * 2.0) + np.cos(Y * 2.0)) * (np.cos(Z * 2.0) + 2.0))
    return cfg, (rho0, p, U0, V0, W0)


def hit(N, seed=0, mach_t=0.3, k0=8.0, precision=_abi.FP64, CFL=0.5, alphaF=0.49,
        filter_step=1, mu_ref=2.0e-4):
    """Decaying isotropic turbulence on [0, 2pi)^3: a solenoidal random-phase
    velocity with energy spectrum E(k) ~ (k/k0)^4 exp(-2 (k/k0)^2)
    (homogenous_turbulence/generate_init_hit.f90:277), scaled to turbulent
    Mach number sqrt(<u.u>)/c = mach_t; rho = 1, uniform p = 1/gamma (c = 1).
    Seeded with numpy default_rng(seed)."""
    L = 2.0 * math.pi - (2.0 * math.pi / float(N))
    cfg = _abi.make_config(N, L, alphaF=alphaF, mu_ref=mu_ref, CFL=CFL, filter_step=filter_step,
                           precision=precision)
    rng = np.random.default_rng(seed)
    k1 = np.fft.fftfreq(N, d=1.0 / N)
    KZ, KY, KX = np.meshgrid(k1, k1, k1, indexing="ij")
    K2 = KX * KX + KY * KY + KZ * KZ
    K = np.sqrt(K2)
    Ek = (K / k0) ** 4 * np.exp(-2.0 * (K / k0) ** 2)
    amp = np.zeros_like(K)
    nz = K > 0
    amp[nz] = np.sqrt(Ek[nz] / (4.0 * math.pi * K2[nz]))
    # no energy on the Nyquist planes: the real part of the inverse transform
    # would otherwise break the projection there
    nyq = (np.abs(KX) == N // 2) | (np.abs(KY) == N // 2) | (np.abs(KZ) == N // 2)
    amp[nyq] = 0.0
    comps = []
    for _ in range(3):
        ph = rng.uniform(0.0, 2.0 * math.pi, K.shape)
        comps.append(amp * (rng.standard_normal(K.shape) + 1j * rng.standard_normal(K.shape))
                     * np.exp(1j * ph))
    uh, vh, wh = comps
    # project onto divergence-free fields
    with np.errstate(invalid="ignore", divide="ignore"):
        dot = (KX * uh + KY * vh + KZ * wh) / np.where(nz, K2, 1.0)
    uh = uh - KX * dot
    vh = vh - KY * dot
    wh = wh - KZ * dot
    U0 = np.real(np.fft.ifftn(uh))
    V0 = np.real(np.fft.ifftn(vh))
    W0 = np.real(np.fft.ifftn(wh))
    urms = math.sqrt(float(np.mean(U0 * U0 + V0 * V0 + W0 * W0)))
    p0 = 1.0 / GAMMA
    c0 = math.sqrt(GAMMA * p0 / 1.0)
    scale = mach_t * c0 / urms
    U0, V0, W0 = U0 * scale, V0 * scale, W0 * scale
    rho0 = np.ones_like(U0)
    p = np.full_like(U0, p0)
    return cfg, (rho0, p, np.ascontiguousarray(U0), np.ascontiguousarray(V0),
                 np.ascontiguousarray(W0))


def shear_layer(Nx=256, Ny=128, Nz=42, seed=0, du=0.6, delta=2.0, h=0.5,
                sponge_frac=0.15, precision=_abi.FP32_MIXED, CFL=0.5, alphaF=0.495,
                filter_step=5, mu_ref=0.00375, perturb=0.1):
    """Temporal shear layer: x and z periodic, no-slip adiabatic walls at the
    y faces with a sponge over sponge_frac of Ly next to each wall, TVD-RK3.

    rho = 1 and p = 1/gamma (sound speed 1), the state of the reference's
    shear-layer case program (3DCompact.cpp:221-222) and the pressure its sponge
    relaxes toward (SpongeBC.hpp:56-58); U = (du/2) tanh((y - Ly/2)/delta),
    the profile of 3DCompact.cpp:223 with that program's du = 0.6 (:117), so the
    free streams run at Mach du/2 = 0.3.  mu_ref, alphaF and the filter
    interval are that program's (:61, :90-91).  Seeded random velocity
    perturbations of amplitude perturb*du/2 under the Gaussian window
    exp(-(y - Ly/2)^2) of 3DCompact.cpp:199-206.  The reference allows one BC
    kind per face, so the walls are ADIABATIC_WALL faces and the sponge is
    built as a band (SPONGE_BANDS).  With the filter applied every step (or
    CFL 0.8) the wall-adjacent points of this case grow until the solution
    blows up within a few hundred steps, in the reference as on the GPU."""
    Lx, Ly, Lz = h * (Nx - 1), h * (Ny - 1), h * (Nz - 1)
    cfg = _abi.make_config(
        (Nx, Ny, Nz), (Lx, Ly, Lz),
        bc_type=(_abi.PERIODIC_SOLVE, _abi.DIRICHLET_SOLVE, _abi.PERIODIC_SOLVE),
        bc_kind=(_abi.PERIODIC, _abi.PERIODIC, _abi.ADIABATIC_WALL, _abi.ADIABATIC_WALL,
                 _abi.PERIODIC, _abi.PERIODIC),
        alphaF=alphaF, mu_ref=mu_ref, CFL=CFL, filter_step=filter_step, rk=_abi.TVDRK3,
        precision=precision, sponge_mode=_abi.SPONGE_BANDS,
        sponge_frac=(0.0, 0.0, sponge_frac, sponge_frac, 0.0, 0.0))
    X, Y, Z = _mesh(cfg)
    p0 = 1.0 / GAMMA
    rng = np.random.default_rng(seed)
    win = np.exp(-((Y - Ly / 2.0) ** 2))
    amp = perturb * du / 2.0
    U0 = (du / 2.0) * np.tanh((Y - Ly / 2.0) / delta) + amp * win * rng.uniform(-1, 1, X.shape)
    V0 = amp * win * rng.uniform(-1, 1, X.shape)
    W0 = amp * win * rng.uniform(-1, 1, X.shape)
    rho0 = np.ones_like(X)
    p = np.full_like(X, p0)
    return cfg, (rho0, p, U0, V0, W0)


def wall_box(N=(20, 18, 16), seed=1, precision=_abi.FP64, rk=_abi.RK4, moving=False,
             sponge=False):
    """Small mixed-boundary case for parity tests: walls (or moving walls) at
    the x faces, sponge faces (reference sponge rule) at the z faces when
    sponge=True, y periodic; a smooth seeded perturbation of a uniform state."""
    Nx, Ny, Nz = N
    wall = _abi.MOVING_ADIABATIC_WALL if moving else _abi.ADIABATIC_WALL
    zk = _abi.SPONGE if sponge else _abi.PERIODIC
    zt = _abi.DIRICHLET_SOLVE if sponge else _abi.PERIODIC_SOLVE
    cfg = _abi.make_config(
        (Nx, Ny, Nz), (3.0, 2.5, 2.0),
        bc_type=(_abi.DIRICHLET_SOLVE, _abi.PERIODIC_SOLVE, zt),
        bc_kind=(wall, wall, _abi.PERIODIC, _abi.PERIODIC, zk, zk),
        alphaF=0.45, mu_ref=2.0e-3, CFL=0.4, filter_step=1, rk=rk, precision=precision,
        wall_vel=(0.05, -0.02, 0.03, 0.01, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0))
    X, Y, Z = _mesh(cfg)
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 2 * math.pi, 6)
    rho0 = 1.0 + 0.05 * np.sin(2 * math.pi * Y / 2.5 + ph[0]) * np.cos(X + ph[1])
    U0 = 0.1 * np.sin(2 * math.pi * Y / 2.5 + ph[2]) * np.sin(math.pi * X / 3.0)
    V0 = 0.1 * np.cos(Z * 2.0 + ph[3]) * np.sin(math.pi * X / 3.0)
    W0 = 0.05 * np.sin(X * 2.0 + ph[4]) * np.cos(Z + ph[5])
    p = (1.0 / GAMMA) * (1.0 + 0.02 * np.cos(X + Y + Z))
    return cfg, (rho0, p, U0, V0, W0)


def postprocess_grid():
    """The grid of the reference's post-processor (PostProcess.cpp:44-79):
    512 x 256 x 128 points over 345 x 172 x 86, x and z periodic, y solved
    with the wall closures (its faces there are SPONGE kinds, which only the
    solver uses; ADIABATIC_WALL here, so no sponge is built).  Returns
    (config, conserved state q of shape (5, Nz, Ny, Nx)) with a smooth
    analytic shear-layer-like state: a tanh profile in y with three-
    dimensional perturbations, rho and p varying."""
    cfg = _abi.make_config(
        (512, 256, 128), (345.0, 172.0, 86.0),
        bc_type=(_abi.PERIODIC_SOLVE, _abi.DIRICHLET_SOLVE, _abi.PERIODIC_SOLVE),
        bc_kind=(_abi.PERIODIC, _abi.PERIODIC, _abi.ADIABATIC_WALL, _abi.ADIABATIC_WALL,
                 _abi.PERIODIC, _abi.PERIODIC),
        alphaF=0.49, mu_ref=0.0035, CFL=0.5)
    X, Y, Z = _mesh(cfg)
    ax, ay, az = 2.0 * math.pi * X / cfg.Lx, Y / cfg.Ly, 2.0 * math.pi * Z / cfg.Lz
    env = np.exp(-((Y - cfg.Ly / 2.0) / 20.0) ** 2)
    rho = 1.0 + 0.1 * np.sin(2.0 * ax + 0.3) * np.cos(math.pi * ay) * np.cos(az)
    U = 0.5 * np.tanh((Y - cfg.Ly / 2.0) / 6.0) + 0.05 * env * np.sin(3.0 * ax) * np.sin(2.0 * az + 0.7)
    V = 0.03 * env * np.cos(5.0 * ax + 0.2) * np.cos(az) + 0.01 * np.sin(math.pi * ay) * np.sin(ax)
    W = 0.02 * (1.0 - (2.0 * ay - 1.0) ** 2) * np.sin(ax + 2.0 * az)
    p = (1.0 / GAMMA) * (1.0 + 0.01 * np.cos(ax) * np.cos(3.0 * math.pi * ay))
    rhoE = p / (GAMMA - 1.0) + 0.5 * rho * (U * U + V * V + W * W)
    q = np.stack([rho, rho * U, rho * V, rho * W, rhoE])
    return cfg, q
