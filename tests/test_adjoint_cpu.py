"""CPU checks of the pieces of the discrete adjoint.

1. On periodic grids the compact operators of the oracle satisfy
   D1^T = -D1, D2^T = D2, F^T = F (the identity the transposed line solves
   use); on wall (Dirichlet-closure) lines they do not.
2. The generated pointwise right-hand side (cs3d_rhs_adjoint.cuh, compiled
   here with g++) equals a restatement of the sweep kernels' formulas, and
   its vector-Jacobian product equals central differences of it.
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "3dcompactsolver_gb300", "csrc")


def _dense(oracle, kind, bc, N, dh, alphaF=0.49):
    eye = np.eye(N)
    return oracle.line_op_port(kind, bc, N, dh, alphaF, eye).T


@pytest.mark.parametrize("N", [8, 17, 32, 64])
def test_periodic_operators_transpose(oracle, N):
    dh = 2.0 * math.pi / N
    D1 = _dense(oracle, 1, 0, N, dh)
    D2 = _dense(oracle, 2, 0, N, dh)
    F = _dense(oracle, 3, 0, N, dh)
    assert np.abs(D1.T + D1).max() <= 1e-13 * np.abs(D1).max()
    assert np.abs(D2.T - D2).max() <= 1e-13 * np.abs(D2).max()
    assert np.abs(F.T - F).max() <= 1e-13 * np.abs(F).max()


def test_wall_operators_are_not_self_adjoint(oracle):
    N, dh = 32, 0.1
    D1 = _dense(oracle, 1, 1, N, dh)
    assert np.abs(D1.T + D1).max() > 1e-3 * np.abs(D1).max()


@pytest.fixture(scope="module")
def rhs_lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("rhs")
    src = d / "rhs.cpp"
    src.write_text(
        "#define __device__\n#define __forceinline__ inline\n#include <cmath>\nusing std::pow;\n"
        # the viscosity law's power as the host library computes it (the
        # device's visc_pow agrees with it to 2 ulp)
        "namespace cs3d { inline double visc_pow(double T) { return std::pow(T, 0.76); } }\n"
        '#include "cs3d_rhs_adjoint.cuh"\n'
        'extern "C" void eval(const double *in, double mr, double cp, double *R) '
        "{ cs3d::rhs_eval<double>(in, mr, cp, R); }\n"
        'extern "C" void vjp(const double *in, const double *l, double mr, double cp, double *o) '
        "{ cs3d::rhs_vjp<double>(in, l, mr, cp, o); }\n")
    so = d / "rhs.so"
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(so)],
                   check=True)
    L = ctypes.CDLL(str(so))
    dp = ctypes.POINTER(ctypes.c_double)
    L.eval.argtypes = [dp, ctypes.c_double, ctypes.c_double, dp]
    L.vjp.argtypes = [dp, dp, ctypes.c_double, ctypes.c_double, dp]
    return L


NAMES = ("U V W T Ux Vx Wx Tx Uxx Vxx Wxx Txx CEx F1x F2x F3x F4x "
         "Uy Vy Wy Ty Uyy Vyy Wyy Tyy Uxy Vxy CEy G1y G2y G3y G4y "
         "Uz Vz Wz Tz Uzz Vzz Wzz Tzz S Wxz Wyz CEz H1z H2z H3z H4z").split()


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _eval(L, x, mr, cp):
    R = np.zeros(5)
    L.eval(_p(np.ascontiguousarray(x)), mr, cp, _p(R))
    return R


def _sweeps(x, mr, cp):
    """The x, y and z consume phases of the sweep kernels, term by term."""
    g = dict(zip(NAMES, x))
    c43, c13, c23 = 4.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0
    U, V, W, T = g["U"], g["V"], g["W"], g["T"]
    mu = mr * T ** 0.76
    amu = 0.76 * mu / T
    R = np.zeros(5)
    R[0] = -g["CEx"]
    R[1] = mu * (c43 * g["Uxx"]) - g["F1x"]
    R[2] = mu * g["Vxx"] - g["F2x"]
    R[3] = mu * g["Wxx"] - g["F3x"]
    R[4] = cp * mu * g["Txx"] + mu * (U * (c43 * g["Uxx"]) + V * g["Vxx"] + W * g["Wxx"]) - g["F4x"]
    R[0] += -g["CEy"]
    R[1] += mu * (g["Uyy"] + c13 * g["Vxy"]) - g["G1y"]
    R[2] += mu * (c43 * g["Vyy"] + c13 * g["Uxy"]) - g["G2y"]
    R[3] += mu * g["Wyy"] - g["G3y"]
    R[4] += (cp * mu * g["Tyy"] + mu * (U * g["Uyy"] + V * (c43 * g["Vyy"]) + W * g["Wyy"]
                                        + c13 * (U * g["Vxy"] + V * g["Uxy"])) - g["G4y"])
    Ux, Vx, Wx, Tx = g["Ux"], g["Vx"], g["Wx"], g["Tx"]
    Uy, Vy, Wy, Ty = g["Uy"], g["Vy"], g["Wy"], g["Ty"]
    Uz, Vz, Wz, Tz = g["Uz"], g["Vz"], g["Wz"], g["Tz"]
    Uzz, Vzz, Wzz, Tzz, S = g["Uzz"], g["Vzz"], g["Wzz"], g["Tzz"], g["S"]
    Wxz, Wyz = g["Wxz"], g["Wyz"]
    MuX, MuY, MuZ = amu * Tx, amu * Ty, amu * Tz
    R[1] += (mu * (Uzz + c13 * Wxz) - g["H1z"] + c43 * MuX * (Ux - 0.5 * Vy - 0.5 * Wz)
             + MuY * (Uy + Vx) + MuZ * (Wx + Uz))
    R[2] += (mu * (Vzz + c13 * Wyz) - g["H2z"] + c43 * MuY * (Vy - 0.5 * Ux - 0.5 * Wz)
             + MuX * (Uy + Vx) + MuZ * (Wy + Vz))
    R[3] += (mu * (c43 * Wzz + c13 * S) - g["H3z"] + c43 * MuZ * (Wz - 0.5 * Ux - 0.5 * Vy)
             + MuX * (Wx + Uz) + MuY * (Wy + Vz))
    q2s = Ux * Ux + Vy * Vy + Wz * Wz
    sq = Uy * Uy + Uz * Uz + Vx * Vx + Vz * Vz + Wx * Wx + Wy * Wy
    cr = Ux * Vy + Ux * Wz + Vy * Wz
    sh = Uy * Vx + Uz * Wx + Vz * Wy
    v1 = mu * (U * Uzz + V * Vzz + W * (c43 * Wzz) + c13 * (U * Wxz + V * Wyz + W * S) + c43 * q2s + sq
               - c43 * cr + 2.0 * sh)
    v2 = (c43 * (U * MuX * Ux + V * MuY * Vy + W * MuZ * Wz) - c23 * U * MuX * (Vy + Wz)
          - c23 * V * MuY * (Ux + Wz) - c23 * W * MuZ * (Ux + Vy) + U * MuY * (Uy + Vx) + U * MuZ * (Uz + Wx)
          + V * MuX * (Uy + Vx) + V * MuZ * (Vz + Wy) + W * MuX * (Uz + Wx) + W * MuY * (Vz + Wy))
    R[4] += cp * (MuX * Tx + MuY * Ty + MuZ * Tz + mu * Tzz) + v1 + v2 - g["H4z"]
    R[0] += -g["CEz"]
    return R


def _inputs(rng):
    x = rng.uniform(-1.0, 1.0, 48)
    x[3] = rng.uniform(50.0, 150.0)  # temperature
    return x


def test_generated_rhs_matches_sweeps(rhs_lib):
    rng = np.random.default_rng(3)
    for _ in range(20):
        x = _inputs(rng)
        mr, cp = 1e-3, 3.5 / 0.7
        a = _eval(rhs_lib, x, mr, cp)
        b = _sweeps(x, mr, cp)
        assert np.abs(a - b).max() <= 1e-13 * max(np.abs(b).max(), 1.0), (a, b)


def test_generated_vjp_matches_differences(rhs_lib):
    rng = np.random.default_rng(4)
    mr, cp = 2e-3, 5.0
    for _ in range(10):
        x = _inputs(rng)
        lam = rng.standard_normal(5)
        out = np.zeros(48)
        rhs_lib.vjp(_p(x), _p(lam), mr, cp, _p(out))
        for i in range(48):
            # R is at most quadratic along any one input but T, so a wide
            # central difference is exact there up to rounding; along T the
            # truncation error is (h/T)^2
            h = 1e-4 * x[i] if i == 3 else 1e-2
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            fd = (lam @ _eval(rhs_lib, xp, mr, cp) - lam @ _eval(rhs_lib, xm, mr, cp)) / (2 * h)
            assert abs(out[i] - fd) <= 1e-8 * max(abs(fd), 1e-2), (NAMES[i], out[i], fd)


def test_generated_header_is_current(tmp_path):
    """The committed header is what the generator writes."""
    pytest.importorskip("sympy")
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen", os.path.join(CSRC, "gen_rhs_adjoint.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    out = tmp_path / "h.cuh"
    gen.emit(str(out))
    with open(os.path.join(CSRC, "cs3d_rhs_adjoint.cuh")) as f:
        assert out.read_text() == f.read()
