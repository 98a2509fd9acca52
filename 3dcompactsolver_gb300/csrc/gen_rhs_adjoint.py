"""Generate cs3d_rhs_adjoint.cuh: the pointwise right-hand side of one RK
stage and its vector-Jacobian product.

At a grid point the five right-hand sides R are a function of the primitives
U, V, W, T and of 44 derivative values (48 inputs, order NAMES).  It is the
sum the three sweep kernels form (x, y and z parts), i.e. the reference's
solveContinuity ... solveEnergy (CSolver_AWS.cpp:1246-1504) on periodic
boundaries without sponge.  The viscosity enters through
mu = mu_ref T^0.76 and amu = dmu/dT = 0.76 mu / T (CSolver_AWS.hpp:228-240).

The script writes two device functions:
  rhs_eval(in, muref, cpPr, R)      R[0..4] from the 48 inputs;
  rhs_vjp(in, l, muref, cpPr, out)  out[i] = d(l . R)/d(in[i]).
The T entry of rhs_vjp goes through mu and amu:
  d/dT = (dL/dmu) amu + (dL/damu) damu/dT,  damu/dT = -0.24 amu / T.

    python 3dcompactsolver_gb300/csrc/gen_rhs_adjoint.py
"""
import os
import re

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))

NAMES = ("U V W T Ux Vx Wx Tx Uxx Vxx Wxx Txx CEx F1x F2x F3x F4x "
         "Uy Vy Wy Ty Uyy Vyy Wyy Tyy Uxy Vxy CEy G1y G2y G3y G4y "
         "Uz Vz Wz Tz Uzz Vzz Wzz Tzz S Wxz Wyz CEz H1z H2z H3z H4z").split()


def rhs(g, mu, amu, cpPr):
    """The five right-hand sides as sympy expressions of the inputs g."""
    c43, c13, c23, half = sp.Rational(4, 3), sp.Rational(1, 3), sp.Rational(2, 3), sp.Rational(1, 2)
    U, V, W = g["U"], g["V"], g["W"]
    Ux, Uy, Uz = g["Ux"], g["Uy"], g["Uz"]
    Vx, Vy, Vz = g["Vx"], g["Vy"], g["Vz"]
    Wx, Wy, Wz = g["Wx"], g["Wy"], g["Wz"]
    MuX, MuY, MuZ = amu * g["Tx"], amu * g["Ty"], amu * g["Tz"]
    R0 = -(g["CEx"] + g["CEy"] + g["CEz"])
    R1 = (mu * (c43 * g["Uxx"]) - g["F1x"] + mu * (g["Uyy"] + c13 * g["Vxy"]) - g["G1y"]
          + mu * (g["Uzz"] + c13 * g["Wxz"]) - g["H1z"]
          + c43 * MuX * (Ux - half * Vy - half * Wz) + MuY * (Uy + Vx) + MuZ * (Wx + Uz))
    R2 = (mu * g["Vxx"] - g["F2x"] + mu * (c43 * g["Vyy"] + c13 * g["Uxy"]) - g["G2y"]
          + mu * (g["Vzz"] + c13 * g["Wyz"]) - g["H2z"]
          + c43 * MuY * (Vy - half * Ux - half * Wz) + MuX * (Uy + Vx) + MuZ * (Wy + Vz))
    R3 = (mu * g["Wxx"] - g["F3x"] + mu * g["Wyy"] - g["G3y"]
          + mu * (c43 * g["Wzz"] + c13 * g["S"]) - g["H3z"]
          + c43 * MuZ * (Wz - half * Ux - half * Vy) + MuX * (Wx + Uz) + MuY * (Wy + Vz))
    v1 = mu * (U * g["Uzz"] + V * g["Vzz"] + W * (c43 * g["Wzz"])
               + c13 * (U * g["Wxz"] + V * g["Wyz"] + W * g["S"])
               + c43 * (Ux * Ux + Vy * Vy + Wz * Wz)
               + (Uy * Uy + Uz * Uz + Vx * Vx + Vz * Vz + Wx * Wx + Wy * Wy)
               - c43 * (Ux * Vy + Ux * Wz + Vy * Wz) + 2 * (Uy * Vx + Uz * Wx + Vz * Wy))
    v2 = (c43 * (U * MuX * Ux + V * MuY * Vy + W * MuZ * Wz) - c23 * U * MuX * (Vy + Wz)
          - c23 * V * MuY * (Ux + Wz) - c23 * W * MuZ * (Ux + Vy) + U * MuY * (Uy + Vx)
          + U * MuZ * (Uz + Wx) + V * MuX * (Uy + Vx) + V * MuZ * (Vz + Wy) + W * MuX * (Uz + Wx)
          + W * MuY * (Vz + Wy))
    R4 = (cpPr * mu * g["Txx"] + mu * (U * (c43 * g["Uxx"]) + V * g["Vxx"] + W * g["Wxx"]) - g["F4x"]
          + cpPr * mu * g["Tyy"]
          + mu * (U * g["Uyy"] + V * (c43 * g["Vyy"]) + W * g["Wyy"] + c13 * (U * g["Vxy"] + V * g["Uxy"]))
          - g["G4y"]
          + cpPr * (MuX * g["Tx"] + MuY * g["Ty"] + MuZ * g["Tz"] + mu * g["Tzz"]) + v1 + v2 - g["H4z"])
    return [R0, R1, R2, R3, R4]


def build():
    # the temperature is the symbol Tt (T is the type name in the C++ output)
    g = {n: sp.Symbol("Tt" if n == "T" else n, real=True) for n in NAMES}
    mu, amu, cpPr = sp.symbols("mu amu cpPr", real=True)
    lam = sp.symbols("l0:5", real=True)
    R = rhs(g, mu, amu, cpPr)
    L = sum(l * r for l, r in zip(lam, R))
    grads = [sp.expand(sp.diff(L, g[n])) for n in NAMES]
    Lmu = sp.expand(sp.diff(L, mu))
    Lamu = sp.expand(sp.diff(L, amu))
    grads[NAMES.index("T")] = Lmu * amu - sp.Rational(24, 100) * Lamu * amu / g["T"]
    return R, grads


def _c(e):
    """C++ text of e in the work type T: squares as products, rational
    constants as T(...) so that the FP32 form stays in FP32."""
    s = sp.ccode(e)
    s = re.sub(r"pow\((\w+), 2\)", r"(\1*\1)", s)
    s = s.replace("1.0/3.0", "c13").replace("4.0/3.0", "c43").replace("2.0/3.0", "c23")
    s = re.sub(r"(?<![\w.])(\d+\.\d+/\d+\.\d+)", r"T(\1)", s)
    assert "pow(" not in s, s
    return s


def emit(path):
    R, grads = build()
    out = []
    out.append("// cs3d_rhs_adjoint.cuh -- GENERATED by gen_rhs_adjoint.py from the right-hand")
    out.append("// side of the stage sweeps; do not edit.  Inputs in[0..47] in the order")
    for k in range(0, len(NAMES), 16):
        out.append("//   " + " ".join(NAMES[k:k + 16]))
    out.append("#pragma once")
    out.append("namespace cs3d {")
    out.append("")
    out.append("constexpr int kRhsIn = %d;" % len(NAMES))
    for i, n in enumerate(NAMES):
        out.append("constexpr int kIn%s = %d;" % (n, i))
    out.append("")

    def prologue():
        lines = []
        for i, n in enumerate(NAMES):
            lines.append(f"    const T {'Tt' if n == 'T' else n} = in[{i}];")
        lines.append("    const T c13 = T(1.0 / 3.0), c43 = T(4.0 / 3.0), c23 = T(2.0 / 3.0);")
        lines.append("    const T mu = muref * visc_pow(Tt);")
        lines.append("    const T amu = (T)0.76 * mu / Tt;")
        lines.append("    (void)c23;")
        return lines

    # rhs_eval
    repl, red = sp.cse(R, symbols=sp.numbered_symbols("e"), optimizations="basic")
    out.append("// the five right-hand sides at one point")
    out.append("template <typename T>")
    out.append("__device__ __forceinline__ void rhs_eval(const T *in, T muref, T cpPr, T R[5]) {")
    out.extend(prologue())
    for s, e in repl:
        out.append(f"    const T {s} = {_c(e)};")
    for i, e in enumerate(red):
        out.append(f"    R[{i}] = {_c(e)};")
    out.append("}")
    out.append("")
    # rhs_vjp
    repl, red = sp.cse(grads, symbols=sp.numbered_symbols("t"), optimizations="basic")
    out.append("// out[i] = d(l . R)/d(in[i]) at one point")
    out.append("template <typename T>")
    out.append("__device__ __forceinline__ void rhs_vjp(const T *in, const T l[5], T muref, T cpPr, T *out) {")
    out.extend(prologue())
    out.append("    const T l0 = l[0], l1 = l[1], l2 = l[2], l3 = l[3], l4 = l[4];")
    for s, e in repl:
        out.append(f"    const T {s} = {_c(e)};")
    for i, e in enumerate(red):
        out.append(f"    out[{i}] = {_c(e)};")
    out.append("}")
    out.append("")
    out.append("}  // namespace cs3d")
    src = "\n".join(out) + "\n"
    with open(path, "w") as f:
        f.write(src)
    return src


if __name__ == "__main__":
    s = emit(os.path.join(HERE, "cs3d_rhs_adjoint.cuh"))
    print(f"wrote {len(s.splitlines())} lines")
