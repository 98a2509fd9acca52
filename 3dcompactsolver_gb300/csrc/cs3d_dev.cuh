// cs3d_dev.cuh -- device-side data structures and helpers shared by the
// kernels and the host set-up code of the GB300 stage path.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cs3d {

// Maximum half width of a compact stencil's right-hand side: 2 for the
// derivatives (Derivatives.cpp:119-247), 4 for the filter (Filter.cpp:5-96).
constexpr int kMaxH = 4;
constexpr int kTaps = 2 * kMaxH + 1;

// One compact operator along one direction with its Thomas factors
// precomputed on the host.  The reference re-derives the factors, the
// Sherman-Morrison vector z and every division on every line of every call
// (Utils.cpp:4-46); here they are computed once per solver, so a line solve
// is one multiply-add forward and one multiply-add plus multiply backward.
//
//   forward   y_0 = r_0,  y_n = r_n - m_n y_{n-1}
//   backward  x_{N-1} = y_{N-1} iw_{N-1},  x_n = (y_n - c_n x_{n+1}) iw_n
//   cyclic    x_n -= f z_n,   f = (x_0 + bog x_{N-1}) inv_den   (f in FP64)
constexpr int kU = 4;  // rows per unrolled chunk of the line solves

template <typename T>
struct LineOp {
    const T *m;          // forward multipliers a_n / w_{n-1}        [N]
    const T *iw;         // reciprocals of the eliminated diagonal    [N]
    const T *c;          // super-diagonal                           [N]
    const T *z;          // Sherman-Morrison vector (periodic only)   [N]
    const T *mf;         // m from row H on: mf[k] = m[H+k]  (chunked forward loads)
    const T *cbk;        // c backwards: cbk[k] = c[N-2-k]   (chunked backward loads)
    const T *ibk;        // iw backwards: ibk[k] = iw[N-2-k]
    T taps[kTaps];       // interior RHS stencil, centred at kMaxH
    T btaps[2 * kMaxH][kTaps]; // the first H and last H rows, explicit
    int boff[2 * kMaxH]; // first column of each boundary row
    T scale;             // 1/h, 1/h^2 or 1
    // Rows [klo, khi) (kU <= klo, khi <= N-1) where m, iw and c equal km,
    // kiw, kc bit for bit in T: the factors of the Toeplitz interior converge
    // geometrically, and there the recurrences run on register constants.
    T km, kiw, kc;
    int klo, khi;
    double bog;          // beta / gamma of the cyclic correction
    double inv_den;      // 1 / (1 + z_0 + beta z_{N-1} / gamma)
    int N;
    int H;               // stencil half width (2 or 4)
    int periodic;
};

// Loads of operator coefficients (a few kB per operator, read by every line
// solve) through the read-only data path.
__device__ __forceinline__ float ldc(const float *p) { return __ldg(p); }
__device__ __forceinline__ double ldc(const double *p) { return __ldg(p); }

// Four consecutive coefficients from a 16-byte aligned address in one or two
// 128-bit loads.
__device__ __forceinline__ void load4(const float *p, float v[4]) {
    const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void load4(const double *p, double v[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p + 2));
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

// Conserved variables of one state (five FP64 arrays, XYZ layout).
struct Q5 {
    double *f[5];
};

// Division by a fixed d > 0 of numerators below 2^31:
// p / d = (umulhi(p, mul) + p) >> sh  (Granlund-Montgomery, round-up form).
struct FastDiv {
    unsigned mul;
    int sh;
};

inline FastDiv make_fastdiv(unsigned d) {
    FastDiv f;
    int sh = 0;
    while ((1ull << sh) < d) ++sh;
    f.sh = sh;
    f.mul = (unsigned)((((1ull << 32) * ((1ull << sh) - d)) / d) + 1ull);
    return f;
}

// Grid geometry.
struct Geom {
    int Nx, Ny, Nz;
    long long npts;
};

// ---------------------------------------------------------------------
// FP32 <-> FP64 conversion with integer instructions.  On this part the
// hardware conversions issue on the FP64 pipe, which runs at 1/64 of the
// FP32 rate; these take a handful of integer operations instead.  Both follow
// the IEEE-754 binary32/binary64 layouts: exact widening, and narrowing with
// round-to-nearest-even.  Subnormal results are flushed to signed zero and
// values beyond the binary32 range become infinity (NaN as well), which is
// immaterial for a flow state and its increments.
// ---------------------------------------------------------------------
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u;
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned man = ex == 0u ? 0u : (u & 0x7fffffu);
    const unsigned e64 = ex == 0u ? 0u : (ex == 0xffu ? 0x7ffu : ex + 896u);
    const unsigned hi = sign | (e64 << 20) | (man >> 3);
    const unsigned lo = man << 29;
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float narrow(double d) {
    const unsigned hi = (unsigned)__double2hiint(d);
    const unsigned lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int ex = (int)((hi >> 20) & 0x7ffu);
    const int e32 = ex - 896;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned bits = ((unsigned)e32 << 23) + m;
    bits += (rest > 0x10000000u) | ((rest == 0x10000000u) & (m & 1u));
    bits = e32 <= 0 ? 0u : (e32 >= 255 ? 0x7f800000u : bits);
    bits = bits > 0x7f800000u ? 0x7f800000u : bits;
    return __uint_as_float(sign | bits);
}

// Work-precision <-> FP64 without the FP64 conversion pipe.
template <typename T> __device__ __forceinline__ T to_work(double d);
template <> __device__ __forceinline__ double to_work<double>(double d) { return d; }
template <> __device__ __forceinline__ float to_work<float>(double d) { return narrow(d); }
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) { return widen(x); }

// Bit f set if point (i,j,k) lies on face f (X0,X1,Y0,Y1,Z0,Z1).
__device__ __forceinline__ int faces_of(const Geom &g, int i, int j, int k) {
    int f = 0;
    f |= (i == 0) << 0; f |= (i == g.Nx - 1) << 1;
    f |= (j == 0) << 2; f |= (j == g.Ny - 1) << 3;
    f |= (k == 0) << 4; f |= (k == g.Nz - 1) << 5;
    return f;
}

// T^0.76, the exponent of the viscosity law mu = mu_ref T^0.76 (IdealGas.hpp).
// FP32: exp2(0.76 log2 T) with the hardware log2 (absolute error about 2^-22,
// so about 1.5e-7 relative in the result: an FP32 rounding).  FP64, whose pipe issues two operations per SM and
// clock: y^25 = T^19 solved by one step of Halley's method (cubic
// convergence) from an FP32 estimate exp2(0.76 log2 T) (relative error below
// 2e-6), written as the correction y + y (c - a) / (13 a + 12 c) with
// a = y^25, c = T^19 by repeated squaring: about 20 FP64 operations and one
// division, within 2 ulp of the library pow on [1e-6, 1e6] (sampled against
// it: the cubic step leaves the estimate's error at ~1e-17).  Outside that
// range, and for NaN, the library pow.
__device__ __forceinline__ float visc_pow(float T) { return exp2f(0.76f * __log2f(T)); }
__device__ __forceinline__ double visc_pow(double T) {
    if (!(T > 1e-6 && T < 1e6)) return pow(T, 0.76);
    const double y = (double)exp2f(0.76f * log2f((float)T));
    const double t2 = T * T, t4 = t2 * t2, t8 = t4 * t4, t16 = t8 * t8;
    const double c = t16 * t2 * T;
    const double y2 = y * y, y4 = y2 * y2, y8 = y4 * y4, y16 = y8 * y8;
    const double a = y16 * y8 * y;
    return y + y * ((c - a) / (13.0 * a + 12.0 * c));
}

// Direction whose continuity derivative survives at a wall point: the
// reference applies the wall faces in the order X0,X1,Y0,Y1,Z0,Z1 and the
// last write wins (CSolver_AWS.cpp:1526-1609).  -1 if not on a wall.
__device__ __forceinline__ int wall_dir(int onwall) {
    return (onwall & 0x30) ? 2 : (onwall & 0x0c) ? 1 : (onwall & 0x03) ? 0 : -1;
}

}  // namespace cs3d
