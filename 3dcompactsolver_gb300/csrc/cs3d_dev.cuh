// cs3d_dev.cuh -- device-side data structures shared by the kernels and the
// host set-up code of the GB300 stage path.
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
//   cyclic    x_n -= f z_n,   f = (x_0 + bog x_{N-1}) inv_den   (in FP64)
template <typename T>
struct LineOp {
    const T *m;          // forward multipliers a_n / w_{n-1}        [N]
    const T *iw;         // reciprocals of the eliminated diagonal    [N]
    const T *c;          // super-diagonal                           [N]
    const T *z;          // Sherman-Morrison vector (periodic only)   [N]
    T taps[kTaps];       // interior RHS stencil, centred at kMaxH
    T btaps[2 * kMaxH][kTaps]; // the first H and last H rows, explicit
    int boff[2 * kMaxH]; // first column of each boundary row
    T scale;             // 1/h, 1/h^2 or 1
    double bog;          // beta / gamma of the cyclic correction
    double inv_den;      // 1 / (1 + z_0 + beta z_{N-1} / gamma)
    int N;
    int H;               // stencil half width (2 or 4)
    int periodic;
};

// Conserved variables of one state (five FP64 arrays, XYZ layout).
struct Q5 {
    double *f[5];
};

// Grid geometry of a sweep direction.
struct Geom {
    int Nx, Ny, Nz;
    long long npts;
};

}  // namespace cs3d
