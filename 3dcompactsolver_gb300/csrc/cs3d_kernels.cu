// cs3d_kernels.cu -- sm_103a kernels of the per-RK-stage path.
//
// One stage is three fused directional sweeps.  Each sweep kernel takes a
// pencil tile -- L complete grid lines along the sweep direction -- stages the
// inputs of every line solve of that direction in shared memory, solves all of
// them (one thread per line and operator, Thomas with precomputed factors, in
// place), then consumes the derivatives point by point:
//
//   sweep x : primitives, Euler x-fluxes, 13 x-solves; writes Ux,Vx,Wx,Tx,
//             mu, mu'(T) and the linear x-part of the five right-hand sides
//   sweep y : 15 y-solves (incl. the cross derivatives Uxy, Vxy); writes
//             Uy,Vy,Wy,Ty and adds the linear y-part
//   sweep z : 16 z-solves (incl. d/dz of Ux+Vy, Wx, Wy), the nonlinear viscous
//             terms, sponge sources, dt, the wall/sponge increment fix-up and
//             the RK4 / TVD-RK3 update of the conserved state
//
// The reference instead stores ~48 derivative fields and makes ~54 layout
// transposes per stage (CSolver_AWS.cpp:829-1243).  Lines along y and z are
// read in place in the XYZ layout: a tile is L consecutive x-columns, so every
// global access is a contiguous row segment.  x-lines are transposed into
// shared memory on load.
//
// T is the work precision: double for the plain form, float for the mixed
// form.  The conserved state (q1, qk, q2) is always FP64.
#include <cstdio>
#include <cmath>
#include "cs3d_dev.cuh"
#include "cs3d_kernels.cuh"

namespace cs3d {

// ---------------------------------------------------------------------
// line solve
// ---------------------------------------------------------------------

// Apply operator op to one line: reads the line from src (stride P), writes
// the uncorrected solution to dst (stride P).  src may equal dst: the forward
// pass reads position n+H+1 before writing position n, and the first and last
// H rows are evaluated before any write.  Returns the Sherman-Morrison factor
// (0 for walls); the caller applies x_n - f z_n when it reads the result.
template <typename T, int H>
__device__ __forceinline__ double line_solve(const T *src, T *dst, int P, const LineOp<T> &op) {
    const int N = op.N;
    const T *__restrict__ m = op.m;
    const T *__restrict__ iw = op.iw;
    const T *__restrict__ c = op.c;
    T pre[2 * H];
#pragma unroll
    for (int b = 0; b < 2 * H; ++b) {
        int col = op.boff[b];
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < kTaps; ++k) {
            int cc = col + k;
            cc = cc < 0 ? cc + N : (cc >= N ? cc - N : cc);
            acc = fma(op.btaps[b][k], src[cc * P], acc);
        }
        pre[b] = acc * op.scale;
    }
    T w[2 * H + 1];
#pragma unroll
    for (int k = 0; k < H; ++k) w[k] = T(0);
#pragma unroll
    for (int k = H; k < 2 * H + 1; ++k) w[k] = src[(k - H) * P];
    T taps[2 * H + 1];
#pragma unroll
    for (int k = 0; k < 2 * H + 1; ++k) taps[k] = op.taps[kMaxH - H + k];
    const T scale = op.scale;

    T y = pre[0];
    // rows 0..H-1
#pragma unroll
    for (int n = 0; n < H; ++n) {
        if (n > 0) y = fma(-__ldg(&m[n]), y, pre[n]);
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) w[k] = w[k + 1];
        int pos = n + H + 1;
        w[2 * H] = pos < N ? src[pos * P] : T(0);
        dst[n * P] = y;
    }
    // interior rows
    for (int n = H; n < N - H; ++n) {
        T r = T(0);
#pragma unroll
        for (int k = 0; k < 2 * H + 1; ++k) r = fma(taps[k], w[k], r);
        y = fma(-__ldg(&m[n]), y, r * scale);
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) w[k] = w[k + 1];
        int pos = n + H + 1;
        w[2 * H] = pos < N ? src[pos * P] : T(0);
        dst[n * P] = y;
    }
    // rows N-H..N-1
#pragma unroll
    for (int b = 0; b < H; ++b) {
        int n = N - H + b;
        y = fma(-__ldg(&m[n]), y, pre[H + b]);
        dst[n * P] = y;
    }
    // back substitution
    T x = y * __ldg(&iw[N - 1]);
    dst[(N - 1) * P] = x;
    const T xlast = x;
    for (int n = N - 2; n >= 0; --n) {
        x = fma(-__ldg(&c[n]), x, dst[n * P]) * __ldg(&iw[n]);
        dst[n * P] = x;
    }
    if (!op.periodic) return 0.0;
    return ((double)x + op.bog * (double)xlast) * op.inv_den;
}

// Corrected value of solution n of a line whose factor is f.
template <typename T>
__device__ __forceinline__ T corr(T x, double f, const LineOp<T> &op, int n) {
    return op.periodic ? fma(-(T)f, __ldg(&op.z[n]), x) : x;
}

// ---------------------------------------------------------------------
// tile geometry
// ---------------------------------------------------------------------
struct Tile {
    long long base;   // global index of (line 0, position 0)
    long long sl, sn; // strides between lines and along a line
    int nlines;       // valid lines in this tile (<= L)
    int N;            // line length
    int ci, cj, ck;   // coordinates of (line 0, position 0)
};

template <int DIR>
__device__ __forceinline__ Tile make_tile(const Geom &g, int L) {
    Tile t;
    const long long nxy = (long long)g.Nx * g.Ny;
    if (DIR == 0) {  // x-lines at rows j0.., plane k
        int j0 = blockIdx.x * L, k = blockIdx.y;
        t.base = (long long)k * nxy + (long long)j0 * g.Nx;
        t.sl = g.Nx; t.sn = 1;
        t.nlines = min(L, g.Ny - j0);
        t.N = g.Nx;
        t.ci = 0; t.cj = j0; t.ck = k;
    } else if (DIR == 1) {  // y-lines at columns i0.., plane k
        int i0 = blockIdx.x * L, k = blockIdx.y;
        t.base = (long long)k * nxy + i0;
        t.sl = 1; t.sn = g.Nx;
        t.nlines = min(L, g.Nx - i0);
        t.N = g.Ny;
        t.ci = i0; t.cj = 0; t.ck = k;
    } else {  // z-lines at columns i0.., row j
        int i0 = blockIdx.x * L, j = blockIdx.y;
        t.base = (long long)j * g.Nx + i0;
        t.sl = 1; t.sn = nxy;
        t.nlines = min(L, g.Nx - i0);
        t.N = g.Nz;
        t.ci = i0; t.cj = j; t.ck = 0;
    }
    return t;
}

// Enumerate the points of a tile so that consecutive threads touch
// consecutive global addresses: position-major for x-lines, line-major
// otherwise.
template <int DIR>
__device__ __forceinline__ void point_of(int p, int L, int N, int &l, int &n) {
    if (DIR == 0) { l = p / N; n = p - l * N; }
    else { n = p / L; l = p - n * L; }
}

template <int DIR>
__device__ __forceinline__ void coords(const Tile &t, int l, int n, int &i, int &j, int &k) {
    if (DIR == 0) { i = n; j = t.cj + l; k = t.ck; }
    else if (DIR == 1) { i = t.ci + l; j = n; k = t.ck; }
    else { i = t.ci + l; j = t.cj; k = n; }
}

// Boundary classification of a point: bit f set if the point lies on face f
// (X0,X1,Y0,Y1,Z0,Z1) and that face has the given property.
__device__ __forceinline__ int faces_of(const Geom &g, int i, int j, int k) {
    int f = 0;
    f |= (i == 0) << 0; f |= (i == g.Nx - 1) << 1;
    f |= (j == 0) << 2; f |= (j == g.Ny - 1) << 3;
    f |= (k == 0) << 4; f |= (k == g.Nz - 1) << 5;
    return f;
}

// Direction whose continuity derivative survives at a wall point: the
// reference applies the wall faces in the order X0,X1,Y0,Y1,Z0,Z1 and the
// last write wins (CSolver_AWS.cpp:1526-1609).  -1 if not on a wall.
__device__ __forceinline__ int wall_dir(int onwall) {
    return (onwall & 0x30) ? 2 : (onwall & 0x0c) ? 1 : (onwall & 0x03) ? 0 : -1;
}

// ---------------------------------------------------------------------
// ideal gas (IdealGas.hpp:49-80)
// ---------------------------------------------------------------------
template <typename T>
struct Prim {
    T rho, ru, rv, rw, re;  // conserved
    T U, V, W, p, Tt;       // primitives
};

template <typename T>
__device__ __forceinline__ Prim<T> prim_from(const GasParams &gp, double r0, double r1, double r2,
                                             double r3, double r4) {
    Prim<T> s;
    s.rho = (T)r0; s.ru = (T)r1; s.rv = (T)r2; s.rw = (T)r3; s.re = (T)r4;
    s.U = s.ru / s.rho;
    s.V = s.rv / s.rho;
    s.W = s.rw / s.rho;
    s.p = (T)gp.gm1 * (s.re - T(0.5) * s.rho * (s.U * s.U + s.V * s.V + s.W * s.W));
    s.Tt = s.p / (s.rho * (T)gp.R);
    return s;
}

// ---------------------------------------------------------------------
// shared-memory layout of a sweep tile
// ---------------------------------------------------------------------
template <typename T>
struct Smem {
    T *buf;        // nbuf buffers of stride bstride
    double *fact;  // [nbuf][L]
    int bstride;
    int P;
    __device__ T *b(int k) const { return buf + (size_t)k * bstride; }
};

template <typename T>
__device__ __forceinline__ Smem<T> smem_layout(int nbuf, int L, int P, int N) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<T> s;
    s.P = P;
    int st = N * P + L;  // padding of L elements shifts banks between buffers
    st = (st + 1) & ~1;
    s.bstride = st;
    s.fact = reinterpret_cast<double *>(smem_raw);
    s.buf = reinterpret_cast<T *>(smem_raw + sizeof(double) * (size_t)nbuf * L);
    return s;
}

// Run the solve tasks of a sweep.  Task t on line l: if d2out >= 0 it first
// computes the 2nd derivative of buffer src into buffer d2out, then the 1st
// derivative of src in place.
struct SolveTask {
    signed char src, d2out;
};

template <typename T>
__device__ __forceinline__ void run_tasks(const Smem<T> &sm, const SolveTask *tasks, int ntask, int L,
                                          int nlines, const LineOp<T> &d1, const LineOp<T> &d2) {
    for (int w = threadIdx.x; w < ntask * L; w += blockDim.x) {
        int t = w / L, l = w - t * L;
        if (l >= nlines) continue;
        SolveTask tk = tasks[t];
        T *srcb = sm.b(tk.src) + l;
        if (tk.d2out >= 0) {
            T *o = sm.b(tk.d2out) + l;
            sm.fact[tk.d2out * L + l] = line_solve<T, 2>(srcb, o, sm.P, d2);
        }
        sm.fact[tk.src * L + l] = line_solve<T, 2>(srcb, srcb, sm.P, d1);
    }
}

template <typename T>
__device__ __forceinline__ T get(const Smem<T> &sm, int k, int l, int n, int L, const LineOp<T> &op) {
    return corr<T>(sm.b(k)[n * sm.P + l], sm.fact[k * L + l], op, n);
}

// ---------------------------------------------------------------------
// sweep x
// ---------------------------------------------------------------------
// buffers
enum { XU = 0, XU2, XV, XV2, XW, XW2, XT, XT2, XRU, XF1, XF2, XF3, XF4, XNB };
__constant__ SolveTask kTasksX[9] = {{XU, XU2}, {XV, XV2}, {XW, XW2}, {XT, XT2}, {XRU, -1},
                                     {XF1, -1}, {XF2, -1}, {XF3, -1}, {XF4, -1}};

template <typename T>
__global__ void __launch_bounds__(256) k_sweep_x(SweepArgs<T> a) {
    const int L = a.L;
    const Tile t = make_tile<0>(a.g, L);
    const int N = t.N;
    Smem<T> sm = smem_layout<T>(XNB, L, a.P, N);
    const GasParams gp = a.gas;

    // phase A: primitives and the inputs of the x-solves
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<0>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        Prim<T> s = prim_from<T>(gp, a.q.f[0][gi], a.q.f[1][gi], a.q.f[2][gi], a.q.f[3][gi], a.q.f[4][gi]);
        a.prim[0][gi] = s.U; a.prim[1][gi] = s.V; a.prim[2][gi] = s.W;
        a.prim[3][gi] = s.p; a.prim[4][gi] = s.Tt;
        // stage-start primitives: on stage 1, points of SPONGE faces (not on a
        // wall) use the state before the sponge overwrite of the previous
        // step, as the reference's U,V,W,p,T arrays still hold it.
        Prim<T> ss = s;
        if (a.use_backup) {
            int i, j, k;
            coords<0>(t, l, n, i, j, k);
            int f = faces_of(a.g, i, j, k);
            if ((f & a.sponge_faces) && !(f & a.wall_faces))
                ss = prim_from<T>(gp, a.backup.f[0][gi], a.backup.f[1][gi], a.backup.f[2][gi],
                                  a.backup.f[3][gi], a.backup.f[4][gi]);
        }
        int o = n * sm.P + l;
        sm.b(XU)[o] = ss.U;
        sm.b(XV)[o] = ss.V;
        sm.b(XW)[o] = ss.W;
        sm.b(XT)[o] = ss.Tt;
        sm.b(XRU)[o] = s.ru;
        sm.b(XF1)[o] = s.ru * ss.U + ss.p;
        sm.b(XF2)[o] = s.rv * ss.U;
        sm.b(XF3)[o] = s.rw * ss.U;
        sm.b(XF4)[o] = s.re * ss.U + ss.U * ss.p;
    }
    __syncthreads();
    run_tasks<T>(sm, kTasksX, 9, L, t.nlines, a.d1, a.d2);
    __syncthreads();
    // phase C
    const T c43 = T(4.0 / 3.0), cpPr = (T)gp.cpPr;
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<0>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        T U = a.prim[0][gi], V = a.prim[1][gi], W = a.prim[2][gi], Tt = a.prim[4][gi];
        T mu = (T)gp.mu_ref * pow(Tt, (T)0.76);
        T amu = (T)0.76 * mu / Tt;
        a.mu[gi] = mu;
        a.amu[gi] = amu;
        T Ux = get(sm, XU, l, n, L, a.d1), Uxx = get(sm, XU2, l, n, L, a.d2);
        T Vx = get(sm, XV, l, n, L, a.d1), Vxx = get(sm, XV2, l, n, L, a.d2);
        T Wx = get(sm, XW, l, n, L, a.d1), Wxx = get(sm, XW2, l, n, L, a.d2);
        T Tx = get(sm, XT, l, n, L, a.d1), Txx = get(sm, XT2, l, n, L, a.d2);
        T cex = get(sm, XRU, l, n, L, a.d1);
        T f1 = get(sm, XF1, l, n, L, a.d1), f2 = get(sm, XF2, l, n, L, a.d1);
        T f3 = get(sm, XF3, l, n, L, a.d1), f4 = get(sm, XF4, l, n, L, a.d1);
        a.dx[0][gi] = Ux; a.dx[1][gi] = Vx; a.dx[2][gi] = Wx; a.dx[3][gi] = Tx;
        a.R[0][gi] = -cex;
        a.R[1][gi] = mu * (c43 * Uxx) - f1;
        a.R[2][gi] = mu * Vxx - f2;
        a.R[3][gi] = mu * Wxx - f3;
        a.R[4][gi] = cpPr * mu * Txx + mu * (U * (c43 * Uxx) + V * Vxx + W * Wxx) - f4;
    }
}

// ---------------------------------------------------------------------
// sweep y
// ---------------------------------------------------------------------
enum { YU = 0, YU2, YV, YV2, YW, YW2, YT, YT2, YUX, YVX, YRV, YF1, YF2, YF3, YF4, YNB };
__constant__ SolveTask kTasksY[11] = {{YU, YU2}, {YV, YV2}, {YW, YW2}, {YT, YT2}, {YUX, -1}, {YVX, -1},
                                      {YRV, -1}, {YF1, -1}, {YF2, -1}, {YF3, -1}, {YF4, -1}};

template <typename T>
__global__ void __launch_bounds__(256) k_sweep_y(SweepArgs<T> a) {
    const int L = a.L;
    const Tile t = make_tile<1>(a.g, L);
    const int N = t.N;
    Smem<T> sm = smem_layout<T>(YNB, L, a.P, N);
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<1>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        T ru = (T)a.q.f[1][gi], rv = (T)a.q.f[2][gi], rw = (T)a.q.f[3][gi], re = (T)a.q.f[4][gi];
        T U = a.prim[0][gi], V = a.prim[1][gi], W = a.prim[2][gi], pp = a.prim[3][gi], Tt = a.prim[4][gi];
        int o = n * sm.P + l;
        sm.b(YU)[o] = U;
        sm.b(YV)[o] = V;
        sm.b(YW)[o] = W;
        sm.b(YT)[o] = Tt;
        sm.b(YUX)[o] = a.dx[0][gi];
        sm.b(YVX)[o] = a.dx[1][gi];
        sm.b(YRV)[o] = rv;
        sm.b(YF1)[o] = ru * V;
        sm.b(YF2)[o] = rv * V + pp;
        sm.b(YF3)[o] = rw * V;
        sm.b(YF4)[o] = re * V + V * pp;
    }
    __syncthreads();
    run_tasks<T>(sm, kTasksY, 11, L, t.nlines, a.d1, a.d2);
    __syncthreads();
    const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0), cpPr = (T)a.gas.cpPr;
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<1>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        T U = a.prim[0][gi], V = a.prim[1][gi], W = a.prim[2][gi];
        T mu = a.mu[gi];
        T Uy = get(sm, YU, l, n, L, a.d1), Uyy = get(sm, YU2, l, n, L, a.d2);
        T Vy = get(sm, YV, l, n, L, a.d1), Vyy = get(sm, YV2, l, n, L, a.d2);
        T Wy = get(sm, YW, l, n, L, a.d1), Wyy = get(sm, YW2, l, n, L, a.d2);
        T Ty = get(sm, YT, l, n, L, a.d1), Tyy = get(sm, YT2, l, n, L, a.d2);
        T Uxy = get(sm, YUX, l, n, L, a.d1), Vxy = get(sm, YVX, l, n, L, a.d1);
        T cey = get(sm, YRV, l, n, L, a.d1);
        T f1 = get(sm, YF1, l, n, L, a.d1), f2 = get(sm, YF2, l, n, L, a.d1);
        T f3 = get(sm, YF3, l, n, L, a.d1), f4 = get(sm, YF4, l, n, L, a.d1);
        a.dy[0][gi] = Uy; a.dy[1][gi] = Vy; a.dy[2][gi] = Wy; a.dy[3][gi] = Ty;
        int i, j, k;
        coords<1>(t, l, n, i, j, k);
        int wd = a.wall_faces ? wall_dir(faces_of(a.g, i, j, k) & a.wall_faces) : -1;
        if (wd == 1) a.R[0][gi] = -cey;
        else if (wd < 0) a.R[0][gi] = a.R[0][gi] - cey;
        a.R[1][gi] = a.R[1][gi] + (mu * (Uyy + c13 * Vxy) - f1);
        a.R[2][gi] = a.R[2][gi] + (mu * (c43 * Vyy + c13 * Uxy) - f2);
        a.R[3][gi] = a.R[3][gi] + (mu * Wyy - f3);
        a.R[4][gi] = a.R[4][gi] +
                     (cpPr * mu * Tyy + mu * (U * Uyy + V * (c43 * Vyy) + W * Wyy + c13 * (U * Vxy + V * Uxy)) - f4);
    }
}

// ---------------------------------------------------------------------
// sweep z + right-hand side + RK update
// ---------------------------------------------------------------------
enum { ZU = 0, ZU2, ZV, ZV2, ZW, ZW2, ZT, ZT2, ZS, ZWX, ZWY, ZRW, ZF1, ZF2, ZF3, ZF4, ZNB };
__constant__ SolveTask kTasksZ[12] = {{ZU, ZU2}, {ZV, ZV2}, {ZW, ZW2}, {ZT, ZT2}, {ZS, -1}, {ZWX, -1},
                                      {ZWY, -1}, {ZRW, -1}, {ZF1, -1}, {ZF2, -1}, {ZF3, -1}, {ZF4, -1}};

template <typename T>
__global__ void __launch_bounds__(256) k_sweep_z(SweepArgs<T> a) {
    const int L = a.L;
    const Tile t = make_tile<2>(a.g, L);
    const int N = t.N;
    Smem<T> sm = smem_layout<T>(ZNB, L, a.P, N);
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<2>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        T ru = (T)a.q.f[1][gi], rv = (T)a.q.f[2][gi], rw = (T)a.q.f[3][gi], re = (T)a.q.f[4][gi];
        T U = a.prim[0][gi], V = a.prim[1][gi], W = a.prim[2][gi], pp = a.prim[3][gi], Tt = a.prim[4][gi];
        int o = n * sm.P + l;
        sm.b(ZU)[o] = U;
        sm.b(ZV)[o] = V;
        sm.b(ZW)[o] = W;
        sm.b(ZT)[o] = Tt;
        sm.b(ZS)[o] = a.dx[0][gi] + a.dy[1][gi];
        sm.b(ZWX)[o] = a.dx[2][gi];
        sm.b(ZWY)[o] = a.dy[2][gi];
        sm.b(ZRW)[o] = rw;
        sm.b(ZF1)[o] = ru * W;
        sm.b(ZF2)[o] = rv * W;
        sm.b(ZF3)[o] = rw * W + pp;
        sm.b(ZF4)[o] = re * W + W * pp;
    }
    __syncthreads();
    run_tasks<T>(sm, kTasksZ, 12, L, t.nlines, a.d1, a.d2);
    __syncthreads();
    const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0), c23 = T(2.0 / 3.0), cpPr = (T)a.gas.cpPr;
    const double dt = *a.dt;
    const int st = a.rk_step;
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<2>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        T U = a.prim[0][gi], V = a.prim[1][gi], W = a.prim[2][gi];
        T mu = a.mu[gi], amu = a.amu[gi];
        T Ux = a.dx[0][gi], Vx = a.dx[1][gi], Wx = a.dx[2][gi], Tx = a.dx[3][gi];
        T Uy = a.dy[0][gi], Vy = a.dy[1][gi], Wy = a.dy[2][gi], Ty = a.dy[3][gi];
        T Uz = get(sm, ZU, l, n, L, a.d1), Uzz = get(sm, ZU2, l, n, L, a.d2);
        T Vz = get(sm, ZV, l, n, L, a.d1), Vzz = get(sm, ZV2, l, n, L, a.d2);
        T Wz = get(sm, ZW, l, n, L, a.d1), Wzz = get(sm, ZW2, l, n, L, a.d2);
        T Tz = get(sm, ZT, l, n, L, a.d1), Tzz = get(sm, ZT2, l, n, L, a.d2);
        T S = get(sm, ZS, l, n, L, a.d1);  // Uxz + Vyz
        T Wxz = get(sm, ZWX, l, n, L, a.d1), Wyz = get(sm, ZWY, l, n, L, a.d1);
        T cez = get(sm, ZRW, l, n, L, a.d1);
        T f1 = get(sm, ZF1, l, n, L, a.d1), f2 = get(sm, ZF2, l, n, L, a.d1);
        T f3 = get(sm, ZF3, l, n, L, a.d1), f4 = get(sm, ZF4, l, n, L, a.d1);
        if (a.diag[0]) {  // derivative fields of the last stage, for diagnostics
            a.diag[0][gi] = Uz; a.diag[1][gi] = Vz; a.diag[2][gi] = Wz;
        }
        double q[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) q[f] = a.q.f[f][gi];
        T src[5] = {T(0), T(0), T(0), T(0), T(0)};
        if (a.sponge) {
            double sg = a.sigma[gi];
#pragma unroll
            for (int f = 0; f < 5; ++f) src[f] = (T)(sg * (a.savg.f[f][gi] - q[f]));
        }
        const T MuX = amu * Tx, MuY = amu * Ty, MuZ = amu * Tz;
        T R[5];
        R[0] = a.R[0][gi];
        R[1] = a.R[1][gi] + mu * (Uzz + c13 * Wxz) - f1 + c43 * MuX * (Ux - T(0.5) * Vy - T(0.5) * Wz) +
               MuY * (Uy + Vx) + MuZ * (Wx + Uz) + src[1];
        R[2] = a.R[2][gi] + mu * (Vzz + c13 * Wyz) - f2 + c43 * MuY * (Vy - T(0.5) * Ux - T(0.5) * Wz) +
               MuX * (Uy + Vx) + MuZ * (Wy + Vz) + src[2];
        R[3] = a.R[3][gi] + mu * (c43 * Wzz + c13 * S) - f3 + c43 * MuZ * (Wz - T(0.5) * Ux - T(0.5) * Vy) +
               MuX * (Wx + Uz) + MuY * (Wy + Vz) + src[3];
        T q2 = Ux * Ux + Vy * Vy + Wz * Wz;
        T sq = Uy * Uy + Uz * Uz + Vx * Vx + Vz * Vz + Wx * Wx + Wy * Wy;
        T cr = Ux * Vy + Ux * Wz + Vy * Wz;
        T sh = Uy * Vx + Uz * Wx + Vz * Wy;
        T v1 = mu * (U * Uzz + V * Vzz + W * (c43 * Wzz) + c13 * (U * Wxz + V * Wyz + W * S) + c43 * q2 + sq -
                     c43 * cr + T(2.0) * sh);
        T v2 = c43 * (U * MuX * Ux + V * MuY * Vy + W * MuZ * Wz) - c23 * U * MuX * (Vy + Wz) -
               c23 * V * MuY * (Ux + Wz) - c23 * W * MuZ * (Ux + Vy) + U * MuY * (Uy + Vx) + U * MuZ * (Uz + Wx) +
               V * MuX * (Uy + Vx) + V * MuZ * (Vz + Wy) + W * MuX * (Uz + Wx) + W * MuY * (Vz + Wy);
        R[4] = a.R[4][gi] + cpPr * (MuX * Tx + MuY * Ty + MuZ * Tz + mu * Tzz) + v1 + v2 - f4 + T(2.0) * src[4];
        // continuity and the post-step boundary fix-up (CSolver_AWS.cpp:1506-1679)
        int i, j, k;
        coords<2>(t, l, n, i, j, k);
        int fc = faces_of(a.g, i, j, k);
        int wd = a.wall_faces ? wall_dir(fc & a.wall_faces) : -1;
        double dq[5];
        if (wd == 2) R[0] = -cez;
        else if (wd < 0) R[0] = R[0] - cez + src[0];
        dq[0] = dt * (double)R[0];
#pragma unroll
        for (int f = 1; f < 5; ++f) dq[f] = dt * (double)R[f];
        if (wd >= 0) {
#pragma unroll
            for (int f = 1; f < 5; ++f) dq[f] = 0.0;
        }
        if (fc & a.sponge_kind_faces) {
#pragma unroll
            for (int f = 0; f < 5; ++f) dq[f] = 0.0;
        }
        if (a.dq_out[0]) {
#pragma unroll
            for (int f = 0; f < 5; ++f) a.dq_out[f][gi] = dq[f];
        }
        // RK update (RK4.hpp:35-118, TVDRK3.hpp:38-96)
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            double q1 = a.q1.f[f][gi];
            if (a.rk == 1) {  // TVD-RK3
                if (st == 1) a.qk.f[f][gi] = q1 + dq[f];
                else if (st == 2) a.qk.f[f][gi] = 0.75 * q1 + 0.25 * q[f] + 0.25 * dq[f];
                else a.q2.f[f][gi] = (1.0 / 3.0) * q1 + (2.0 / 3.0) * q[f] + (2.0 / 3.0) * dq[f];
            } else {
                const double ca = (st == 1 || st == 4) ? (1.0 / 6.0) : (1.0 / 3.0);
                const double cb = (st == 3) ? 1.0 : 0.5;
                if (st == 1) a.q2.f[f][gi] = q1 + ca * dq[f];
                else a.q2.f[f][gi] = a.q2.f[f][gi] + ca * dq[f];
                if (st < 4) a.qk.f[f][gi] = q1 + cb * dq[f];
            }
        }
    }
}

// ---------------------------------------------------------------------
// compact filter, one direction, five fields (Filter.cpp:98-171)
// ---------------------------------------------------------------------
// FP64 form: src/dst are double.  Mixed form: the first pass reads FP64 q2
// minus a per-field reference value, the middle pass works in FP32, and the
// last pass writes q1 = q2 + (filtered - unfiltered) in FP64.
template <typename T, int DIR>
__global__ void __launch_bounds__(256) k_filter(FilterArgs<T> a) {
    const int L = a.L;
    const Tile t = make_tile<DIR>(a.g, L);
    const int N = t.N;
    Smem<T> sm = smem_layout<T>(5, L, a.P, N);
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<DIR>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
        int o = n * sm.P + l;
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            T v;
            if (a.src64.f[f]) v = (T)(a.src64.f[f][gi] - a.ref[f]);
            else v = a.src32[f][gi];
            sm.b(f)[o] = v;
        }
    }
    __syncthreads();
    for (int w = threadIdx.x; w < 5 * L; w += blockDim.x) {
        int f = w / L, l = w - f * L;
        if (l >= t.nlines) continue;
        T *b = sm.b(f) + l;
        sm.fact[f * L + l] = line_solve<T, 4>(b, b, sm.P, a.op);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l, n;
        point_of<DIR>(p, L, N, l, n);
        if (l >= t.nlines) continue;
        long long gi = t.base + l * t.sl + n * t.sn;
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            T v = get(sm, f, l, n, L, a.op);
            if (a.dst64.f[f]) {
                if (a.delta_from.f[f]) {
                    double q = a.delta_from.f[f][gi];
                    T v0 = (T)(q - a.ref[f]);
                    a.dst64.f[f][gi] = q + (double)(v - v0);
                } else {
                    a.dst64.f[f][gi] = (double)v + a.ref[f];
                }
            } else {
                a.dst32[f][gi] = v;
            }
        }
    }
}

// ---------------------------------------------------------------------
// single operator on contiguous lines (Derivatives::calc1stDerivField etc.)
// ---------------------------------------------------------------------
template <int H>
__global__ void __launch_bounds__(256) k_line_op(LineOpArgs a) {
    const int L = a.L, N = a.op.N;
    const long long l0 = (long long)blockIdx.x * L;
    const int nl = (int)min((long long)L, a.nlines - l0);
    Smem<double> sm = smem_layout<double>(1, L, a.P, N);
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l = p / N, n = p - l * N;
        if (l >= nl) continue;
        sm.b(0)[n * sm.P + l] = a.in[(l0 + l) * N + n];
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nl; l += blockDim.x) {
        double *b = sm.b(0) + l;
        sm.fact[l] = line_solve<double, H>(b, b, sm.P, a.op);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        int l = p / N, n = p - l * N;
        if (l >= nl) continue;
        a.out[(l0 + l) * N + n] = get(sm, 0, l, n, L, a.op);
    }
}

// ---------------------------------------------------------------------
// wall boundary conditions before the derivatives (CSolver_AWS.cpp:553-826)
// ---------------------------------------------------------------------
// One launch per face, in the reference's order.  Temperatures of interior
// points come from the current state; on stage 1, points of SPONGE faces that
// are not on a wall use the state saved before the previous step's sponge
// overwrite.
__device__ __forceinline__ double temp_at(const BCArgs &a, long long gi, int fc) {
    const double *q[5];
    bool bk = a.use_backup && (fc & a.sponge_faces) && !(fc & a.wall_faces);
#pragma unroll
    for (int f = 0; f < 5; ++f) q[f] = bk ? a.backup.f[f] : a.q.f[f];
    double r = q[0][gi];
    double U = q[1][gi] / r, V = q[2][gi] / r, W = q[3][gi] / r;
    double p = a.gas.gm1 * (q[4][gi] - 0.5 * r * (U * U + V * V + W * W));
    return p / (r * a.gas.R);
}

__global__ void k_wall_pre(BCArgs a) {
    const Geom g = a.g;
    const int dir = a.face / 2, hi = a.face % 2;
    const int n1 = dir == 0 ? g.Ny : g.Nx, n2 = dir == 2 ? g.Ny : g.Nz;
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n1 * n2) return;
    int a1 = (int)(idx % n1), a2 = (int)(idx / n1);
    int Nd = dir == 0 ? g.Nx : dir == 1 ? g.Ny : g.Nz;
    int fix = hi ? Nd - 1 : 0, sg = hi ? -1 : 1;
    int i, j, k;
    if (dir == 0) { i = fix; j = a1; k = a2; }
    else if (dir == 1) { i = a1; j = fix; k = a2; }
    else { i = a1; j = a2; k = fix; }
    const long long nxy = (long long)g.Nx * g.Ny;
    const long long gi = (long long)k * nxy + (long long)j * g.Nx + i;
    const long long step = dir == 0 ? 1 : dir == 1 ? g.Nx : nxy;
    double Tn[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        long long nb = gi + sg * (m + 1) * step;
        int ii = i, jj = j, kk = k;
        if (dir == 0) ii += sg * (m + 1); else if (dir == 1) jj += sg * (m + 1); else kk += sg * (m + 1);
        Tn[m] = temp_at(a, nb, faces_of(g, ii, jj, kk));
    }
    // Utils.hpp:52-54
    double Tw = (Tn[0] * 360.0 - Tn[1] * 450.0 + Tn[2] * 400.0 - Tn[3] * 225.0 + Tn[4] * 72.0 - Tn[5] * 10.0) / 147.0;
    double r = a.q.f[0][gi];
    double u[3] = {a.uw[0], a.uw[1], a.uw[2]};
    a.q.f[1][gi] = dir == 0 ? 0.0 : r * u[0];
    a.q.f[2][gi] = dir == 1 ? 0.0 : r * u[1];
    a.q.f[3][gi] = dir == 2 ? 0.0 : r * u[2];
    double p = r * a.gas.R * Tw;
    a.q.f[4][gi] = p / a.gas.gm1 + 0.5 * r * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
}

// ---------------------------------------------------------------------
// CFL reduction (CSolver_AWS.cpp:507-525): max over points of
// (|u|+c)/dx + (|v|+c)/dy + (|w|+c)/dz, kept as the bit pattern of a
// positive double so atomicMax on 64-bit integers orders it.
// ---------------------------------------------------------------------
__global__ void k_cfl(CflArgs a) {
    double mx = 0.0;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double r = a.q.f[0][gi];
        double U = a.q.f[1][gi] / r, V = a.q.f[2][gi] / r, W = a.q.f[3][gi] / r;
        double p = a.gas.gm1 * (a.q.f[4][gi] - 0.5 * r * (U * U + V * V + W * W));
        double c = sqrt(a.gas.gamma * p / r);
        double v = (fabs(U) + c) / a.dx + (fabs(V) + c) / a.dy + (fabs(W) + c) / a.dz;
        if (!(v == v) || isinf(v)) { *a.nan_flag = 1; v = 0.0; }
        mx = fmax(mx, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double red[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = mx;
    __syncthreads();
    if (wid == 0) {
        mx = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) atomicMax(reinterpret_cast<unsigned long long *>(a.max_out), __double_as_longlong(mx));
    }
}

// dt = CFL / max and the step/time counters (CSolver_AWS.cpp:530-543).
__global__ void k_finalize_dt(DtArgs a) {
    double mx = *a.max_in;
    double dt = a.dt_fixed > 0.0 ? a.dt_fixed : a.CFL / mx;
    *a.dt = dt;
    if (a.first) *a.time = 0.0;
    else *a.time = *a.time + dt;
}

// ---------------------------------------------------------------------
// updateSponge (CSolver_AWS.cpp:1937-2031)
// ---------------------------------------------------------------------
__global__ void k_sponge_update(SpongeArgs a) {
    const double eps = 1.0 / (a.avgT / *a.dt + 1.0);
    const long long nxy = (long long)a.g.Nx * a.g.Ny;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double av[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            double s = a.savg.f[f][gi];
            s += eps * (a.q1.f[f][gi] - s);
            av[f] = s;
        }
        av[4] = a.epsP * av[4] +
                (1.0 - a.epsP) * (a.spongeP / a.gm1 + 0.5 * (av[1] * av[1] + av[2] * av[2] + av[3] * av[3]) / av[0]);
#pragma unroll
        for (int f = 0; f < 5; ++f) a.savg.f[f][gi] = av[f];
        if (a.sponge_kind_faces) {
            int k = (int)(gi / nxy);
            long long rem = gi - k * nxy;
            int j = (int)(rem / a.g.Nx), i = (int)(rem - (long long)j * a.g.Nx);
            if (faces_of(a.g, i, j, k) & a.sponge_kind_faces) {
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    a.backup.f[f][gi] = a.q1.f[f][gi];
                    a.q1.f[f][gi] = av[f];
                }
            }
        }
    }
}

// ---------------------------------------------------------------------
// initial conditions (CSolver_AWS.cpp:199-504)
// ---------------------------------------------------------------------
// q1 from rho, p, U, V, W (:207-233); T0 = p/(rho R) (:233).
__global__ void k_ic(IcArgs a) {
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double r = a.rho0[gi], U = a.U0[gi], V = a.V0[gi], W = a.W0[gi], p = a.p0[gi];
        a.q1.f[0][gi] = r;
        a.q1.f[1][gi] = r * U;
        a.q1.f[2][gi] = r * V;
        a.q1.f[3][gi] = r * W;
        a.q1.f[4][gi] = p / (a.gas.gamma - 1.0) + 0.5 * r * (U * U + V * V + W * W);
        a.T0[gi] = p / (r * a.gas.R);
    }
}

// One wall face of the initial state (:258-472): wall velocity into U0,V0,W0
// and the momenta, Neumann temperature into T0.  One launch per face in the
// reference's order, so later faces read the temperatures earlier faces set.
__global__ void k_ic_wall(IcArgs a) {
    const Geom g = a.g;
    const int dir = a.face / 2, hi = a.face % 2;
    const int n1 = dir == 0 ? g.Ny : g.Nx, n2 = dir == 2 ? g.Ny : g.Nz;
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n1 * n2) return;
    int a1 = (int)(idx % n1), a2 = (int)(idx / n1);
    int Nd = dir == 0 ? g.Nx : dir == 1 ? g.Ny : g.Nz;
    int fix = hi ? Nd - 1 : 0, sg = hi ? -1 : 1;
    int i, j, k;
    if (dir == 0) { i = fix; j = a1; k = a2; }
    else if (dir == 1) { i = a1; j = fix; k = a2; }
    else { i = a1; j = a2; k = fix; }
    const long long nxy = (long long)g.Nx * g.Ny;
    const long long gi = (long long)k * nxy + (long long)j * g.Nx + i;
    const long long step = dir == 0 ? 1 : dir == 1 ? g.Nx : nxy;
    double Tn[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) Tn[m] = a.T0[gi + sg * (m + 1) * step];
    double Tw = (Tn[0] * 360.0 - Tn[1] * 450.0 + Tn[2] * 400.0 - Tn[3] * 225.0 + Tn[4] * 72.0 - Tn[5] * 10.0) / 147.0;
    a.T0[gi] = Tw;
    double r = a.q1.f[0][gi];
    a.U0[gi] = a.uw[0];
    a.V0[gi] = a.uw[1];
    a.W0[gi] = a.uw[2];
    a.q1.f[1][gi] = dir == 0 ? 0.0 : r * a.uw[0];
    a.q1.f[2][gi] = dir == 1 ? 0.0 : r * a.uw[1];
    a.q1.f[3][gi] = dir == 2 ? 0.0 : r * a.uw[2];
}

// With any wall present the reference recomputes p = rho R T and rhoE from
// the (wall-modified) U,V,W arrays at every point (:476-484).
__global__ void k_ic_wall_eos(IcArgs a) {
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double r = a.q1.f[0][gi];
        double U = a.U0[gi], V = a.V0[gi], W = a.W0[gi];
        double p = r * a.gas.R * a.T0[gi];
        a.q1.f[4][gi] = p / (a.gas.gamma - 1.0) + 0.5 * r * (U * U + V * V + W * W);
    }
}

// Primitives of q1 for diagnostics: U,V,W,p,T,mu,sos (updateNonConservedData,
// CSolver_AWS.cpp:1895-1935).
__global__ void k_primitives(PrimArgs a) {
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double r = a.q.f[0][gi];
        double U = a.q.f[1][gi] / r, V = a.q.f[2][gi] / r, W = a.q.f[3][gi] / r;
        double p = a.gas.gm1 * (a.q.f[4][gi] - 0.5 * r * (U * U + V * V + W * W));
        double T = p / (r * a.gas.R);
        a.out[0][gi] = U; a.out[1][gi] = V; a.out[2][gi] = W; a.out[3][gi] = p; a.out[4][gi] = T;
        a.out[5][gi] = a.gas.mu_ref * pow(T, 0.76);
        a.out[6][gi] = sqrt(a.gas.gamma * p / r);
    }
}

// Scan a state for non-finite values.
__global__ void k_nan_scan(CflArgs a) {
    int bad = 0;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            double v = a.q.f[f][gi];
            bad |= !(v == v) || isinf(v);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *a.nan_flag = 1;
}


// ---------------------------------------------------------------------
// Taylor-Green diagnostics (CSolver_AWS.cpp:2175-2236): per-block partial
// sums of enstrophy, 2mu-enstrophy, dissipation, kinetic energy, squared
// dilatation and mu, reduced in a fixed order on the host.
// ---------------------------------------------------------------------
template <typename T>
__global__ void k_tgv(TgvArgs<T> a) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    const double inv_n = 1.0 / (double)a.g.npts;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double Ux = a.dx[0][gi], Vx = a.dx[1][gi], Wx = a.dx[2][gi];
        double Uy = a.dy[0][gi], Vy = a.dy[1][gi], Wy = a.dy[2][gi];
        double Uz = a.dz[0][gi], Vz = a.dz[1][gi], Wz = a.dz[2][gi];
        double r = a.q.f[0][gi];
        double U = a.q.f[1][gi] / r, V = a.q.f[2][gi] / r, W = a.q.f[3][gi] / r;
        double p = a.gas.gm1 * (a.q.f[4][gi] - 0.5 * r * (U * U + V * V + W * W));
        double mu = a.gas.mu_ref * pow(p / (r * a.gas.R), 0.76);
        double tr = (1.0 / 3.0) * (Ux + Vy + Wz);
        double S00 = Ux - tr, S11 = Vy - tr, S22 = Wz - tr;
        double S01 = 0.5 * (Uy + Vx), S02 = 0.5 * (Uz + Wx), S12 = 0.5 * (Vz + Wy);
        double td = S00 * Ux + S01 * Uy + S02 * Uz + S01 * Vx + S11 * Vy + S12 * Vz + S02 * Wx + S12 * Wy + S22 * Wz;
        double wx = Wy - Vz, wy = Uz - Wx, wz = Vx - Uy;
        double om = wx * wx + wy * wy + wz * wz;
        s[0] += 0.5 * r * om;
        s[1] += mu * r * om;
        s[2] += 2.0 * mu * td;
        s[3] += r * (U * U + V * V + W * W) / 2.0;
        s[4] += (Ux + Vy + Wz) * (Ux + Vy + Wz) * inv_n;
        s[5] += mu * inv_n;
    }
    __shared__ double red[6][32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double v = s[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[i][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
        a.out[blockIdx.x * 6 + threadIdx.x] = v;
    }
}

template <typename T>
cudaError_t launch_tgv(const TgvArgs<T> &a, int blocks, cudaStream_t s) {
    k_tgv<T><<<blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}
template cudaError_t launch_tgv<double>(const TgvArgs<double> &, int, cudaStream_t);
template cudaError_t launch_tgv<float>(const TgvArgs<float> &, int, cudaStream_t);

// ---------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------
template <typename T>
static size_t sweep_smem(int nbuf, int L, int P, int N) {
    int st = N * P + L;
    st = (st + 1) & ~1;
    return sizeof(double) * (size_t)nbuf * L + sizeof(T) * (size_t)nbuf * st;
}

template <typename T>
cudaError_t launch_sweep(int dir, const SweepArgs<T> &a, cudaStream_t s) {
    const int nb = dir == 0 ? XNB : dir == 1 ? YNB : ZNB;
    const int N = dir == 0 ? a.g.Nx : dir == 1 ? a.g.Ny : a.g.Nz;
    size_t sm = sweep_smem<T>(nb, a.L, a.P, N);
    dim3 grid, block(a.threads);
    if (dir == 0) grid = dim3((a.g.Ny + a.L - 1) / a.L, a.g.Nz);
    else if (dir == 1) grid = dim3((a.g.Nx + a.L - 1) / a.L, a.g.Nz);
    else grid = dim3((a.g.Nx + a.L - 1) / a.L, a.g.Ny);
    cudaError_t e;
    if (dir == 0) {
        e = cudaFuncSetAttribute(k_sweep_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_sweep_x<T><<<grid, block, sm, s>>>(a);
    } else if (dir == 1) {
        e = cudaFuncSetAttribute(k_sweep_y<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_sweep_y<T><<<grid, block, sm, s>>>(a);
    } else {
        e = cudaFuncSetAttribute(k_sweep_z<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_sweep_z<T><<<grid, block, sm, s>>>(a);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_filter(int dir, const FilterArgs<T> &a, cudaStream_t s) {
    const int N = dir == 0 ? a.g.Nx : dir == 1 ? a.g.Ny : a.g.Nz;
    size_t sm = sweep_smem<T>(5, a.L, a.P, N);
    dim3 grid, block(a.threads);
    if (dir == 0) grid = dim3((a.g.Ny + a.L - 1) / a.L, a.g.Nz);
    else if (dir == 1) grid = dim3((a.g.Nx + a.L - 1) / a.L, a.g.Nz);
    else grid = dim3((a.g.Nx + a.L - 1) / a.L, a.g.Ny);
    cudaError_t e;
#define CS3D_FL(D)                                                                                    \
    e = cudaFuncSetAttribute(k_filter<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);   \
    if (e != cudaSuccess) return e;                                                                   \
    k_filter<T, D><<<grid, block, sm, s>>>(a);
    if (dir == 0) { CS3D_FL(0) } else if (dir == 1) { CS3D_FL(1) } else { CS3D_FL(2) }
#undef CS3D_FL
    return cudaGetLastError();
}

cudaError_t launch_line_op(const LineOpArgs &a, cudaStream_t s) {
    size_t sm = sweep_smem<double>(1, a.L, a.P, a.op.N);
    dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L)), block(a.threads);
    cudaError_t e;
    if (a.op.H == 4) {
        e = cudaFuncSetAttribute(k_line_op<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_line_op<4><<<grid, block, sm, s>>>(a);
    } else {
        e = cudaFuncSetAttribute(k_line_op<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_line_op<2><<<grid, block, sm, s>>>(a);
    }
    return cudaGetLastError();
}

size_t sweep_smem_bytes(int prec_bytes, int nbuf, int L, int P, int N) {
    return prec_bytes == 8 ? sweep_smem<double>(nbuf, L, P, N) : sweep_smem<float>(nbuf, L, P, N);
}

int sweep_nbuf(int dir) { return dir == 0 ? XNB : dir == 1 ? YNB : ZNB; }
int sweep_ntask(int dir) { return dir == 0 ? 9 : dir == 1 ? 11 : 12; }

static int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152 * 16) b = 152 * 16;
    if (b < 1) b = 1;
    return (int)b;
}

cudaError_t launch_wall_pre(const BCArgs &a, cudaStream_t s) {
    const int dir = a.face / 2;
    long long n = dir == 0 ? (long long)a.g.Ny * a.g.Nz : dir == 1 ? (long long)a.g.Nx * a.g.Nz
                                                                   : (long long)a.g.Nx * a.g.Ny;
    k_wall_pre<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_cfl(const CflArgs &a, cudaStream_t s) {
    k_cfl<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_nan_scan(const CflArgs &a, cudaStream_t s) {
    k_nan_scan<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_finalize_dt(const DtArgs &a, cudaStream_t s) {
    k_finalize_dt<<<1, 1, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_sponge_update(const SpongeArgs &a, cudaStream_t s) {
    k_sponge_update<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_ic(const IcArgs &a, cudaStream_t s) {
    k_ic<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_ic_wall(const IcArgs &a, cudaStream_t s) {
    const int dir = a.face / 2;
    long long n = dir == 0 ? (long long)a.g.Ny * a.g.Nz : dir == 1 ? (long long)a.g.Nx * a.g.Nz
                                                                   : (long long)a.g.Nx * a.g.Ny;
    k_ic_wall<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_ic_wall_eos(const IcArgs &a, cudaStream_t s) {
    k_ic_wall_eos<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_primitives(const PrimArgs &a, cudaStream_t s) {
    k_primitives<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_sweep<double>(int, const SweepArgs<double> &, cudaStream_t);
template cudaError_t launch_sweep<float>(int, const SweepArgs<float> &, cudaStream_t);
template cudaError_t launch_filter<double>(int, const FilterArgs<double> &, cudaStream_t);
template cudaError_t launch_filter<float>(int, const FilterArgs<float> &, cudaStream_t);

}  // namespace cs3d
