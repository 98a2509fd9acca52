// cs3d_tile.cuh -- pencil-tile machinery shared by the stage sweeps and the
// adjoint kernels: chunked Thomas line solves with the cyclic correction,
// tile geometry, shared-memory layout, point loops and primitives.
#pragma once
#include "cs3d_dev.cuh"
#include "cs3d_kernels.cuh"
#include <type_traits>

namespace cs3d {

// ---------------------------------------------------------------------
// line solves
// ---------------------------------------------------------------------
// Rows of padding after each line buffer in shared memory, so that the
// chunked forward pass may read ahead past the line's end without a test:
// it reads rows up to max(2H + kU, N + kU) = N + kU for N >= 8.
constexpr int kPad = kU + 2;

// The first H and last H rows of the right-hand side, from explicit rows.
template <typename T, int H>
__device__ __forceinline__ void boundary_rows(const T *src, int P, const LineOp<T> &op, T pre[2 * H]) {
    const int N = op.N;
#pragma unroll
    for (int b = 0; b < 2 * H; ++b) {
        const int col = op.boff[b];
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < kTaps; ++k) {
            int cc = col + k;
            cc = cc < 0 ? cc + N : (cc >= N ? cc - N : cc);
            acc = fma(op.btaps[b][k], src[cc * P], acc);
        }
        pre[b] = acc;
    }
}

// ---------------------------------------------------------------------
// line solves of the sweeps
// ---------------------------------------------------------------------
// One compact-operator line solve (`solve_lanes`): the explicit right-hand
// side formed on the fly from a sliding register window, the Thomas forward
// pass and back substitution over the precomputed factors, in place (the
// forward pass reads rows beyond those it writes, and the first and last H
// explicit rows are formed before any write); for a periodic line the
// Sherman-Morrison factor is formed in FP64 from the solution's end values and
// stored for the consumers, which apply the correction on read.
// FP32-mixed tiles keep the two solves of a task pair-interleaved in shared
// memory: element n of the pair is the float2 at row n, lane x holding solve
// A's line and lane y solve B's, each solve reading and writing its own lane
// (where both solves differentiate one field, the load phase stores the field
// in both lanes).  A task runs on two threads, one lane each (NL = 1: a warp's
// 32 lanes read 16 lines x 2 lanes, 128 contiguous bytes a row), or on one
// thread that takes both lanes with 64-bit accesses (NL = 2).  The plain FP64
// tiles are planar, one buffer per solve (NL = 1, RS = 1).  The arithmetic is
// per solve and its order fixed, so every form gives the same bits.
template <int NL, typename S = float>
struct Lanes;
template <>
struct Lanes<2, float> {
    using V = float2;
    static __device__ __forceinline__ V mk(float a, float b) { return make_float2(a, b); }
    static __device__ __forceinline__ V fma_(V a, V b, V c) {
        return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
    }
    static __device__ __forceinline__ V mul(V a, V b) { return make_float2(a.x * b.x, a.y * b.y); }
    static __device__ __forceinline__ float la(V v) { return v.x; }
    static __device__ __forceinline__ float lb(V v) { return v.y; }
};
template <typename S>
struct Lanes<1, S> {
    using V = S;
    static __device__ __forceinline__ V mk(S a, S) { return a; }
    static __device__ __forceinline__ V fma_(V a, V b, V c) { return fma(a, b, c); }
    static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
    static __device__ __forceinline__ S la(V v) { return v; }
    static __device__ __forceinline__ S lb(V v) { return v; }
};

// NL = 2: pr is the pair (row stride P float2s), A = lane x with (oa, fa),
// B = lane y with (ob, fb).  NL = 1: pr points at one solve's first element,
// row stride RS * P elements of type S (RS = 2: one lane of a pair array;
// RS = 1: a planar buffer), and only (oa, fa) are used -- ob bounds the
// constant-factor rows with oa.
template <int NL, int H, int PC, typename S = float, int RS = 2>
__device__ __forceinline__ void solve_lanes(typename Lanes<NL, S>::V *pr, const LineOp<S> &oa, S *fa,
                                            const LineOp<S> &ob, S *fb, int P_) {
    using Ls = Lanes<NL, S>;
    using V = typename Ls::V;
    constexpr int W = 2 * H + 1;
    const int P = (PC > 0 ? PC : P_) * (NL == 2 ? 1 : RS);  // row stride in V
    const int N = oa.N;
    const S *lx = reinterpret_cast<const S *>(pr);
    S pa[2 * H], pb[2 * H];
    boundary_rows<S, H>(lx, NL == 2 ? 2 * P : P, oa, pa);
    if constexpr (NL == 2) boundary_rows<S, H>(lx + 1, 2 * P, ob, pb);
    else {
#pragma unroll
        for (int b = 0; b < 2 * H; ++b) pb[b] = pa[b];
    }
    V t2[W];
#pragma unroll
    for (int k = 0; k < W; ++k) t2[k] = Ls::mk(oa.taps[kMaxH - H + k], ob.taps[kMaxH - H + k]);
    const S *__restrict__ ma = oa.m;
    const S *__restrict__ mb = ob.m;
    // window of the first interior row H: positions 0..2H
    V w[W];
#pragma unroll
    for (int k = 0; k < W; ++k) w[k] = pr[k * P];
    // rows 0..H-1
    V y = Ls::mk(pa[0], pb[0]);
    pr[0] = y;
#pragma unroll
    for (int n = 1; n < H; ++n) {
        y = Ls::fma_(Ls::mk(-ldc(&ma[n]), -ldc(&mb[n])), y, Ls::mk(pa[n], pb[n]));
        pr[n * P] = y;
    }
    // interior rows H..N-H-1 in chunks of kU, the next chunk read ahead;
    // chunks inside [klo, khi) of both operators (chunk starts kept on the kU
    // lattice from H, so the 128-bit factor loads stay aligned) run on the
    // register constants km, the others load m through mf
    const int nend = N - H;
    int n = H;
    const int klo = max(oa.klo, ob.klo), khi = min(oa.khi, ob.khi);
    const int clo = H + kU * ((max(klo - H, 0) + kU - 1) / kU);
    const V km2 = Ls::mk(-oa.km, -ob.km);
    V nx[kU];
#pragma unroll
    for (int j = 0; j < kU; ++j) nx[j] = pr[(n + H + 1 + j) * P];
    S ma4[kU], mb4[kU];
    load4(oa.mf, ma4);
    load4(ob.mf, mb4);
    auto fwd_chunk = [&](auto kconst) {
        constexpr bool K = decltype(kconst)::value;
        V c[kU], mc[kU];
#pragma unroll
        for (int j = 0; j < kU; ++j) {
            c[j] = nx[j];
            mc[j] = K ? km2 : Ls::mk(-ma4[j], -mb4[j]);
        }
#pragma unroll
        for (int j = 0; j < kU; ++j) nx[j] = pr[(n + kU + H + 1 + j) * P];
        if (!K) {
            load4(oa.mf + (n + kU - H), ma4);
            load4(ob.mf + (n + kU - H), mb4);
        }
        V e[W + kU];
#pragma unroll
        for (int k = 0; k < W; ++k) e[k] = w[k];
#pragma unroll
        for (int j = 0; j < kU; ++j) e[W + j] = c[j];
#pragma unroll
        for (int j = 0; j < kU; ++j) {
            V acc = Ls::mk(S(0), S(0));
#pragma unroll
            for (int k = 0; k < W; ++k) acc = Ls::fma_(t2[k], e[j + k], acc);
            y = Ls::fma_(mc[j], y, acc);
            pr[(n + j) * P] = y;
        }
#pragma unroll
        for (int k = 0; k < W; ++k) w[k] = e[kU + k];
    };
    for (; n + kU <= nend && n < clo; n += kU) fwd_chunk(std::false_type{});
    if (n + kU <= khi) {
#pragma unroll 2
        for (; n + kU <= nend && n + kU <= khi; n += kU) fwd_chunk(std::true_type{});
        load4(oa.mf + (n - H), ma4);
        load4(ob.mf + (n - H), mb4);
    }
#pragma unroll 2
    for (; n + kU <= nend; n += kU) fwd_chunk(std::false_type{});
    for (; n < nend; ++n) {
        V acc = Ls::mk(S(0), S(0));
#pragma unroll
        for (int k = 0; k < W; ++k) acc = Ls::fma_(t2[k], w[k], acc);
        y = Ls::fma_(Ls::mk(-ldc(&ma[n]), -ldc(&mb[n])), y, acc);
#pragma unroll
        for (int k = 0; k < W - 1; ++k) w[k] = w[k + 1];
        const int pos = n + H + 1;
        w[W - 1] = pos < N ? pr[pos * P] : Ls::mk(S(0), S(0));
        pr[n * P] = y;
    }
    // rows N-H..N-1
#pragma unroll
    for (int b = 0; b < H; ++b) {
        const int r = N - H + b;
        y = Ls::fma_(Ls::mk(-ldc(&ma[r]), -ldc(&mb[r])), y, Ls::mk(pa[H + b], pb[H + b]));
        pr[r * P] = y;
    }
    // back substitution in chunks of kU, next chunk prefetched
    const S *__restrict__ ca_ = oa.c;
    const S *__restrict__ cb_ = ob.c;
    const S *__restrict__ ia = oa.iw;
    const S *__restrict__ ib = ob.iw;
    V x = Ls::mul(y, Ls::mk(ldc(&ia[N - 1]), ldc(&ib[N - 1])));
    pr[(N - 1) * P] = x;
    const V xl = x;
    n = N - 2;
    V y4[kU];
#pragma unroll
    for (int j = 0; j < kU; ++j) y4[j] = pr[max(n - j, 0) * P];
    S cA[kU], cB[kU], iA[kU], iB[kU];
    load4(oa.cbk, cA); load4(ob.cbk, cB);
    load4(oa.ibk, iA); load4(ob.ibk, iB);
    const V kc2 = Ls::mk(-oa.kc, -ob.kc), ki2 = Ls::mk(oa.kiw, ob.kiw);
    auto bwd_chunk = [&](auto kconst) {
        constexpr bool K = decltype(kconst)::value;
        V y0[kU], c0[kU], i0[kU];
#pragma unroll
        for (int j = 0; j < kU; ++j) {
            y0[j] = y4[j];
            c0[j] = K ? kc2 : Ls::mk(-cA[j], -cB[j]);
            i0[j] = K ? ki2 : Ls::mk(iA[j], iB[j]);
        }
        // (inside [klo, khi), klo >= kU: the rows read ahead are >= 0)
#pragma unroll
        for (int j = 0; j < kU; ++j) y4[j] = pr[(K ? n - kU - j : max(n - kU - j, 0)) * P];
        if (!K) {
            const int kb = N - 2 - (n - kU);
            load4(oa.cbk + kb, cA); load4(ob.cbk + kb, cB);
            load4(oa.ibk + kb, iA); load4(ob.ibk + kb, iB);
        }
#pragma unroll
        for (int j = 0; j < kU; ++j) {
            x = Ls::mul(Ls::fma_(c0[j], x, y0[j]), i0[j]);
            pr[(n - j) * P] = x;
        }
    };
    for (; n - kU + 1 >= 0 && n >= khi; n -= kU) bwd_chunk(std::false_type{});
    if (n - kU + 1 >= klo) {
#pragma unroll 2
        for (; n - kU + 1 >= klo; n -= kU) bwd_chunk(std::true_type{});
        const int kb = N - 2 - n;
        load4(oa.cbk + kb, cA); load4(ob.cbk + kb, cB);
        load4(oa.ibk + kb, iA); load4(ob.ibk + kb, iB);
    }
#pragma unroll 2
    for (; n - kU + 1 >= 0; n -= kU) bwd_chunk(std::false_type{});
    for (; n >= 0; --n) {
        x = Ls::mul(Ls::fma_(Ls::mk(-ldc(&ca_[n]), -ldc(&cb_[n])), x, pr[n * P]),
                    Ls::mk(ldc(&ia[n]), ldc(&ib[n])));
        pr[n * P] = x;
    }
    *fa = oa.periodic ? (S)((to_f64(Ls::la(x)) + oa.bog * to_f64(Ls::la(xl))) * oa.inv_den) : S(0);
    if constexpr (NL == 2)
        *fb = ob.periodic ? (S)((to_f64(Ls::lb(x)) + ob.bog * to_f64(Ls::lb(xl))) * ob.inv_den) : S(0);
}

// Row n of the explicit right-hand side of a line read from src (stride P):
// the interior stencil, or the explicit boundary row (wrapped columns), with
// the products summed in the same order as solve_lanes.
template <typename T, int H>
__device__ __forceinline__ T rhs_row(const T *src, int P, const LineOp<T> &op, int n) {
    const int N = op.N;
    T acc = T(0);
    if (n >= H && n < N - H) {
#pragma unroll
        for (int k = 0; k < 2 * H + 1; ++k) acc = fma(op.taps[kMaxH - H + k], src[(n - H + k) * P], acc);
        return acc;
    }
    const int b = n < H ? n : n - (N - H) + H;
    const int col = op.boff[b];
#pragma unroll
    for (int k = 0; k < kTaps; ++k) {
        int cc = col + k;
        cc = cc < 0 ? cc + N : (cc >= N ? cc - N : cc);
        acc = fma(op.btaps[b][k], src[cc * P], acc);
    }
    return acc;
}

// One Thomas solve in place on a line whose right-hand side is already in d
// (stride P, a compile-time constant when PC > 0).  Rows outside [klo, khi)
// load their factors; rows inside run on the register constants km, kiw, kc
// in chunks of kU with the next chunk's values read ahead (reads past the
// body stay inside the line).  The operations and their order are those of
// solve_lanes, so the results are the same bit for bit.
template <typename T, int PC>
__device__ __forceinline__ void thomas_inplace(T *d, const LineOp<T> &op, T *fac, int P_) {
    const int P = PC > 0 ? PC : P_;
    const int N = op.N, lo = op.klo, hi = op.khi;
    const T km = op.km, kiw = op.kiw, kc = op.kc;
    // forward: y_0 = r_0, y_n = r_n - m_n y_{n-1}
    T y = d[0];
    int n = 1;
    for (; n < lo; ++n) {
        y = fma(-ldc(&op.m[n]), y, d[n * P]);
        d[n * P] = y;
    }
    if (n + kU <= hi) {
        T rn[kU];
#pragma unroll
        for (int j = 0; j < kU; ++j) rn[j] = d[(n + j) * P];
#pragma unroll 2
        for (; n + kU <= hi; n += kU) {
            T rc[kU];
#pragma unroll
            for (int j = 0; j < kU; ++j) rc[j] = rn[j];
            if (n + 2 * kU <= hi) {
#pragma unroll
                for (int j = 0; j < kU; ++j) rn[j] = d[(n + kU + j) * P];
            }
#pragma unroll
            for (int j = 0; j < kU; ++j) {
                y = fma(-km, y, rc[j]);
                d[(n + j) * P] = y;
            }
        }
    }
    for (; n < hi; ++n) {
        y = fma(-km, y, d[n * P]);
        d[n * P] = y;
    }
    for (; n < N; ++n) {
        y = fma(-ldc(&op.m[n]), y, d[n * P]);
        d[n * P] = y;
    }
    // backward: x_{N-1} = y_{N-1} iw_{N-1}, x_n = (y_n - c_n x_{n+1}) iw_n
    T x = y * ldc(&op.iw[N - 1]);
    d[(N - 1) * P] = x;
    const T xl = x;
    n = N - 2;
    for (; n >= hi; --n) {
        x = fma(-ldc(&op.c[n]), x, d[n * P]) * ldc(&op.iw[n]);
        d[n * P] = x;
    }
    if (n - kU + 1 >= lo) {
        T y4[kU];
#pragma unroll
        for (int j = 0; j < kU; ++j) y4[j] = d[(n - j) * P];
#pragma unroll 2
        for (; n - kU + 1 >= lo; n -= kU) {
            T y0[kU];
#pragma unroll
            for (int j = 0; j < kU; ++j) y0[j] = y4[j];
            if (n - 2 * kU + 1 >= lo) {
#pragma unroll
                for (int j = 0; j < kU; ++j) y4[j] = d[(n - kU - j) * P];
            }
#pragma unroll
            for (int j = 0; j < kU; ++j) {
                x = fma(-kc, x, y0[j]) * kiw;
                d[(n - j) * P] = x;
            }
        }
    }
    for (; n >= lo; --n) {
        x = fma(-kc, x, d[n * P]) * kiw;
        d[n * P] = x;
    }
    for (; n >= 0; --n) {
        x = fma(-ldc(&op.c[n]), x, d[n * P]) * ldc(&op.iw[n]);
        d[n * P] = x;
    }
    *fac = op.periodic ? (T)((to_f64(x) + op.bog * to_f64(xl)) * op.inv_den) : T(0);
}

// Corrected value of solution n of a line whose factor is f.
template <typename T>
__device__ __forceinline__ T corr(T x, T f, const LineOp<T> &op, int n) {
    return op.periodic ? fma(-f, ldc(&op.z[n]), x) : x;
}

// ---------------------------------------------------------------------
// tile geometry
// ---------------------------------------------------------------------
struct Tile {
    unsigned base;    // global index of (line 0, position 0)
    unsigned sl, sn;  // strides between lines and along a line
    int nlines;       // valid lines in this tile (<= L)
    int N;            // line length
    int ci, cj, ck;   // coordinates of (line 0, position 0)
};

// The tile of block coordinates (bx, by): bx counts tiles across the lines'
// transverse direction (rows j for x-lines, columns i otherwise), by the
// plane (k for x- and y-lines, row j for z-lines).
template <int DIR>
__device__ __forceinline__ Tile make_tile_at(const Geom &g, int L, int bx, int by) {
    Tile t;
    const unsigned nxy = (unsigned)g.Nx * (unsigned)g.Ny;
    if (DIR == 0) {  // x-lines at rows j0.., plane k
        int j0 = bx * L, k = by;
        t.base = (unsigned)k * nxy + (unsigned)j0 * g.Nx;
        t.sl = g.Nx; t.sn = 1;
        t.nlines = min(L, g.Ny - j0);
        t.N = g.Nx;
        t.ci = 0; t.cj = j0; t.ck = k;
    } else if (DIR == 1) {  // y-lines at columns i0.., plane k
        int i0 = bx * L, k = by;
        t.base = (unsigned)k * nxy + i0;
        t.sl = 1; t.sn = g.Nx;
        t.nlines = min(L, g.Nx - i0);
        t.N = g.Ny;
        t.ci = i0; t.cj = 0; t.ck = k;
    } else {  // z-lines at columns i0.., row j
        int i0 = bx * L, j = by;
        t.base = (unsigned)j * g.Nx + i0;
        t.sl = 1; t.sn = nxy;
        t.nlines = min(L, g.Nx - i0);
        t.N = g.Nz;
        t.ci = i0; t.cj = j; t.ck = 0;
    }
    return t;
}

template <int DIR>
__device__ __forceinline__ Tile make_tile(const Geom &g, int L) {
    return make_tile_at<DIR>(g, L, blockIdx.x, blockIdx.y);
}

// Point p of a tile: consecutive threads touch consecutive global addresses
// (position-major for x-lines, line-major otherwise).  L is a power of two
// (lgL its logarithm); division by the x-line length uses a precomputed
// multiplier (divN: p / N = (umulhi(p, mul) + p) >> sh for p < 2^31).
struct Pt {
    unsigned gi;   // global index (a valid address even when !ok)
    int o;         // shared-memory offset
    int l, n;
    bool ok;
};

// Point p of a tile: LF false walks along a line first (x tiles of the mixed
// form: a warp's loads cover contiguous x; the shared-memory pitch P = L + 1
// keeps the transposed stores off common banks); LF true walks across the
// tile's lines first (y and z tiles, whose lines are adjacent in memory, and
// the FP64 x tiles: 8-byte elements give each line a 32- or 64-byte run per
// warp, whole sectors, and the stores are then conflict-free at P = L).
template <int DIR, bool LF = (DIR != 0)>
__device__ __forceinline__ Pt point(const Tile &t, int p, int L, int P, int lgL, FastDiv dv) {
    Pt q;
    if (!LF) {
        q.l = (int)((__umulhi((unsigned)p, dv.mul) + (unsigned)p) >> dv.sh);
        q.n = p - q.l * t.N;
    } else {
        q.n = p >> lgL;
        q.l = p & (L - 1);
    }
    q.ok = q.l < t.nlines && q.n < t.N;
    q.gi = q.ok ? t.base + (unsigned)q.l * t.sl + (unsigned)q.n * t.sn : t.base;
    q.o = q.n * P + q.l;
    return q;
}

template <int DIR>
__device__ __forceinline__ void coords(const Tile &t, int l, int n, int &i, int &j, int &k) {
    if (DIR == 0) { i = n; j = t.cj + l; k = t.ck; }
    else if (DIR == 1) { i = t.ci + l; j = n; k = t.ck; }
    else { i = t.ci + l; j = t.cj; k = n; }
}

// ---------------------------------------------------------------------
// shared-memory layout of a tile: per-line factors, then nbuf buffers
// ---------------------------------------------------------------------
template <typename T>
struct Smem {
    T *buf;
    T *fact;  // [nbuf][L]
    int bstride;
    int P;
    int nbuf;
    __device__ T *b(int k) const { return buf + (size_t)k * bstride; }
    __device__ T &at(int k, int o) const { return buf[(size_t)k * bstride + o]; }
};

// Pair-interleaved layout of the FP32-mixed sweep tiles: buffers 2t and
// 2t+1 (the two solves of task t) share one float2 array, element (n, l) of
// the pair at float2 index n*P + l; pairs pstride floats apart with no rows
// of padding between them, pstride = 16 (mod 32) so that a warp whose
// one-lane solves span two tasks (tiles of 8 lines) covers distinct banks.
// Per-line factors stay planar: fact[k*L + l].
struct SmemPair {
    float *buf;
    float *fact;
    int pstride;
    int P;
    __device__ float2 *pair(int t) const { return reinterpret_cast<float2 *>(buf + (size_t)t * pstride); }
    __device__ float &at(int k, int o) const { return buf[(size_t)(k >> 1) * pstride + 2 * o + (k & 1)]; }
};

__host__ __device__ inline int pair_stride(int N, int P) {
    int st = 2 * N * P;
    st += ((16 - st % 32) + 32) % 32;
    return st;
}

// Elements between consecutive buffers.  The solve tasks of one warp use
// buffers two apart (A solves 0,2,4,..; B solves 1,3,5,..), each touching L
// consecutive lines: a stride s with 2*s*e = L*e (mod 32 banks), e the
// element size in 4-byte words, places the tasks of a warp on distinct banks.
__host__ __device__ inline int buf_stride(int N, int P, int L, int e) {
    const int mod = 16 / e;
    const int want = (L / 2) % mod;
    int st = N * P;
    st += ((want - st % mod) + mod) % mod;
    return st;
}

template <typename T>
__device__ __forceinline__ Smem<T> smem_layout_at(unsigned char *base, int nbuf, int L, int P, int N) {
    Smem<T> s;
    s.P = P;
    s.nbuf = nbuf;
    s.bstride = buf_stride(N + kPad, P, L, (int)(sizeof(T) / 4));
    s.fact = reinterpret_cast<T *>(base);
    const int nf = (nbuf * L + 3) & ~3;
    s.buf = reinterpret_cast<T *>(base) + nf;
    return s;
}

extern __shared__ __align__(16) unsigned char smem_raw[];

__device__ __forceinline__ SmemPair smem_pair_at(unsigned char *base, int nbuf, int L, int P, int N) {
    SmemPair s;
    s.P = P;
    s.pstride = pair_stride(N, P);
    s.fact = reinterpret_cast<float *>(base);
    const int nf = (nbuf * L + 3) & ~3;
    s.buf = reinterpret_cast<float *>(base) + nf;
    return s;
}

// The sweep kernels' tile layout: pair-interleaved in the FP32-mixed form,
// planar in the FP64 form.
template <typename T>
struct SweepSmem {
    using type = Smem<T>;
    static __device__ __forceinline__ type at(unsigned char *base, int nbuf, int L, int P, int N) {
        return smem_layout_at<T>(base, nbuf, L, P, N);
    }
};
template <>
struct SweepSmem<float> {
    using type = SmemPair;
    static __device__ __forceinline__ type at(unsigned char *base, int nbuf, int L, int P, int N) {
        return smem_pair_at(base, nbuf, L, P, N);
    }
};

template <typename T>
__device__ __forceinline__ Smem<T> smem_layout(int nbuf, int L, int P, int N) {
    return smem_layout_at<T>(smem_raw, nbuf, L, P, N);
}

// Right-hand sides of nf line solves per line, computed by every thread of
// the block: buffer dst0 + f gets the right-hand side of buffer src0 + f.
// A work item is 4 consecutive rows of one (field, line); interior items
// slide a register window over the 4 + 2H rows they need.  Lines are the
// fastest index, so a warp reads consecutive banks.
template <typename T, int H, int NF>
__device__ __forceinline__ void rhs_pass(const Smem<T> &sm, int src0, int dst0, int L, int lgL, int nlines,
                                         const LineOp<T> &op) {
    constexpr int R = 4;
    const int N = op.N, P = sm.P;
    const int ng = (N + R - 1) / R;
    for (int w = threadIdx.x; w < NF * ng * L; w += blockDim.x) {
        const int l = w & (L - 1), g = w >> lgL;
        if (l >= nlines) continue;
        const int f = g % NF, n0 = (g / NF) * R;
        const T *src = sm.b(src0 + f) + l;
        T *dst = sm.b(dst0 + f) + l;
        if (n0 >= H && n0 + R <= N - H) {
            T e[R + 2 * H];
#pragma unroll
            for (int k = 0; k < R + 2 * H; ++k) e[k] = src[(n0 - H + k) * P];
#pragma unroll
            for (int j = 0; j < R; ++j) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 2 * H + 1; ++k) acc = fma(op.taps[kMaxH - H + k], e[j + k], acc);
                dst[(n0 + j) * P] = acc;
            }
        } else {
            for (int n = n0; n < min(n0 + R, N); ++n) dst[n * P] = rhs_row<T, H>(src, P, op, n);
        }
    }
}

// Per-thread loop over the points of a tile with a software pipeline: the
// global loads of the thread's next point are issued before the current
// point is computed, so memory latency overlaps the arithmetic.
// ld(S&, p) loads point p; cp(S&) computes and stores it.
// tid / nthr: this thread's index among the nthr threads sharing the loop.
template <typename S, typename LD, typename CP>
__device__ __forceinline__ void pipelined(int NL, int tid, int nthr, LD &&ld, CP &&cp) {
    int p = tid;
    if (p >= NL) return;
    S s0, s1;
    ld(s0, p);
    for (;;) {
        const int p1 = p + nthr;
        if (p1 < NL) ld(s1, p1);
        cp(s0);
        if (p1 >= NL) break;
        const int p2 = p1 + nthr;
        if (p2 < NL) ld(s0, p2);
        cp(s1);
        if (p2 >= NL) break;
        p = p2;
    }
}

// Per-thread loop over the points of a tile in batches of B: the loads of B
// points are issued together, then the B points are computed and stored.
template <typename S, int B, typename LD, typename CP>
__device__ __forceinline__ void batched(int NL, int tid, int nthr, LD &&ld, CP &&cp) {
    for (int p0 = tid; p0 < NL; p0 += B * nthr) {
        S s[B];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int p = p0 + b * nthr;
            ld(s[b], p < NL ? p : p0);
            if (p >= NL) s[b].pt.ok = false;
        }
#pragma unroll
        for (int b = 0; b < B; ++b) cp(s[b]);
    }
}
template <typename S, int B, typename LD, typename CP>
__device__ __forceinline__ void batched(int NL, LD &&ld, CP &&cp) {
    batched<S, B>(NL, (int)threadIdx.x, (int)blockDim.x, ld, cp);
}

// A task: solve A (src a, dst da, operator oa) and solve B, run together.
// op: 0 = 1st derivative, 1 = 2nd derivative, 2 = filter.
struct Task {
    signed char a, da, oa, b, db, ob;
};

// The tasks of a sweep tile; sweep task t solves into buffers 2t and 2t+1.
// FP32-mixed: one lane of the pair-interleaved layout per thread, the lane
// whose destination buffer is `skip` (a task's unused duplicate) left out.
template <int H, int PC>
__device__ __forceinline__ void run_sweep_tasks(const SmemPair &sm, const Task *tasks, int ntask, int L, int nlines,
                                                const LineOp<float> &op0, const LineOp<float> &op1, int tid,
                                                int nthr, int skip = -1) {
    for (int w = tid; w < 2 * ntask * L; w += nthr) {
        // w = (task, line, lane), lane fastest: a warp holds 16 (task, line)
        // pairs' two lanes
        const int lane = w & 1, tl = w >> 1;
        const int t = tl / L, l = tl - t * L;
        if (l >= nlines) continue;
        const Task tk = tasks[t];
        const int op = lane ? tk.ob : tk.oa, dst = lane ? tk.db : tk.da;
        if (dst == skip) continue;
        // the other operator passed as B: its rows bound [klo, khi) too, so
        // both lanes of a task (one warp) leave the constant-factor run together
        solve_lanes<1, H, PC, float, 2>(reinterpret_cast<float *>(sm.pair(tk.da >> 1) + l) + lane,
                                        op == 1 ? op1 : op0, &sm.fact[dst * L + l], op == 1 ? op0 : op1, nullptr,
                                        sm.P);
    }
}
// The plain FP64 sweeps' solves: one solve per thread, in place in its
// destination buffer (the load phase stores a field whose two solves read it
// in both of its task's buffers), the duplicate solve of a one-field task
// left out.  The mixed form is run_sweep_tasks.
template <int H, int PC>
__device__ __forceinline__ void run_sweep_solves(const Smem<double> &sm, const Task *tasks, int ntask, int L,
                                                 int nlines, const LineOp<double> &op0, const LineOp<double> &op1,
                                                 int tid, int nthr, int = -1) {
    for (int w = tid; w < 2 * ntask * L; w += nthr) {
        const int lane = w & 1, tl = w >> 1;
        const int t = tl / L, l = tl - t * L;
        if (l >= nlines) continue;
        const Task tk = tasks[t];
        if (lane && tk.db == tk.da) continue;
        const int op = lane ? tk.ob : tk.oa, dst = lane ? tk.db : tk.da;
        solve_lanes<1, H, PC, double, 1>(sm.b(dst) + l, op == 1 ? op1 : op0, &sm.fact[dst * L + l],
                                         op == 1 ? op0 : op1, nullptr, sm.P);
    }
}
template <int H, int PC>
__device__ __forceinline__ void run_sweep_solves(const SmemPair &sm, const Task *tasks, int ntask, int L,
                                                 int nlines, const LineOp<float> &op0, const LineOp<float> &op1,
                                                 int tid, int nthr, int skip) {
    run_sweep_tasks<H, PC>(sm, tasks, ntask, L, nlines, op0, op1, tid, nthr, skip);
}

// Phase-A stores of task t's inputs at offset o: put1 for a task whose two
// solves read one field, put2 for two fields.  In the pair layout both are
// one 64-bit store (put1 stores the field in both lanes); in the planar
// layout put1 stores the field in both of the task's buffers (each solve runs
// in place), or in its one buffer where the task's last buffer is the tile's
// last (a one-field task).
__device__ __forceinline__ void put1(const SmemPair &sm, int t, int o, float v) { sm.pair(t)[o] = make_float2(v, v); }
__device__ __forceinline__ void put2(const SmemPair &sm, int t, int o, float v0, float v1) {
    sm.pair(t)[o] = make_float2(v0, v1);
}
template <typename T>
__device__ __forceinline__ void put1(const Smem<T> &sm, int t, int o, T v) {
    sm.at(2 * t, o) = v;
    if (2 * t + 1 < sm.nbuf) sm.at(2 * t + 1, o) = v;
}
template <typename T>
__device__ __forceinline__ void put2(const Smem<T> &sm, int t, int o, T v0, T v1) {
    sm.at(2 * t, o) = v0;
    sm.at(2 * t + 1, o) = v1;
}

// Corrected solutions (Sherman-Morrison term -f z, f the buffer's line factor,
// z the operator's vector at the point) of task t's two buffers at point p,
// and of one buffer k.
__device__ __forceinline__ void get2(const SmemPair &sm, int t, const Pt &p, int L, float za, float zb, float &a,
                                     float &b) {
    const float2 v = sm.pair(t)[p.o];
    a = fmaf(-sm.fact[(2 * t) * L + p.l], za, v.x);
    b = fmaf(-sm.fact[(2 * t + 1) * L + p.l], zb, v.y);
}
template <typename T>
__device__ __forceinline__ void get2(const Smem<T> &sm, int t, const Pt &p, int L, T za, T zb, T &a, T &b) {
    a = fma(-sm.fact[(2 * t) * L + p.l], za, sm.at(2 * t, p.o));
    b = fma(-sm.fact[(2 * t + 1) * L + p.l], zb, sm.at(2 * t + 1, p.o));
}
template <typename SM, typename T>
__device__ __forceinline__ T get1(const SM &sm, int k, const Pt &p, int L, T z) {
    return fma(-sm.fact[k * L + p.l], z, sm.at(k, p.o));
}

template <typename T>
__device__ __forceinline__ T get(const Smem<T> &sm, int k, const Pt &p, int L, const LineOp<T> &op) {
    return corr<T>(sm.b(k)[p.o], sm.fact[k * L + p.l], op, p.n);
}

// Sherman-Morrison vectors of the 1st and 2nd derivative at position n
// (zero for wall lines), loaded once per point.
template <typename T>
struct Zn {
    T z1, z2;
};
template <typename T>
__device__ __forceinline__ Zn<T> zn(const LineOp<T> &d1, const LineOp<T> &d2, int n) {
    Zn<T> z;
    z.z1 = d1.periodic ? ldc(&d1.z[n]) : T(0);
    z.z2 = d2.periodic ? ldc(&d2.z[n]) : T(0);
    return z;
}
// ---------------------------------------------------------------------
// primitives of one point (IdealGas.hpp:49-80)
// ---------------------------------------------------------------------
template <typename T>
struct PrimW {
    T ru, rv, rw, re, U, V, W, p, Tt;
};

template <typename T>
__device__ __forceinline__ PrimW<T> prim_w(const GasParams &gp, T r0, T r1, T r2, T r3, T r4) {
    PrimW<T> s;
    s.ru = r1; s.rv = r2; s.rw = r3; s.re = r4;
    if constexpr (sizeof(T) == 8) {
        // one correctly rounded reciprocal of rho instead of four FP64
        // divisions (within an ulp of the quotients)
        const double ir = __drcp_rn(r0);
        s.U = r1 * ir;
        s.V = r2 * ir;
        s.W = r3 * ir;
        s.p = gp.gm1 * (r4 - 0.5 * r0 * (s.U * s.U + s.V * s.V + s.W * s.W));
        s.Tt = s.p * ir * (1.0 / gp.R);  // 1/R: invariant, formed once per thread
    } else {
        // FP32 keeps the quotients: the reciprocal's rounding, shared by the
        // points of a region of near-uniform density, doubled the mixed
        // form's error in the shear layer's fluctuation statistics
        s.U = r1 / r0;
        s.V = r2 / r0;
        s.W = r3 / r0;
        s.p = (T)gp.gm1 * (r4 - T(0.5) * r0 * (s.U * s.U + s.V * s.V + s.W * s.W));
        s.Tt = s.p / (r0 * (T)gp.R);
    }
    return s;
}

}  // namespace cs3d
