// cs3d_adjoint.cu -- kernels of the discrete adjoint of one RK stage
// (sm_103a), periodic boundaries.
//
// The stage's right-hand side is R(q) = P(G(q)): G holds, per point, the
// primitives U, V, W, T and 44 derivative values (first and second
// derivatives of U, V, W, T along x, y, z; d/dx of the five x-fluxes and so
// on; the cross derivatives Uxy, Vxy, d/dz(Ux+Vy), Wxz, Wyz), and P is the
// pointwise combination of the sweep kernels.  Its transposed Jacobian is
//
//   J^T lam = C^T [ D^T (dP/dG)^T lam ]
//
// with dP/dG from the generated rhs_vjp, D^T the transposed line operators,
// and C^T the pointwise chain rule through the fluxes and primitives.  On a
// periodic uniform grid every compact operator is A^-1 B with A and B
// circulant; A is symmetric, B of the 1st derivative antisymmetric and B of
// the 2nd derivative and the filter symmetric, and circulants commute, so
//   D1^T = -D1,  D2^T = D2,  F^T = F,
// which k_apply evaluates with the forward solve and a sign.
#include <cstdio>
#include <cmath>
#include "cs3d_tile.cuh"
#include "cs3d_rhs_adjoint.cuh"

namespace cs3d {

constexpr int kTMinBlocksX = 3;  // resident blocks per SM the transposed x sweep is compiled for

// ---------------------------------------------------------------------
// line operators along DIR on XYZ-layout fields
// ---------------------------------------------------------------------
// Tasks 2i and 2i+1 share a solve pair; in FP32 the tile is pair-interleaved
// (an odd last task pairs with a copy of itself in a spare buffer) and the
// loads and stores run several points per thread in flight, as in the sweeps.
// Destinations are read (where a task adds) together with the sources, so no
// store waits on a load.
// F64IO: every task reads an FP64 field (narrowed to T) and adds its result
// into an FP64 field.
template <typename T, int DIR, int H, bool F64IO = false>
__global__ void __launch_bounds__(apply_threads<T>()) k_apply(ApplyArgs<T> a) {
    constexpr bool kPair = sizeof(T) == 4;
    constexpr int BL = kPair ? 4 : 2, BS = 2;  // points per thread in flight: loads, stores
    const int L = a.L, P = a.P;
    const Tile t = make_tile<DIR>(a.g, L);
    const int N = t.N, NL = N * L;
    const int nt = a.ntask, np = (nt + 1) / 2;
    const auto sm = SweepSmem<T>::at(smem_raw, kPair ? 2 * np : nt, L, P, N);
    __shared__ Task tasks[kApplyMax / 2];
    if ((int)threadIdx.x < np) {
        const int i = 2 * threadIdx.x, j = min(i + 1, nt - 1);
        tasks[threadIdx.x] = Task{(signed char)i, (signed char)i, (signed char)a.t[i].op,
                                  (signed char)(kPair ? i + 1 : j), (signed char)(kPair ? i + 1 : j),
                                  (signed char)a.t[j].op};
    }
    struct In { Pt pt; T v[kApplyMax]; };
    batched<In, BL>(NL,
        [&](In &in, int p) {
            in.pt = point<DIR>(t, p, L, P, a.lgL, a.divN);
            const unsigned gi = in.pt.gi;
#pragma unroll
            for (int k = 0; k < kApplyMax; ++k) {
                if (k >= nt) break;
                if constexpr (F64IO) {
                    in.v[k] = to_work<T>(a.t[k].src64[gi]);
                } else {
                    T v = a.t[k].src[gi];
                    if (a.t[k].src2) v += a.t[k].src2[gi];
                    in.v[k] = v;
                }
            }
        },
        [&](In &in) {
            if (!in.pt.ok) return;
            const int o = in.pt.o;
#pragma unroll
            for (int k = 0; k < kApplyMax; k += 2) {
                if (k >= nt) break;
                if constexpr (kPair) {
                    // (an odd last task pairs with a copy of itself)
                    const T second = k + 1 < kApplyMax && k + 1 < nt ? in.v[k + 1 < kApplyMax ? k + 1 : k] : in.v[k];
                    put2(sm, k / 2, o, in.v[k], second);
                }
                else {
                    sm.at(k, o) = in.v[k];
                    if (k + 1 < nt) sm.at(k + 1, o) = in.v[k + 1];
                }
            }
        });
    __syncthreads();
    // FP64: one solve per thread, each task in place in its own buffer
    run_sweep_solves<H, 0>(sm, tasks, np, L, t.nlines, a.op0, a.op1, (int)threadIdx.x, (int)blockDim.x, -1);
    __syncthreads();
    if constexpr (F64IO) {
        struct Out64 { Pt pt; double e[kApplyMax]; };
        batched<Out64, BS>(NL,
            [&](Out64 &o, int p) {
                o.pt = point<DIR>(t, p, L, P, a.lgL, a.divN);
#pragma unroll
                for (int k = 0; k < kApplyMax; ++k) {
                    if (k >= nt) break;
                    o.e[k] = a.t[k].dst64[o.pt.gi];
                }
            },
            [&](Out64 &o) {
                if (!o.pt.ok) return;
#pragma unroll
                for (int k = 0; k < kApplyMax; ++k) {
                    if (k >= nt) break;
                    const ApplyTask<T> &tk = a.t[k];
                    const LineOp<T> &op = tk.op == 1 ? a.op1 : a.op0;
                    const T z = op.periodic ? ldc(&op.z[o.pt.n]) : T(0);
                    tk.dst64[o.pt.gi] = o.e[k] + to_f64(tk.scale * get1(sm, k, o.pt, L, z));
                }
            });
        return;
    }
    struct Out { Pt pt; T d[kApplyMax], d2[kApplyMax]; };
    batched<Out, BS>(NL,
        [&](Out &o, int p) {
            o.pt = point<DIR>(t, p, L, P, a.lgL, a.divN);
            const unsigned gi = o.pt.gi;
#pragma unroll
            for (int k = 0; k < kApplyMax; ++k) {
                if (k >= nt) break;
                const ApplyTask<T> &tk = a.t[k];
                const bool second = (k & 1) && a.merge[k / 2];
                o.d[k] = (tk.dst && tk.acc && !second) ? tk.dst[gi] : T(0);
                o.d2[k] = tk.dst2 ? tk.dst2[gi] : T(0);
            }
        },
        [&](Out &o) {
            if (!o.pt.ok) return;
            const unsigned gi = o.pt.gi;
            const int n = o.pt.n;
#pragma unroll
            for (int k = 0; k < kApplyMax; ++k) {
                if (k >= nt) break;
                const ApplyTask<T> &tk = a.t[k];
                const LineOp<T> &op = tk.op == 1 ? a.op1 : a.op0;
                const T z = op.periodic ? ldc(&op.z[n]) : T(0);
                const T v = tk.scale * get1(sm, k, o.pt, L, z);
                if ((k & 1) && a.merge[k / 2]) {
                    // the pair's one destination: (first task's result) then this task
                    const T r = tk.acc ? o.d[k - 1] + v : v;
                    tk.dst[gi] = r;
                } else if ((k & 1) == 0 && k + 1 < nt && a.merge[k / 2]) {
                    o.d[k] = tk.acc ? o.d[k] + v : v;  // carried to task k + 1
                } else if (tk.dst) {
                    tk.dst[gi] = tk.acc ? o.d[k] + v : v;
                }
                if (tk.dst2) tk.dst2[gi] = o.d2[k] + v;
            }
        });
}

// ---------------------------------------------------------------------
// transposed sweeps (FP32-mixed adjoint)
// ---------------------------------------------------------------------
// The transposed line operators of one direction in one launch, laid out as
// the forward sweep of that direction: pair t holds two cotangent fields
// (the 1st and 2nd derivative entries of U, V, W, T, then the 1st-derivative
// entries two by two; an odd last pair repeats its field in a spare buffer),
// solved with the forward operators; the consume phase applies the signs of
// D1^T = -D1, D2^T = D2 and adds each result to its destination in the order
// the tape's formulas used them.  Cotangent entries of the fluxes (CE, F/G/H)
// are replaced in place; those of U, V, W, T and of the x/y derivatives that
// a later direction differentiates (Ux, Vy, Wx, Wy from z; Ux, Vx from y) are
// added to.
__constant__ Task kTasksT[8] = {{0, 0, 0, 1, 1, 1}, {2, 2, 0, 3, 3, 1}, {4, 4, 0, 5, 5, 1}, {6, 6, 0, 7, 7, 1},
                                {8, 8, 0, 9, 9, 0}, {10, 10, 0, 11, 11, 0}, {12, 12, 0, 13, 13, 0},
                                {14, 14, 0, 15, 15, 0}};

// cotangent entries solved along DIR, lane by lane (-1: the spare buffer)
template <int DIR>
struct TSweepSrc;
template <>
struct TSweepSrc<2> {
    static constexpr int n = 16;
    static __host__ __device__ constexpr int e(int k) {
        constexpr int v[16] = {kInUz, kInUzz, kInVz,  kInVzz, kInWz,  kInWzz, kInTz,  kInTzz,
                               kInS,  kInWxz, kInWyz, kInCEz, kInH1z, kInH2z, kInH3z, kInH4z};
        return v[k];
    }
};
template <>
struct TSweepSrc<1> {
    static constexpr int n = 15;
    static __host__ __device__ constexpr int e(int k) {
        constexpr int v[16] = {kInUy,  kInUyy, kInVy,  kInVyy, kInWy,  kInWyy, kInTy,  kInTyy,
                               kInUxy, kInVxy, kInCEy, kInG1y, kInG2y, kInG3y, kInG4y, -1};
        return v[k];
    }
};
template <>
struct TSweepSrc<0> {
    static constexpr int n = 13;
    static __host__ __device__ constexpr int e(int k) {
        constexpr int v[16] = {kInUx,  kInUxx, kInVx,  kInVxx, kInWx, kInWxx, kInTx, kInTxx,
                               kInCEx, kInF1x, kInF2x, kInF3x, kInF4x, -1,    -1,    -1};
        return v[k];
    }
};

template <int DIR, int PC>
__global__ void __launch_bounds__(sweep_threads<float>(DIR), DIR == 0 ? kTMinBlocksX : 1) k_tsweep(TSweepArgs a) {
    using S = TSweepSrc<DIR>;
    constexpr int NP = (S::n + 1) / 2;
    const int L = a.L, P = PC > 0 ? PC : a.P;
    const Tile t = make_tile<DIR>(a.g, L);
    const int N = t.N, NL = N * L;
    const SmemPair sm = smem_pair_at(smem_raw, 2 * NP, L, P, N);
    float *const *B = a.gbar;
    struct In { Pt pt; float v[S::n]; };
    batched<In, 4>(NL,
        [&](In &in, int p) {
            in.pt = point<DIR>(t, p, L, P, a.lgL, a.divN);
#pragma unroll
            for (int k = 0; k < S::n; ++k) in.v[k] = B[S::e(k)][in.pt.gi];
        },
        [&](In &in) {
            if (!in.pt.ok) return;
#pragma unroll
            for (int q = 0; q < NP; ++q) put2(sm, q, in.pt.o, in.v[2 * q], in.v[2 * q + 1 < S::n ? 2 * q + 1 : 2 * q]);
        });
    __syncthreads();
    run_sweep_tasks<2, PC>(sm, kTasksT, NP, L, t.nlines, a.d1, a.d2, threadIdx.x, blockDim.x);
    __syncthreads();
    // destinations added to: U V W T, then (z) Ux Vy Wx Wy / (y) Ux Vx
    constexpr int ND = DIR == 2 ? 8 : DIR == 1 ? 6 : 4;
    struct Out { Pt pt; float d[ND]; };
    batched<Out, 2>(NL,
        [&](Out &o, int p) {
            o.pt = point<DIR>(t, p, L, P, a.lgL, a.divN);
            const unsigned gi = o.pt.gi;
#pragma unroll
            for (int f = 0; f < 4; ++f) o.d[f] = B[kInU + f][gi];
            if constexpr (DIR == 2) {
                o.d[4] = B[kInUx][gi]; o.d[5] = B[kInVy][gi]; o.d[6] = B[kInWx][gi]; o.d[7] = B[kInWy][gi];
            } else if constexpr (DIR == 1) {
                o.d[4] = B[kInUx][gi]; o.d[5] = B[kInVx][gi];
            }
        },
        [&](Out &o) {
            if (!o.pt.ok) return;
            const Pt &p = o.pt;
            const unsigned gi = p.gi;
            const Zn<float> zz = zn(a.d1, a.d2, p.n);
            float g[2 * NP];
#pragma unroll
            for (int q = 0; q < NP; ++q)
                get2(sm, q, p, L, zz.z1, q < 4 ? zz.z2 : zz.z1, g[2 * q], g[2 * q + 1]);
            // U V W T: (dst + (-D1 g_d)) + D2 g_dd
#pragma unroll
            for (int f = 0; f < 4; ++f) B[kInU + f][gi] = (o.d[f] + (-g[2 * f])) + g[2 * f + 1];
            if constexpr (DIR == 2) {
                B[kInUx][gi] = o.d[4] + (-g[8]);
                B[kInVy][gi] = o.d[5] + (-g[8]);
                B[kInWx][gi] = o.d[6] + (-g[9]);
                B[kInWy][gi] = o.d[7] + (-g[10]);
#pragma unroll
                for (int k = 11; k < 16; ++k) B[S::e(k)][gi] = -g[k];
            } else if constexpr (DIR == 1) {
                B[kInUx][gi] = o.d[4] + (-g[8]);
                B[kInVx][gi] = o.d[5] + (-g[9]);
#pragma unroll
                for (int k = 10; k < 15; ++k) B[S::e(k)][gi] = -g[k];
            } else {
#pragma unroll
                for (int k = 8; k < 13; ++k) B[S::e(k)][gi] = -g[k];
            }
        });
}

// ---------------------------------------------------------------------
// pointwise parts
// ---------------------------------------------------------------------
__device__ __forceinline__ long long gstride() { return (long long)gridDim.x * blockDim.x; }
__device__ __forceinline__ long long gfirst() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }

// primitives and the Euler fluxes of the sweeps (the x, y, z phase A inputs)
template <typename T>
__global__ void k_tape_prep(TapePrepArgs<T> a) {
    for (long long gi = gfirst(); gi < a.g.npts; gi += gstride()) {
        const PrimW<T> s = prim_w<T>(a.gas, a.qin[0][gi], a.qin[1][gi], a.qin[2][gi], a.qin[3][gi], a.qin[4][gi]);
        a.prim[0][gi] = s.U; a.prim[1][gi] = s.V; a.prim[2][gi] = s.W; a.prim[3][gi] = s.Tt;
        a.flux[0][gi] = s.ru;
        a.flux[1][gi] = s.ru * s.U + s.p;
        a.flux[2][gi] = s.rv * s.U;
        a.flux[3][gi] = s.rw * s.U;
        a.flux[4][gi] = s.re * s.U + s.U * s.p;
        a.flux[5][gi] = s.rv;
        a.flux[6][gi] = s.ru * s.V;
        a.flux[7][gi] = s.rv * s.V + s.p;
        a.flux[8][gi] = s.rw * s.V;
        a.flux[9][gi] = s.re * s.V + s.V * s.p;
        a.flux[10][gi] = s.rw;
        a.flux[11][gi] = s.ru * s.W;
        a.flux[12][gi] = s.rv * s.W;
        a.flux[13][gi] = s.rw * s.W + s.p;
        a.flux[14][gi] = s.re * s.W + s.W * s.p;
    }
}

// gbar = (dP/dG)^T lam at every point
template <typename T>
__global__ void __launch_bounds__(128) k_vjp(VjpArgs<T> a) {
    const T muref = (T)a.gas.mu_ref, cpPr = (T)a.gas.cpPr;
    for (long long gi = gfirst(); gi < a.g.npts; gi += gstride()) {
        T in[kRhsIn], l[5], out[kRhsIn];
#pragma unroll
        for (int i = 0; i < kRhsIn; ++i) in[i] = a.tape[i][gi];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            if (a.qb2[0]) {
                double v = a.ca * a.qb2[f][gi];
                if (a.yt[0]) v += a.cb * a.yt[f][gi];
                l[f] = (T)v;
            } else {
                l[f] = (T)a.lam[f][gi];
            }
        }
        rhs_vjp<T>(in, l, muref, cpPr, out);
#pragma unroll
        for (int i = 0; i < kRhsIn; ++i) a.gbar[i][gi] = out[i];
    }
}

// R = P(G): the right-hand side from the tape (checks the tape)
template <typename T>
__global__ void k_rhs_eval(RhsEvalArgs<T> a) {
    const T muref = (T)a.gas.mu_ref, cpPr = (T)a.gas.cpPr;
    for (long long gi = gfirst(); gi < a.g.npts; gi += gstride()) {
        T in[kRhsIn], R[5];
#pragma unroll
        for (int i = 0; i < kRhsIn; ++i) in[i] = a.tape[i][gi];
        rhs_eval<T>(in, muref, cpPr, R);
#pragma unroll
        for (int f = 0; f < 5; ++f) a.R[f][gi] = (double)R[f];
    }
}

// out = C^T gbar: the flux cotangents (gbar slots of CEx..F4x, CEy..G4y,
// CEz..H4z after the transposed operators) and the primitive cotangents
// (slots U, V, W, T) taken back to the conserved variables through
//   fluxes  x: rhoU, rhoU U + p, rhoV U, rhoW U, (rhoE + p) U  (y, z alike)
//   U = rhoU/rho, ..., p = (gamma-1)(rhoE - (rhoU^2+rhoV^2+rhoW^2)/(2 rho)),
//   T = p / (rho R).
template <typename T>
__global__ void k_chain(ChainArgs<T> a) {
    const T gm1 = (T)a.gas.gm1, Rg = (T)a.gas.R;
    for (long long gi = gfirst(); gi < a.g.npts; gi += gstride()) {
        const PrimW<T> s = prim_w<T>(a.gas, a.qin[0][gi], a.qin[1][gi], a.qin[2][gi], a.qin[3][gi], a.qin[4][gi]);
        const T r = a.qin[0][gi];
        const T U = s.U, V = s.V, W = s.W, p = s.p;
        const T ru = s.ru, rv = s.rv, rw = s.rw, rep = s.re + s.p;
        T ax[5], ay[5], az[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            ax[k] = a.gbar[kInCEx + k][gi];
            ay[k] = a.gbar[kInCEy + k][gi];
            az[k] = a.gbar[kInCEz + k][gi];
        }
        T gU = a.gbar[kInU][gi], gV = a.gbar[kInV][gi], gW = a.gbar[kInW][gi];
        const T gT = a.gbar[kInT][gi];
        T gr = T(0), gru = T(0), grv = T(0), grw = T(0), gre = T(0), gp = T(0);
        // x fluxes
        gru += ax[0] + ax[1] * U;
        grv += ax[2] * U;
        grw += ax[3] * U;
        gre += ax[4] * U;
        gU += ax[1] * ru + ax[2] * rv + ax[3] * rw + ax[4] * rep;
        gp += ax[1] + ax[4] * U;
        // y fluxes
        grv += ay[0] + ay[2] * V;
        gru += ay[1] * V;
        grw += ay[3] * V;
        gre += ay[4] * V;
        gV += ay[1] * ru + ay[2] * rv + ay[3] * rw + ay[4] * rep;
        gp += ay[2] + ay[4] * V;
        // z fluxes
        grw += az[0] + az[3] * W;
        gru += az[1] * W;
        grv += az[2] * W;
        gre += az[4] * W;
        gW += az[1] * ru + az[2] * rv + az[3] * rw + az[4] * rep;
        gp += az[3] + az[4] * W;
        // T = p / (rho R)
        gp += gT / (r * Rg);
        gr -= gT * s.Tt / r;
        // primitives -> conserved
        const T ir = T(1) / r;
        gr += -(U * gU + V * gV + W * gW) * ir + gp * gm1 * T(0.5) * (U * U + V * V + W * W);
        gru += gU * ir - gm1 * U * gp;
        grv += gV * ir - gm1 * V * gp;
        grw += gW * ir - gm1 * W * gp;
        gre += gm1 * gp;
        const double o[5] = {(double)gr, (double)gru, (double)grv, (double)grw, (double)gre};
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            a.out[f][gi] = o[f];
            if (a.acc[0]) a.acc[f][gi] = a.acc_set ? o[f] : a.acc[f][gi] + o[f];
        }
    }
}

__global__ void k_lin5(Lin5Args a) {
    for (long long i = gfirst(); i < a.n; i += gstride()) {
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            double v = a.a * a.x[f][i];
            if (a.y[f]) v += a.b * a.y[f][i];
            if (a.z[f]) v += a.c * a.z[f][i];
            a.out[f][i] = v;
        }
    }
}

__global__ void k_ke_seed(KeSeedArgs a) {
    const double inv_n = 1.0 / (double)a.g.npts;
    double s = 0.0;
    for (long long gi = gfirst(); gi < a.g.npts; gi += gstride()) {
        const double r = a.q.f[0][gi];
        const double U = a.q.f[1][gi] / r, V = a.q.f[2][gi] / r, W = a.q.f[3][gi] / r;
        const double k2 = U * U + V * V + W * W;
        s += r * k2 / 2.0;
        a.seed[0][gi] = -0.5 * k2 * inv_n;
        a.seed[1][gi] = U * inv_n;
        a.seed[2][gi] = V * inv_n;
        a.seed[3][gi] = W * inv_n;
        a.seed[4][gi] = 0.0;
    }
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
        a.part[blockIdx.x] = v;
    }
}

// ---------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------
static int pw_grid(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152 * 8) b = 152 * 8;
    return (int)(b < 1 ? 1 : b);
}

template <typename K, typename A>
static cudaError_t tile_launch(K kernel, const A &a, dim3 grid, size_t sm, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    kernel<<<grid, a.threads, sm, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_apply(int dir, int H, const ApplyArgs<T> &a, cudaStream_t s) {
    if (a.ntask < 1 || a.ntask > kApplyMax) return cudaErrorInvalidValue;
    const int N = dir == 0 ? a.g.Nx : dir == 1 ? a.g.Ny : a.g.Nz;
    const size_t sm = sweep_smem_bytes((int)sizeof(T), sizeof(T) == 4 ? 2 * ((a.ntask + 1) / 2) : a.ntask, a.L,
                                       a.P, N);
    const int L = a.L;
    dim3 grid = dir == 0 ? dim3((a.g.Ny + L - 1) / L, a.g.Nz)
                         : dir == 1 ? dim3((a.g.Nx + L - 1) / L, a.g.Nz) : dim3((a.g.Nx + L - 1) / L, a.g.Ny);
    if (H == 4 && a.f64io) {
        if (dir == 0) return tile_launch(k_apply<T, 0, 4, true>, a, grid, sm, s);
        if (dir == 1) return tile_launch(k_apply<T, 1, 4, true>, a, grid, sm, s);
        return tile_launch(k_apply<T, 2, 4, true>, a, grid, sm, s);
    }
    if (H == 4) {
        if (dir == 0) return tile_launch(k_apply<T, 0, 4>, a, grid, sm, s);
        if (dir == 1) return tile_launch(k_apply<T, 1, 4>, a, grid, sm, s);
        return tile_launch(k_apply<T, 2, 4>, a, grid, sm, s);
    }
    if (dir == 0) return tile_launch(k_apply<T, 0, 2>, a, grid, sm, s);
    if (dir == 1) return tile_launch(k_apply<T, 1, 2>, a, grid, sm, s);
    return tile_launch(k_apply<T, 2, 2>, a, grid, sm, s);
}

cudaError_t launch_tsweep(int dir, const TSweepArgs &a, cudaStream_t s) {
    const int N = dir == 0 ? a.g.Nx : dir == 1 ? a.g.Ny : a.g.Nz;
    const int nbuf = dir == 0 ? 14 : 16;
    const size_t sm = sweep_smem_bytes(4, nbuf, a.L, a.P, N);
    const int L = a.L;
    dim3 grid = dir == 0 ? dim3((a.g.Ny + L - 1) / L, a.g.Nz)
                         : dir == 1 ? dim3((a.g.Nx + L - 1) / L, a.g.Nz) : dim3((a.g.Nx + L - 1) / L, a.g.Ny);
    if (dir == 0 && a.P == 9) return tile_launch(k_tsweep<0, 9>, a, grid, sm, s);
    if (dir == 0 && a.P == 5) return tile_launch(k_tsweep<0, 5>, a, grid, sm, s);
    if (dir == 1 && a.P == 16) return tile_launch(k_tsweep<1, 16>, a, grid, sm, s);
    if (dir == 1 && a.P == 8) return tile_launch(k_tsweep<1, 8>, a, grid, sm, s);
    if (dir == 2 && a.P == 16) return tile_launch(k_tsweep<2, 16>, a, grid, sm, s);
    if (dir == 2 && a.P == 8) return tile_launch(k_tsweep<2, 8>, a, grid, sm, s);
    if (dir == 0) return tile_launch(k_tsweep<0, 0>, a, grid, sm, s);
    if (dir == 1) return tile_launch(k_tsweep<1, 0>, a, grid, sm, s);
    return tile_launch(k_tsweep<2, 0>, a, grid, sm, s);
}

template <typename T>
cudaError_t launch_tape_prep(const TapePrepArgs<T> &a, cudaStream_t s) {
    k_tape_prep<T><<<pw_grid(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_vjp(const VjpArgs<T> &a, cudaStream_t s) {
    k_vjp<T><<<pw_grid(a.g.npts, 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_chain(const ChainArgs<T> &a, cudaStream_t s) {
    k_chain<T><<<pw_grid(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_rhs_eval(const RhsEvalArgs<T> &a, cudaStream_t s) {
    k_rhs_eval<T><<<pw_grid(a.g.npts, 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_lin5(const Lin5Args &a, cudaStream_t s) {
    k_lin5<<<pw_grid(a.n, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_ke_seed(const KeSeedArgs &a, cudaStream_t s) {
    k_ke_seed<<<kKeSeedBlocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_apply<double>(int, int, const ApplyArgs<double> &, cudaStream_t);
template cudaError_t launch_apply<float>(int, int, const ApplyArgs<float> &, cudaStream_t);
template cudaError_t launch_tape_prep<double>(const TapePrepArgs<double> &, cudaStream_t);
template cudaError_t launch_tape_prep<float>(const TapePrepArgs<float> &, cudaStream_t);
template cudaError_t launch_vjp<double>(const VjpArgs<double> &, cudaStream_t);
template cudaError_t launch_vjp<float>(const VjpArgs<float> &, cudaStream_t);
template cudaError_t launch_chain<double>(const ChainArgs<double> &, cudaStream_t);
template cudaError_t launch_chain<float>(const ChainArgs<float> &, cudaStream_t);
template cudaError_t launch_rhs_eval<double>(const RhsEvalArgs<double> &, cudaStream_t);
template cudaError_t launch_rhs_eval<float>(const RhsEvalArgs<float> &, cudaStream_t);

}  // namespace cs3d
