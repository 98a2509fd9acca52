// cs3d_sweeps.cu -- the directional sweep kernels of one RK stage, the
// compact filter and the single-operator kernel (sm_103a).
//
// One stage is three fused directional sweeps.  Each sweep kernel takes a
// pencil tile -- L complete grid lines along the sweep direction -- and runs
// three phases:
//
//   A  load the tile's inputs (batched, several points per thread in
//      flight), form primitives and fluxes, stage every line-solve input in
//      shared memory ([position][line] layout);
//   B  solve: one thread per (line, task); a task is two line solves run
//      interleaved -- the 1st and 2nd derivative of one field, or the 1st
//      derivative of two fields -- each a Thomas sweep with precomputed
//      factors, unrolled in chunks of 4 rows with the next chunk's loads
//      issued ahead;
//   C  consume the derivatives point by point.
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
// global access is a contiguous row segment; x-lines are transposed into
// shared memory on load.
//
// T is the work precision: double for the plain form, float for the mixed
// form.  The conserved state (q1, q2, and qk where kept) is FP64.
#include <cstdio>
#include <cmath>
#include "cs3d_tile.cuh"

namespace cs3d {

// Points per thread in flight in the point loops of the mixed form (measured
// at 128^3 and 256^3; deeper batches spill or run no faster).
constexpr int kFilterBatch = 4;         // the mixed filter's load and store loops
constexpr int kFilterConsumeBatch = 2;  // the mixed filter's consume loop
constexpr int kYConsumeBatch = 4;       // the y sweep's consume phase
constexpr int kZUpdateBatch = 2;        // the z sweep's RK-update pass
// Resident blocks per SM the mixed-form kernels are compiled for: the filter
// at 4 (64 registers), the x sweep at 3 blocks of 256 threads (80 registers),
// y and z at one block of 512 (128 registers); the plain form runs 128
// threads, 2 blocks.
constexpr int kFilterMinBlocks = 4;
constexpr int kMinBlocksX = 3, kMinBlocksY = 1, kMinBlocksZ = 1;

// The sweep kernels take the shared-memory pitch of their tile as a template
// parameter PC (0: read at run time).  The launcher instantiates the mixed
// form's usual pitches (x: 9 and 5; y, z: 16 and 8), where every
// shared-memory access of a solve chunk becomes an immediate off one base
// register: x 0.358 -> 0.336 ms, y and z 2-4% faster per step at 128^3.
// ---------------------------------------------------------------------
// sweep x
// ---------------------------------------------------------------------
// Sweep task t solves into buffers 2t and 2t+1.  The FP32-mixed form's pair
// layout gives the last task of the x and y sweeps (one field) a spare second
// lane (XDUM, YDUM), which no thread solves; the FP64 form solves that field
// twice over in its own buffer.
enum { XU = 0, XU2, XV, XV2, XW, XW2, XT, XT2, XRU, XF1, XF2, XF3, XF4, XDUM, XNB2 };
constexpr int XNB = XDUM;
__constant__ Task kTasksX[7] = {{XU, XU, 0, XU, XU2, 1}, {XV, XV, 0, XV, XV2, 1}, {XW, XW, 0, XW, XW2, 1},
                                {XT, XT, 0, XT, XT2, 1}, {XRU, XRU, 0, XF1, XF1, 0},
                                {XF2, XF2, 0, XF3, XF3, 0}, {XF4, XF4, 0, XF4, XF4, 0}};
__constant__ Task kTasksX2[7] = {{XU, XU, 0, XU, XU2, 1}, {XV, XV, 0, XV, XV2, 1}, {XW, XW, 0, XW, XW2, 1},
                                 {XT, XT, 0, XT, XT2, 1}, {XRU, XRU, 0, XF1, XF1, 0},
                                 {XF2, XF2, 0, XF3, XF3, 0}, {XF4, XF4, 0, XF4, XDUM, 0}};

template <typename T, int PC>
__global__ void __launch_bounds__(sweep_threads<T>(0), sizeof(T) == 4 ? kMinBlocksX : 2) k_sweep_x(SweepArgs<T> a) {
    const int L = a.L, P = PC > 0 ? PC : a.P;
    const Tile t = make_tile<0>(a.g, L);
    const int N = t.N, NL = N * L;
    const auto sm = SweepSmem<T>::at(smem_raw, sizeof(T) == 4 ? XNB2 : XNB, L, P, N);
    const GasParams gp = a.gas;
    // FP64 tiles: points across the lines first, pitch P = L (no pad column)
    constexpr bool kXLineFirst = sizeof(T) == 8;
    // phase A: primitives and the inputs of the x-solves
    struct InA { Pt pt; T q[5]; };
    batched<InA, sizeof(T) == 4 ? 4 : 2>(NL,
        [&](InA &in, int p) {
            in.pt = point<0, kXLineFirst>(t, p, L, P, a.lgL, a.divN);
#pragma unroll
            for (int f = 0; f < 5; ++f) in.q[f] = a.qs[f][in.pt.gi];
        },
        [&](InA &in) {
            if (!in.pt.ok) return;
            const unsigned gi = in.pt.gi;
            PrimW<T> s = prim_w<T>(gp, in.q[0], in.q[1], in.q[2], in.q[3], in.q[4]);
            a.prim[0][gi] = s.U; a.prim[1][gi] = s.V; a.prim[2][gi] = s.W;
            a.prim[3][gi] = s.p; a.prim[4][gi] = s.Tt;
            // stage-start primitives: on stage 1, points of SPONGE faces (not
            // on a wall) use the state before the previous step's sponge
            // overwrite, which the reference's U,V,W,p,T arrays still hold.
            PrimW<T> ss = s;
            if (a.use_backup) {
                int i, j, k;
                coords<0>(t, in.pt.l, in.pt.n, i, j, k);
                const int f = faces_of(a.g, i, j, k);
                if ((f & a.sponge_kind_faces) && !(f & a.wall_faces))
                    ss = prim_w<T>(gp, to_work<T>(a.backup.f[0][gi]), to_work<T>(a.backup.f[1][gi]),
                                   to_work<T>(a.backup.f[2][gi]), to_work<T>(a.backup.f[3][gi]),
                                   to_work<T>(a.backup.f[4][gi]));
            }
            const int o = in.pt.o;
            put1(sm, 0, o, ss.U);
            put1(sm, 1, o, ss.V);
            put1(sm, 2, o, ss.W);
            put1(sm, 3, o, ss.Tt);
            put2(sm, 4, o, s.ru, s.ru * ss.U + ss.p);
            put2(sm, 5, o, s.rv * ss.U, s.rw * ss.U);
            put1(sm, 6, o, s.re * ss.U + ss.U * ss.p);
        });
    __syncthreads();
    run_sweep_solves<2, PC>(sm, sizeof(T) == 4 ? kTasksX2 : kTasksX, 7, L, t.nlines, a.d1, a.d2, threadIdx.x,
                            blockDim.x, XDUM);
    __syncthreads();
    // phase C
    const T c43 = T(4.0 / 3.0), cpPr = (T)gp.cpPr, muref = (T)gp.mu_ref;
    struct InC { Pt pt; T v[4]; };
    batched<InC, sizeof(T) == 4 ? 4 : 2>(NL,
        [&](InC &in, int p) {
            in.pt = point<0, kXLineFirst>(t, p, L, P, a.lgL, a.divN);
            const unsigned gi = in.pt.gi;
            in.v[0] = a.prim[0][gi]; in.v[1] = a.prim[1][gi]; in.v[2] = a.prim[2][gi]; in.v[3] = a.prim[4][gi];
        },
        [&](InC &in) {
            if (!in.pt.ok) return;
            const Pt &p = in.pt;
            const unsigned gi = p.gi;
            const Zn<T> zz = zn(a.d1, a.d2, p.n);
            const T U = in.v[0], V = in.v[1], W = in.v[2], Tt = in.v[3];
            const T mu = muref * visc_pow(Tt);
            const T amu = (T)0.76 * mu / Tt;
            a.mu[gi] = mu;
            a.amu[gi] = amu;
            T Ux, Uxx, Vx, Vxx, Wx, Wxx, Tx, Txx, cex, f1, f2, f3;
            get2(sm, 0, p, L, zz.z1, zz.z2, Ux, Uxx);
            get2(sm, 1, p, L, zz.z1, zz.z2, Vx, Vxx);
            get2(sm, 2, p, L, zz.z1, zz.z2, Wx, Wxx);
            get2(sm, 3, p, L, zz.z1, zz.z2, Tx, Txx);
            get2(sm, 4, p, L, zz.z1, zz.z1, cex, f1);
            get2(sm, 5, p, L, zz.z1, zz.z1, f2, f3);
            const T f4 = get1(sm, XF4, p, L, zz.z1);
            a.dx[0][gi] = Ux; a.dx[1][gi] = Vx; a.dx[2][gi] = Wx; a.dx[3][gi] = Tx;
            if (a.tape[0]) {  // the tape's x entries (kIn* 0..16)
                T *const *g = a.tape;
                g[0][gi] = U; g[1][gi] = V; g[2][gi] = W; g[3][gi] = Tt;
                g[4][gi] = Ux; g[5][gi] = Vx; g[6][gi] = Wx; g[7][gi] = Tx;
                g[8][gi] = Uxx; g[9][gi] = Vxx; g[10][gi] = Wxx; g[11][gi] = Txx;
                g[12][gi] = cex; g[13][gi] = f1; g[14][gi] = f2; g[15][gi] = f3; g[16][gi] = f4;
            }
            a.R[0][gi] = -cex;
            a.R[1][gi] = mu * (c43 * Uxx) - f1;
            a.R[2][gi] = mu * Vxx - f2;
            a.R[3][gi] = mu * Wxx - f3;
            a.R[4][gi] = cpPr * mu * Txx + mu * (U * (c43 * Uxx) + V * Vxx + W * Wxx) - f4;
        });
}

// ---------------------------------------------------------------------
// sweep y
// ---------------------------------------------------------------------
enum { YU = 0, YU2, YV, YV2, YW, YW2, YT, YT2, YUX, YVX, YRV, YF1, YF2, YF3, YF4, YDUM, YNB2 };
constexpr int YNB = YDUM;
__constant__ Task kTasksY[8] = {{YU, YU, 0, YU, YU2, 1}, {YV, YV, 0, YV, YV2, 1}, {YW, YW, 0, YW, YW2, 1},
                                {YT, YT, 0, YT, YT2, 1}, {YUX, YUX, 0, YVX, YVX, 0},
                                {YRV, YRV, 0, YF1, YF1, 0}, {YF2, YF2, 0, YF3, YF3, 0},
                                {YF4, YF4, 0, YF4, YF4, 0}};
__constant__ Task kTasksY2[8] = {{YU, YU, 0, YU, YU2, 1}, {YV, YV, 0, YV, YV2, 1}, {YW, YW, 0, YW, YW2, 1},
                                 {YT, YT, 0, YT, YT2, 1}, {YUX, YUX, 0, YVX, YVX, 0},
                                 {YRV, YRV, 0, YF1, YF1, 0}, {YF2, YF2, 0, YF3, YF3, 0},
                                 {YF4, YF4, 0, YF4, YDUM, 0}};

// FP64: 3 blocks per SM (168 registers, no spills): 2.93 -> 2.67 ms per step at
// TGV 128^3, 37.5 -> 27.1 at HIT 256^3, the same bits
template <typename T, int PC>
__global__ void __launch_bounds__(sweep_threads<T>(1), sizeof(T) == 4 ? kMinBlocksY : 3) k_sweep_y(SweepArgs<T> a) {
    const int L = a.L, P = PC > 0 ? PC : a.P;
    const Tile t = make_tile<1>(a.g, L);
    const int N = t.N, NL = N * L;
    const auto sm = SweepSmem<T>::at(smem_raw, sizeof(T) == 4 ? YNB2 : YNB, L, P, N);
    struct InA { Pt pt; T v[11]; };
    batched<InA, sizeof(T) == 4 ? 4 : 2>(NL,
        [&](InA &in, int p) {
            in.pt = point<1>(t, p, L, P, a.lgL, a.divN);
            const unsigned gi = in.pt.gi;
#pragma unroll
            for (int f = 0; f < 4; ++f) in.v[f] = a.qs[f + 1][gi];
#pragma unroll
            for (int f = 0; f < 5; ++f) in.v[4 + f] = a.prim[f][gi];
            in.v[9] = a.dx[0][gi];
            in.v[10] = a.dx[1][gi];
        },
        [&](InA &in) {
            if (!in.pt.ok) return;
            const int o = in.pt.o;
            const T ru = in.v[0], rv = in.v[1], rw = in.v[2], re = in.v[3];
            const T V = in.v[5], pp = in.v[7];
            put1(sm, 0, o, in.v[4]);
            put1(sm, 1, o, V);
            put1(sm, 2, o, in.v[6]);
            put1(sm, 3, o, in.v[8]);
            put2(sm, 4, o, in.v[9], in.v[10]);
            put2(sm, 5, o, rv, ru * V);
            put2(sm, 6, o, rv * V + pp, rw * V);
            put1(sm, 7, o, re * V + V * pp);
        });
    __syncthreads();
    run_sweep_solves<2, PC>(sm, sizeof(T) == 4 ? kTasksY2 : kTasksY, 8, L, t.nlines, a.d1, a.d2, threadIdx.x,
                            blockDim.x, YDUM);
    __syncthreads();
    const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0), cpPr = (T)a.gas.cpPr;
    struct InC { Pt pt; T v[9]; };
    batched<InC, sizeof(T) == 4 ? kYConsumeBatch : 2>(NL,
        [&](InC &in, int p) {
            in.pt = point<1>(t, p, L, P, a.lgL, a.divN);
            const unsigned gi = in.pt.gi;
            in.v[0] = a.prim[0][gi]; in.v[1] = a.prim[1][gi]; in.v[2] = a.prim[2][gi];
            in.v[3] = a.mu[gi];
#pragma unroll
            for (int f = 0; f < 5; ++f) in.v[4 + f] = a.R[f][gi];
        },
        [&](InC &in) {
            if (!in.pt.ok) return;
            const Pt &p = in.pt;
            const unsigned gi = p.gi;
            const Zn<T> zz = zn(a.d1, a.d2, p.n);
            const T U = in.v[0], V = in.v[1], W = in.v[2], mu = in.v[3];
            T Uy, Uyy, Vy, Vyy, Wy, Wyy, Ty, Tyy, Uxy, Vxy, cey, f1, f2, f3;
            get2(sm, 0, p, L, zz.z1, zz.z2, Uy, Uyy);
            get2(sm, 1, p, L, zz.z1, zz.z2, Vy, Vyy);
            get2(sm, 2, p, L, zz.z1, zz.z2, Wy, Wyy);
            get2(sm, 3, p, L, zz.z1, zz.z2, Ty, Tyy);
            get2(sm, 4, p, L, zz.z1, zz.z1, Uxy, Vxy);
            get2(sm, 5, p, L, zz.z1, zz.z1, cey, f1);
            get2(sm, 6, p, L, zz.z1, zz.z1, f2, f3);
            const T f4 = get1(sm, YF4, p, L, zz.z1);
            a.dy[0][gi] = Uy; a.dy[1][gi] = Vy; a.dy[2][gi] = Wy; a.dy[3][gi] = Ty;
            if (a.tape[0]) {  // the tape's y entries (kIn* 17..31)
                T *const *g = a.tape;
                g[17][gi] = Uy; g[18][gi] = Vy; g[19][gi] = Wy; g[20][gi] = Ty;
                g[21][gi] = Uyy; g[22][gi] = Vyy; g[23][gi] = Wyy; g[24][gi] = Tyy;
                g[25][gi] = Uxy; g[26][gi] = Vxy; g[27][gi] = cey;
                g[28][gi] = f1; g[29][gi] = f2; g[30][gi] = f3; g[31][gi] = f4;
            }
            int i, j, k;
            coords<1>(t, p.l, p.n, i, j, k);
            const int wd = a.wall_faces ? wall_dir(faces_of(a.g, i, j, k) & a.wall_faces) : -1;
            if (wd == 1) a.R[0][gi] = -cey;
            else if (wd < 0) a.R[0][gi] = in.v[4] - cey;
            a.R[1][gi] = in.v[5] + (mu * (Uyy + c13 * Vxy) - f1);
            a.R[2][gi] = in.v[6] + (mu * (c43 * Vyy + c13 * Uxy) - f2);
            a.R[3][gi] = in.v[7] + (mu * Wyy - f3);
            a.R[4][gi] = in.v[8] +
                         (cpPr * mu * Tyy + mu * (U * Uyy + V * (c43 * Vyy) + W * Wyy + c13 * (U * Vxy + V * Uxy)) - f4);
        });
}

// ---------------------------------------------------------------------
// sweep z + right-hand side + RK update
// ---------------------------------------------------------------------
enum { ZU = 0, ZU2, ZV, ZV2, ZW, ZW2, ZT, ZT2, ZS, ZWX, ZWY, ZRW, ZF1, ZF2, ZF3, ZF4, ZNB };
__constant__ Task kTasksZ[8] = {{ZU, ZU, 0, ZU, ZU2, 1}, {ZV, ZV, 0, ZV, ZV2, 1}, {ZW, ZW, 0, ZW, ZW2, 1},
                                {ZT, ZT, 0, ZT, ZT2, 1}, {ZS, ZS, 0, ZWX, ZWX, 0},
                                {ZWY, ZWY, 0, ZRW, ZRW, 0}, {ZF1, ZF1, 0, ZF2, ZF2, 0},
                                {ZF3, ZF3, 0, ZF4, ZF4, 0}};

// The z sweep's three phases as functions of (tile, shared-memory layout,
// thread range).
template <typename T, int PC>
struct ZSweep {
    // A: stage the inputs of the 16 z-solves of tile t in sm
    using SM = typename SweepSmem<T>::type;
    static __device__ __forceinline__ void load(const SweepArgs<T> &a, const Tile &t, const SM &sm, int tid,
                                                int nthr) {
        const int L = a.L, P = PC > 0 ? PC : a.P;
        const int NL = t.N * L;
        struct InA { Pt pt; T v[13]; };
        batched<InA, sizeof(T) == 4 ? 4 : 2>(NL, tid, nthr,
            [&](InA &in, int p) {
                in.pt = point<2>(t, p, L, P, a.lgL, a.divN);
                const unsigned gi = in.pt.gi;
#pragma unroll
                for (int f = 0; f < 4; ++f) in.v[f] = a.qs[f + 1][gi];
#pragma unroll
                for (int f = 0; f < 5; ++f) in.v[4 + f] = a.prim[f][gi];
                in.v[9] = a.dx[0][gi];
                in.v[10] = a.dy[1][gi];
                in.v[11] = a.dx[2][gi];
                in.v[12] = a.dy[2][gi];
            },
            [&](InA &in) {
                if (!in.pt.ok) return;
                const int o = in.pt.o;
                const T ru = in.v[0], rv = in.v[1], rw = in.v[2], re = in.v[3];
                const T W = in.v[6], pp = in.v[7];
                put1(sm, 0, o, in.v[4]);
                put1(sm, 1, o, in.v[5]);
                put1(sm, 2, o, W);
                put1(sm, 3, o, in.v[8]);
                put2(sm, 4, o, in.v[9] + in.v[10], in.v[11]);
                put2(sm, 5, o, in.v[12], rw);
                put2(sm, 6, o, ru * W, rv * W);
                put2(sm, 7, o, rw * W + pp, re * W + W * pp);
            });
    }
    // B: the 16 solves (8 pairs) of every line of the tile
    static __device__ __forceinline__ void solve(const SweepArgs<T> &a, const Tile &t, const SM &sm, int tid,
                                                 int nthr) {
        run_sweep_solves<2, PC>(sm, kTasksZ, 8, a.L, t.nlines, a.d1, a.d2, tid, nthr, -1);
    }
    // C: right-hand side, dq and the RK update of every point of the tile
    static __device__ __forceinline__ void consume(const SweepArgs<T> &a, const Tile &t, const SM &sm, int tid,
                                                   int nthr) {
        const int L = a.L, P = PC > 0 ? PC : a.P;
        const int NL = t.N * L;
        const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0), c23 = T(2.0 / 3.0), cpPr = (T)a.gas.cpPr;
        const double dt = *a.dt;
        const T dtw = (T)dt;
        const int st = a.rk_step;
        const bool tvd = a.rk == 1;
        // which state arrays the update reads (uniform over the launch):
        //   qa = q1 (RK4 stage 1, all TVD-RK3 stages) or q2 (RK4 stages 2-4)
        //   qb = q1 for the FP64 RK4 qk update on stages 2-3, or the FP64 qk of
        //        TVD-RK3 stages 2-3
        //   mixed RK4: q2 accumulates every stage's increment in FP64; the next
        //   stage input qk = q1 + b dq exists only as an FP32 shadow, formed from
        //   q1's shadow (the stage input itself on stage 1)
        const bool use_q1a = tvd || st == 1;
        const bool need_qb = (!tvd && !a.mixed_rk4 && st > 1 && st < 4) || (tvd && st > 1);
        const bool need_q1s = a.mixed_rk4 && st > 1 && st < 4;
        const bool need_qs = a.mixed_rk4 && st == 1;
        // Phase C runs in two passes over the same points, each point by the same
        // thread in both (so no barrier between them): C1 forms the right-hand
        // side and parks dq = dt*RHS in the point's own, now unused, solve slots;
        // C2 streams the FP64 state through the RK update.  Each pass keeps fewer
        // values live than one fused pass, so more points' loads are in flight.
        constexpr int kDq[5] = {ZS, ZWX, ZWY, ZRW, ZF1};
        struct InC1 {
            Pt pt;
            T v[18];
            T qsv[5];
        };
        pipelined<InC1>(NL, tid, nthr,
            [&](InC1 &in, int p) {
                in.pt = point<2>(t, p, L, P, a.lgL, a.divN);
                const unsigned gi = in.pt.gi;
                in.v[0] = a.prim[0][gi]; in.v[1] = a.prim[1][gi]; in.v[2] = a.prim[2][gi];
                in.v[3] = a.mu[gi]; in.v[4] = a.amu[gi];
#pragma unroll
                for (int f = 0; f < 4; ++f) { in.v[5 + f] = a.dx[f][gi]; in.v[9 + f] = a.dy[f][gi]; }
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    in.v[13 + f] = a.R[f][gi];
                    in.qsv[f] = a.sponge ? a.qs[f][gi] : T(0);
                }
            },
            [&](InC1 &in) {
                if (!in.pt.ok) return;
                const Pt &p = in.pt;
                const unsigned gi = p.gi;
                const Zn<T> zz = zn(a.d1, a.d2, p.n);
                const T U = in.v[0], V = in.v[1], W = in.v[2], mu = in.v[3], amu = in.v[4];
                const T Ux = in.v[5], Vx = in.v[6], Wx = in.v[7], Tx = in.v[8];
                const T Uy = in.v[9], Vy = in.v[10], Wy = in.v[11], Ty = in.v[12];
                T Uz, Uzz, Vz, Vzz, Wz, Wzz, Tz, Tzz, S, Wxz, Wyz, cez, f1, f2, f3, f4;
                get2(sm, 0, p, L, zz.z1, zz.z2, Uz, Uzz);
                get2(sm, 1, p, L, zz.z1, zz.z2, Vz, Vzz);
                get2(sm, 2, p, L, zz.z1, zz.z2, Wz, Wzz);
                get2(sm, 3, p, L, zz.z1, zz.z2, Tz, Tzz);
                get2(sm, 4, p, L, zz.z1, zz.z1, S, Wxz);  // S = d/dz (Ux + Vy)
                get2(sm, 5, p, L, zz.z1, zz.z1, Wyz, cez);
                get2(sm, 6, p, L, zz.z1, zz.z1, f1, f2);
                get2(sm, 7, p, L, zz.z1, zz.z1, f3, f4);
                T src[5] = {T(0), T(0), T(0), T(0), T(0)};
                if (a.sponge) {  // sigma (avg - q), SpongeBC / CSolver_AWS.hpp:228
                    const T sg = to_work<T>(a.sigma[gi]);
#pragma unroll
                    for (int f = 0; f < 5; ++f) src[f] = sg * (to_work<T>(a.savg.f[f][gi]) - in.qsv[f]);
                }
                const T MuX = amu * Tx, MuY = amu * Ty, MuZ = amu * Tz;
                T R[5];
                R[0] = in.v[13];
                R[1] = in.v[14] + mu * (Uzz + c13 * Wxz) - f1 + c43 * MuX * (Ux - T(0.5) * Vy - T(0.5) * Wz) +
                       MuY * (Uy + Vx) + MuZ * (Wx + Uz) + src[1];
                R[2] = in.v[15] + mu * (Vzz + c13 * Wyz) - f2 + c43 * MuY * (Vy - T(0.5) * Ux - T(0.5) * Wz) +
                       MuX * (Uy + Vx) + MuZ * (Wy + Vz) + src[2];
                R[3] = in.v[16] + mu * (c43 * Wzz + c13 * S) - f3 + c43 * MuZ * (Wz - T(0.5) * Ux - T(0.5) * Vy) +
                       MuX * (Wx + Uz) + MuY * (Wy + Vz) + src[3];
                const T q2s = Ux * Ux + Vy * Vy + Wz * Wz;
                const T sq = Uy * Uy + Uz * Uz + Vx * Vx + Vz * Vz + Wx * Wx + Wy * Wy;
                const T cr = Ux * Vy + Ux * Wz + Vy * Wz;
                const T sh = Uy * Vx + Uz * Wx + Vz * Wy;
                const T v1 = mu * (U * Uzz + V * Vzz + W * (c43 * Wzz) + c13 * (U * Wxz + V * Wyz + W * S) + c43 * q2s +
                                   sq - c43 * cr + T(2.0) * sh);
                const T v2 = c43 * (U * MuX * Ux + V * MuY * Vy + W * MuZ * Wz) - c23 * U * MuX * (Vy + Wz) -
                             c23 * V * MuY * (Ux + Wz) - c23 * W * MuZ * (Ux + Vy) + U * MuY * (Uy + Vx) +
                             U * MuZ * (Uz + Wx) + V * MuX * (Uy + Vx) + V * MuZ * (Vz + Wy) + W * MuX * (Uz + Wx) +
                             W * MuY * (Vz + Wy);
                R[4] = in.v[17] + cpPr * (MuX * Tx + MuY * Ty + MuZ * Tz + mu * Tzz) + v1 + v2 - f4 + T(2.0) * src[4];
                // continuity and the post-step boundary fix-up (CSolver_AWS.cpp:1506-1679)
                int i, j, k;
                coords<2>(t, p.l, p.n, i, j, k);
                const int fc = faces_of(a.g, i, j, k);
                const int wd = a.wall_faces ? wall_dir(fc & a.wall_faces) : -1;
                if (wd == 2) R[0] = -cez;
                else if (wd < 0) R[0] = R[0] - cez + src[0];
                const bool zero_all = (fc & a.sponge_kind_faces) != 0;
                const bool zero_mom = wd >= 0;
                if (a.diag[0]) {  // derivative fields of the last stage, for diagnostics
                    a.diag[0][gi] = Uz; a.diag[1][gi] = Vz; a.diag[2][gi] = Wz;
                }
                if (a.tape[0]) {  // the tape's z entries (kIn* 32..47)
                    T *const *g = a.tape;
                    g[32][gi] = Uz; g[33][gi] = Vz; g[34][gi] = Wz; g[35][gi] = Tz;
                    g[36][gi] = Uzz; g[37][gi] = Vzz; g[38][gi] = Wzz; g[39][gi] = Tzz;
                    g[40][gi] = S; g[41][gi] = Wxz; g[42][gi] = Wyz; g[43][gi] = cez;
                    g[44][gi] = f1; g[45][gi] = f2; g[46][gi] = f3; g[47][gi] = f4;
                }
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    // plain form: dq = dt * RHS in FP64; mixed form: in FP32
                    T d = sizeof(T) == 8 ? (T)(dt * (double)R[f]) : dtw * R[f];
                    if (zero_all || (f > 0 && zero_mom)) d = T(0);
                    if (a.dq_out[0]) a.dq_out[f][gi] = to_f64(d);
                    sm.at(kDq[f], p.o) = d;
                }
            });
        struct InC2 {
            Pt pt;
            double qa[5], qb[5];
            T qsv[5];    // q1's shadow: the stage input qs on stage 1, q1s on 2-3
        };
        batched<InC2, kZUpdateBatch>(NL, tid, nthr,
            [&](InC2 &in, int p) {
                in.pt = point<2>(t, p, L, P, a.lgL, a.divN);
                const unsigned gi = in.pt.gi;
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    in.qa[f] = use_q1a ? a.q1.f[f][gi] : a.q2.f[f][gi];
                    in.qb[f] = need_qb ? (tvd ? a.qk.f[f][gi] : a.q1.f[f][gi]) : 0.0;
                    in.qsv[f] = need_qs ? a.qs[f][gi] : need_q1s ? (T)a.q1s[f][gi] : T(0);
                }
            },
            [&](InC2 &in) {
                if (!in.pt.ok) return;
                const unsigned gi = in.pt.gi;
                if (sizeof(T) == 8) {
                    // plain form: the reference's RK update in FP64
#pragma unroll
                    for (int f = 0; f < 5; ++f) {
                        const double d = (double)sm.at(kDq[f], in.pt.o);
                        if (tvd) {  // TVD-RK3 (TVDRK3.hpp:38-96); qa = q1, qb = qk
                            if (st == 1) a.qk.f[f][gi] = in.qa[f] + d;
                            else if (st == 2) a.qk.f[f][gi] = 0.75 * in.qa[f] + 0.25 * in.qb[f] + 0.25 * d;
                            else a.q2.f[f][gi] = (1.0 / 3.0) * in.qa[f] + (2.0 / 3.0) * in.qb[f] + (2.0 / 3.0) * d;
                        } else {    // RK4 (RK4.hpp:35-118); qa = q1 (stage 1) or q2
                            const double ca = (st == 1 || st == 4) ? (1.0 / 6.0) : (1.0 / 3.0);
                            const double cb = (st == 3) ? 1.0 : 0.5;
                            a.q2.f[f][gi] = in.qa[f] + ca * d;
                            if (st == 1) a.qk.f[f][gi] = in.qa[f] + cb * d;
                            else if (st < 4) a.qk.f[f][gi] = in.qb[f] + cb * d;
                        }
                    }
                } else {
                    // mixed form: the FP32 increment accumulated into the FP64 state
#pragma unroll
                    for (int f = 0; f < 5; ++f) {
                        const T d = sm.at(kDq[f], in.pt.o);
                        if (tvd) {
                            const double dd = to_f64(d);
                            double nv;
                            if (st == 1) { nv = in.qa[f] + dd; a.qk.f[f][gi] = nv; }
                            else if (st == 2) { nv = 0.75 * in.qa[f] + 0.25 * in.qb[f] + 0.25 * dd; a.qk.f[f][gi] = nv; }
                            else { nv = (1.0 / 3.0) * in.qa[f] + (2.0 / 3.0) * in.qb[f] + (2.0 / 3.0) * dd; a.q2.f[f][gi] = nv; }
                            if (a.shadow_target != SHADOW_NONE) a.shadow_out[f][gi] = narrow(nv);
                        } else {
                            // RK4: q2 += a_s dq in FP64 on every stage (RK4.hpp:35-118)
                            const T ca = (st == 1 || st == 4) ? T(1.0 / 6.0) : T(1.0 / 3.0);
                            const T cb = (st == 3) ? T(1.0) : T(0.5);
                            const double q2n = in.qa[f] + to_f64(ca * d);
                            a.q2.f[f][gi] = q2n;
                            if (st < 4) {
                                // the next stage input qk = q1 + cb*dq, kept as an FP32 shadow
                                a.shadow_out[f][gi] = fma(cb, d, in.qsv[f]);
                            } else {
                                if (a.shadow_target == SHADOW_Q2) a.shadow_out[f][gi] = narrow(q2n);
                                // the filter's first pass input, q2 - fref in FP32
                                if (a.fluct_out) a.fluct[f][gi] = narrow(q2n - a.fref[f]);
                            }
                        }
                    }
                }
            });
    }
};

// FP64: 3 blocks per SM (168 registers; 88 bytes of spill stores): 4.70 ->
// 4.52 ms per step at TGV 128^3, 52.5 -> 44.9 at HIT 256^3, the same bits
template <typename T, int PC>
__global__ void __launch_bounds__(sweep_threads<T>(2), sizeof(T) == 4 ? kMinBlocksZ : 3) k_sweep_z(SweepArgs<T> a) {
    const Tile t = make_tile<2>(a.g, a.L);
    const auto sm = SweepSmem<T>::at(smem_raw, ZNB, a.L, PC > 0 ? PC : a.P, t.N);
    ZSweep<T, PC>::load(a, t, sm, threadIdx.x, blockDim.x);
    __syncthreads();
    ZSweep<T, PC>::solve(a, t, sm, threadIdx.x, blockDim.x);
    __syncthreads();
    ZSweep<T, PC>::consume(a, t, sm, threadIdx.x, blockDim.x);
}

// ---------------------------------------------------------------------
// compact filter, one direction, five fields (Filter.cpp:98-171)
// ---------------------------------------------------------------------
// PC: the tile pitch as a compile-time constant (0: at run time); the mixed
// form's 128^3 pitches (x 9, y and z 8) are instantiated.
// Plain form: FP64 in, FP64 out, a.op = F.  Mixed form: a.op is the
// correction F - I, solved out of place (buffers 5..9), and the pass writes
// v + (F - I) v; the first pass reads FP64 q2 minus a per-field reference
// value (the field's initial mean, so the FP32 numbers are fluctuations), the
// middle pass works in FP32, and the last pass writes
// q1 = q2 + (filtered - unfiltered) in FP64 plus q1's FP32 shadow.
__constant__ Task kTasksF[3] = {{0, 0, 2, 1, 1, 2}, {2, 2, 2, 3, 3, 2}, {4, 4, 2, 4, 4, 2}};

template <typename T, int DIR, int PC>
__global__ void __launch_bounds__(filter_threads<T>(), sizeof(T) == 4 ? kFilterMinBlocks : 4) k_filter(FilterArgs<T> a) {
    constexpr int B = sizeof(T) == 4 ? kFilterBatch : 2;
    constexpr bool kCorr = sizeof(T) == 4;
    const int L = a.L, P = PC > 0 ? PC : a.P;
    const Tile t = make_tile<DIR>(a.g, L);
    const int N = t.N, NL = N * L;
    Smem<T> sm = smem_layout<T>(kCorr ? 10 : 5, L, P, N);
    for (int p0 = threadIdx.x; p0 < NL; p0 += B * blockDim.x) {
        Pt pt[B];
        T v[B][5];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            pt[b] = point<DIR>(t, p0 + b * blockDim.x, L, P, a.lgL, a.divN);
            const unsigned gi = pt[b].gi;
#pragma unroll
            for (int f = 0; f < 5; ++f)
                v[b][f] = a.src64.f[f] ? to_work<T>(a.src64.f[f][gi] - a.ref[f]) : a.src32[f][gi];
        }
#pragma unroll
        for (int b = 0; b < B; ++b) {
            if (!pt[b].ok) continue;
#pragma unroll
            for (int f = 0; f < 5; ++f) sm.b(f)[pt[b].o] = v[b][f];
        }
    }
    __syncthreads();
    if constexpr (kCorr) {
        // the five right-hand sides by the whole block, then one thread per
        // (field, line) for the recurrences alone
        rhs_pass<T, 4, 5>(sm, 0, 5, L, a.lgL, t.nlines, a.op);
        __syncthreads();
        for (int w = threadIdx.x; w < 5 * L; w += blockDim.x) {
            const int l = w & (L - 1), f = w >> a.lgL;
            if (l >= t.nlines) continue;
            thomas_inplace<T, PC>(sm.b(5 + f) + l, a.op, &sm.fact[(5 + f) * L + l], P);
        }
    } else {
        // plain form: one solve per thread, each field in place
        run_sweep_solves<4, 0>(sm, kTasksF, 3, L, t.nlines, a.op, a.op, (int)threadIdx.x, (int)blockDim.x);
    }
    __syncthreads();
    constexpr int BC = sizeof(T) == 4 ? kFilterConsumeBatch : 2;
    for (int p0 = threadIdx.x; p0 < NL; p0 += BC * blockDim.x) {
        Pt pt[BC];
        double q[BC][5];
        T u[BC][5];
#pragma unroll
        for (int b = 0; b < BC; ++b) {
            pt[b] = point<DIR>(t, p0 + b * blockDim.x, L, P, a.lgL, a.divN);
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                q[b][f] = a.delta_from.f[f] ? a.delta_from.f[f][pt[b].gi] : 0.0;
                u[b][f] = kCorr && a.unf[f] ? (T)a.unf[f][pt[b].gi] : T(0);
            }
        }
#pragma unroll
        for (int b = 0; b < BC; ++b) {
            if (!pt[b].ok) continue;
            const unsigned gi = pt[b].gi;
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                const T v = kCorr ? sm.b(f)[pt[b].o] + get(sm, 5 + f, pt[b], L, a.op) : get(sm, f, pt[b], L, a.op);
                if (a.dst64.f[f]) {
                    double nv;
                    if (a.delta_from.f[f]) {
                        // the unfiltered value: the first pass's FP32 input, or
                        // formed again from q2 (the same number either way)
                        const T v0 = kCorr && a.unf[f] ? u[b][f] : to_work<T>(q[b][f] - a.ref[f]);
                        nv = q[b][f] + to_f64(v - v0);
                    } else {
                        nv = to_f64(v) + a.ref[f];
                    }
                    a.dst64.f[f][gi] = nv;
                    if (a.shadow_out[0]) a.shadow_out[f][gi] = narrow(nv);
                } else {
                    a.dst32[f][gi] = v;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------
// single operator on contiguous lines (Derivatives::calc1stDerivField etc.)
// ---------------------------------------------------------------------
__constant__ Task kTaskLone[1] = {{0, 0, 0, 0, 0, 0}};

template <int H>
__global__ void __launch_bounds__(128) k_line_op(LineOpArgs a) {
    const int L = a.L, N = a.op.N, P = a.P;
    const long long l0 = (long long)blockIdx.x * L;
    const int nl = (int)min((long long)L, a.nlines - l0);
    Smem<double> sm = smem_layout<double>(1, L, P, N);
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        const int l = p / N, n = p - l * N;
        if (l >= nl) continue;
        sm.b(0)[n * P + l] = a.in[(l0 + l) * N + n];
    }
    __syncthreads();
    // one solve per line (the task's duplicate second solve left out)
    run_sweep_solves<H, 0>(sm, kTaskLone, 1, L, nl, a.op, a.op, (int)threadIdx.x, (int)blockDim.x);
    __syncthreads();
    for (int p = threadIdx.x; p < N * L; p += blockDim.x) {
        Pt q;
        q.l = p / N;
        q.n = p - q.l * N;
        if (q.l >= nl) continue;
        q.o = q.n * P + q.l;
        a.out[(l0 + q.l) * N + q.n] = get(sm, 0, q, L, a.op);
    }
}

// ---------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------
template <typename T>
static size_t tile_smem(int nbuf, int L, int P, int N) {
    const int nf = (nbuf * L + 3) & ~3;
    return sizeof(T) * ((size_t)nf + (size_t)nbuf * buf_stride(N + kPad, P, L, (int)(sizeof(T) / 4)));
}

// The FP32-mixed sweeps' pair-interleaved tiles: the per-line factors, then
// (nbuf + 1) / 2 pair arrays of N rows each, then kPad rows of padding.  A
// solve's read-ahead past its line's end (up to kU + 1 rows, values never
// used) lands in the next pair array, or in the padding after the last one;
// no per-array padding, so that the mixed tiles fit the next-smaller shared
// memory carveout and leave L1 -- where the phases' global loads in flight
// are held -- more room (128^3: y and z 138.8 -> 133.4 kB a block, x
// 3 x 68.1 -> 3 x 65.8 kB).
static size_t pair_tile_smem(int nbuf, int L, int P, int N) {
    const int nf = (nbuf * L + 3) & ~3;
    return 4 * ((size_t)nf + (size_t)((nbuf + 1) / 2) * pair_stride(N, P) + (size_t)2 * kPad * P);
}

size_t planar_smem_bytes(int prec_bytes, int nbuf, int L, int P, int N) {
    return prec_bytes == 8 ? tile_smem<double>(nbuf, L, P, N) : tile_smem<float>(nbuf, L, P, N);
}
size_t sweep_smem_bytes(int prec_bytes, int nbuf, int L, int P, int N) {
    return prec_bytes == 8 ? tile_smem<double>(nbuf, L, P, N) : pair_tile_smem(nbuf, L, P, N);
}
int sweep_nbuf(int dir, int prec_bytes) {
    if (prec_bytes == 4) return dir == 0 ? (int)XNB2 : dir == 1 ? (int)YNB2 : (int)ZNB;
    return dir == 0 ? (int)XNB : dir == 1 ? (int)YNB : (int)ZNB;
}
int sweep_ntask(int dir) { return dir == 0 ? 7 : 8; }
int filter_ntask() { return 3; }

template <typename K, typename A>
static cudaError_t launch_tile_kernel(K kernel, const A &a, dim3 grid, size_t sm, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    kernel<<<grid, a.threads, sm, s>>>(a);
    return cudaGetLastError();
}

static dim3 tile_grid(int dir, const Geom &g, int L) {
    if (dir == 0) return dim3((g.Ny + L - 1) / L, g.Nz);
    if (dir == 1) return dim3((g.Nx + L - 1) / L, g.Nz);
    return dim3((g.Nx + L - 1) / L, g.Ny);
}

template <typename T>
cudaError_t launch_sweep(int dir, const SweepArgs<T> &a, cudaStream_t s) {
    const int N = dir == 0 ? a.g.Nx : dir == 1 ? a.g.Ny : a.g.Nz;
    const size_t sm = sweep_smem_bytes((int)sizeof(T), sweep_nbuf(dir, (int)sizeof(T)), a.L, a.P, N);
    const dim3 grid = tile_grid(dir, a.g, a.L);
    if constexpr (sizeof(T) == 4) {
        if (dir == 0 && a.P == 9) return launch_tile_kernel(k_sweep_x<T, 9>, a, grid, sm, s);
        if (dir == 0 && a.P == 5) return launch_tile_kernel(k_sweep_x<T, 5>, a, grid, sm, s);
        if (dir == 1 && a.P == 16) return launch_tile_kernel(k_sweep_y<T, 16>, a, grid, sm, s);
        if (dir == 1 && a.P == 8) return launch_tile_kernel(k_sweep_y<T, 8>, a, grid, sm, s);
        if (dir == 2 && a.P == 16) return launch_tile_kernel(k_sweep_z<T, 16>, a, grid, sm, s);
        if (dir == 2 && a.P == 8) return launch_tile_kernel(k_sweep_z<T, 8>, a, grid, sm, s);
    }
    if (dir == 0) return launch_tile_kernel(k_sweep_x<T, 0>, a, grid, sm, s);
    if (dir == 1) return launch_tile_kernel(k_sweep_y<T, 0>, a, grid, sm, s);
    return launch_tile_kernel(k_sweep_z<T, 0>, a, grid, sm, s);
}

template <typename T>
cudaError_t launch_filter(int dir, const FilterArgs<T> &a, cudaStream_t s) {
    const int N = dir == 0 ? a.g.Nx : dir == 1 ? a.g.Ny : a.g.Nz;
    const size_t sm = tile_smem<T>(sizeof(T) == 4 ? 10 : 5, a.L, a.P, N);
    const dim3 grid = tile_grid(dir, a.g, a.L);
    if constexpr (sizeof(T) == 4) {
        if (dir == 0 && a.P == 9) return launch_tile_kernel(k_filter<T, 0, 9>, a, grid, sm, s);
        if (dir == 1 && a.P == 8) return launch_tile_kernel(k_filter<T, 1, 8>, a, grid, sm, s);
        if (dir == 2 && a.P == 8) return launch_tile_kernel(k_filter<T, 2, 8>, a, grid, sm, s);
    }
    if (dir == 0) return launch_tile_kernel(k_filter<T, 0, 0>, a, grid, sm, s);
    if (dir == 1) return launch_tile_kernel(k_filter<T, 1, 0>, a, grid, sm, s);
    return launch_tile_kernel(k_filter<T, 2, 0>, a, grid, sm, s);
}

cudaError_t launch_line_op(const LineOpArgs &a, cudaStream_t s) {
    const size_t sm = tile_smem<double>(1, a.L, a.P, a.op.N);
    const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L));
    if (a.op.H == 4) return launch_tile_kernel(k_line_op<4>, a, grid, sm, s);
    return launch_tile_kernel(k_line_op<2>, a, grid, sm, s);
}

template cudaError_t launch_sweep<double>(int, const SweepArgs<double> &, cudaStream_t);
template cudaError_t launch_sweep<float>(int, const SweepArgs<float> &, cudaStream_t);
template cudaError_t launch_filter<double>(int, const FilterArgs<double> &, cudaStream_t);
template cudaError_t launch_filter<float>(int, const FilterArgs<float> &, cudaStream_t);

}  // namespace cs3d
