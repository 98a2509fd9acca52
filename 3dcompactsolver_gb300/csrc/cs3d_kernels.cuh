// cs3d_kernels.cuh -- kernel argument blocks and launch functions.
#pragma once
#include "cs3d_dev.cuh"

namespace cs3d {

constexpr int kTpbX = 256;   // threads per block of the mixed-form x sweep
constexpr int kTpbYZ = 512;  // most threads per block of the mixed-form y and z sweeps
constexpr int kFilterTpb = 256;  // threads per block of the mixed-form filter

// Most threads per block the stage sweeps in work type T, direction dir, are
// compiled for.  The mixed-form x sweep (80 registers) runs 3 blocks of 256
// per SM; the y and z sweeps (up to 128 registers) run either 2 blocks of 256
// or one block of 512 on a tile twice as wide (the host picks per direction).
// The plain FP64 form needs up to 255 registers per thread and runs 128.
template <typename T>
__host__ __device__ constexpr int sweep_threads(int dir) {
    return sizeof(T) == 4 ? (dir == 0 ? kTpbX : kTpbYZ) : 128;
}

template <typename T>
__host__ __device__ constexpr int filter_threads() { return sizeof(T) == 4 ? kFilterTpb : 128; }

// Ideal-gas constants (IdealGas.hpp:36-46).
struct GasParams {
    double gamma;   // 1.4
    double gm1;     // gamma - 1
    double R;       // p_ref / rho_ref / T_ref
    double cpPr;    // cp / Pr
    double mu_ref;
};

// What the z sweep writes as the FP32 shadow of the next stage's input.
enum ShadowTarget { SHADOW_NONE = 0, SHADOW_QK = 1, SHADOW_Q2 = 2 };

template <typename T>
struct SweepArgs {
    Geom g;
    int L;          // lines per tile (a power of two)
    int lgL;        // log2(L)
    FastDiv divN;   // division by the line length (x sweep)
    int P;          // shared-memory pitch between positions of a line
    int threads;    // threads per block
    LineOp<T> d1, d2;
    GasParams gas;
    const T *qs[5]; // stage input q* in the work precision (FP64 q* itself, or
                    // its FP32 shadow in the mixed form)
    Q5 q;           // stage input q* (FP64; the mixed RK4 form keeps qk in FP32 only)
    Q5 backup;      // q1 before the last sponge overwrite (SPONGE faces)
    int use_backup; // stage 1 after a sponge overwrite
    int wall_faces;         // bit per face: wall (adiabatic or moving)
    int sponge_kind_faces;  // bit per face: SPONGE kind
    T *prim[5];     // U V W p T of q*
    T *mu, *amu;    // mu(T), dmu/dT
    T *dx[4];       // Ux Vx Wx Tx
    T *dy[4];       // Uy Vy Wy Ty
    T *R[5];        // right-hand-side accumulators
    T *diag[3];     // Uz Vz Wz of the stage (optional)
    // z sweep only
    const double *dt;
    int rk, rk_step;
    Q5 q1, q2, qk;
    const float *q1s[5];    // FP32 shadow of q1 (mixed RK4, stages 2-3)
    float *fluct[5];        // mixed RK4: q2 - fref in FP32, the filter's first input
    int fluct_out;          // mixed RK4, last stage of a filtered step: write fluct
    double fref[5];         // the filter's per-field reference values
    float *shadow_out[5];   // FP32 shadow of the next stage input (mixed)
    int shadow_target;      // ShadowTarget
    int mixed_rk4;          // mixed form with RK4: qk kept only as FP32 shadow
    int sponge;
    const double *sigma;
    Q5 savg;
    double *dq_out[5];  // increments dq (optional)
    // optional tape of the stage (the discrete adjoint): the primitives
    // U, V, W, T and the 44 derivative values of the right-hand side, in the
    // order of cs3d_rhs_adjoint.cuh's kIn* indices; null = not written
    T *tape[48];
};

template <typename T>
struct FilterArgs {
    Geom g;
    int L, lgL, P, threads;
    FastDiv divN;
    LineOp<T> op;
    Q5 src64;          // FP64 source (or null pointers)
    T *src32[5];       // work-precision source
    Q5 dst64;          // FP64 destination (or null pointers)
    T *dst32[5];       // work-precision destination
    Q5 delta_from;     // mixed last pass: q1 = q2 + (filtered - unfiltered)
    const float *unf[5];   // mixed last pass: the unfiltered first-pass input, if kept
    float *shadow_out[5];  // mixed last pass: FP32 shadow of q1
    double ref[5];     // per-field reference value subtracted on entry
};

struct LineOpArgs {
    int L, P, threads;
    long long nlines;
    LineOp<double> op;
    const double *in;
    double *out;
};

struct BCArgs {
    Geom g;
    int face;
    double uw[3];
    GasParams gas;
    Q5 q;                 // stage input (FP64)
    const float *qs[5];   // ... or its FP32 shadow, when q holds null pointers
    float *qs_out[5];     // FP32 shadow to update (mixed)
    Q5 backup;
    int use_backup;
    int wall_faces, sponge_faces;
};

struct CflArgs {
    Geom g;
    GasParams gas;
    Q5 q;
    const float *qs[5];   // mixed: the FP32 shadow of q1 instead of q
    float idx, idy, idz;  // mixed: 1/dx, 1/dy, 1/dz (formed on the host: an FP64
                          // division per thread costs more than the whole read)
    double idx64, idy64, idz64;  // the same in FP64 for the plain form
    double *max_out;
    int *nan_flag;
};

struct DtArgs {
    const double *max_in;
    double *dt, *time;
    double CFL, dt_fixed;
    int first;
};

struct SpongeArgs {
    Geom g;
    const double *dt;
    double avgT, epsP, spongeP, gm1;
    Q5 q1, savg, backup;
    float *q1s[5];  // FP32 shadow of q1 to keep in step (mixed)
    int sponge_kind_faces;
};

struct IcArgs {
    Geom g;
    GasParams gas;
    const double *rho0, *p0;
    double *U0, *V0, *W0, *T0;
    Q5 q1;
    int face;
    double uw[3];
};

struct PrimArgs {
    Geom g;
    GasParams gas;
    Q5 q;
    double *out[7];
};

struct ShadowArgs {
    Geom g;
    Q5 q;
    float *out[5];
    const float *in[5];     // set: q = widen(in); else out = narrow(q)
    int nf;
};

template <typename T>
struct TgvArgs {
    Geom g;
    GasParams gas;
    Q5 q;
    const T *dx[3], *dy[3], *dz[3];
    double *out;  // [blocks][6]
};

template <typename T>
cudaError_t launch_sweep(int dir, const SweepArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_filter(int dir, const FilterArgs<T> &a, cudaStream_t s);
cudaError_t launch_line_op(const LineOpArgs &a, cudaStream_t s);
template <typename T>
cudaError_t launch_tgv(const TgvArgs<T> &a, int blocks, cudaStream_t s);
// calcTurbulenceQuantities / shearLayerInfoCalc sums over q1 and the
// derivative fields of the last stage
template <typename T>
struct DiagArgs {
    Geom g;
    GasParams gas;
    Q5 q;
    const T *dx[3], *dy[3], *dz[3];
    double *out;
    double meanRho;
};
constexpr int kTurbSums = 11;
template <typename T>
cudaError_t launch_turb(const DiagArgs<T> &a, int blocks, int pass, cudaStream_t s);
cudaError_t launch_shear_info(const DiagArgs<double> &a, cudaStream_t s);
// AeroOptics::computeAO: one warp per (angle, k, i) ray
constexpr int kAeroMaxAngles = 64;
struct AeroArgs {
    Geom g;
    const double *rho;
    double Lx, Ly, Lz, dx, dy, dz, lower;
    int nang;
    int nline[kAeroMaxAngles];
    double dsl[kAeroMaxAngles], dxl[kAeroMaxAngles], dyl[kAeroMaxAngles];
    double *out;  // [nang][Nz][Nx]
};
cudaError_t launch_aero(const AeroArgs &a, cudaStream_t s);
// post-processor: velocity of q1, then |curl u| and the Q-criterion from the
// nine first derivatives d[c][e] = d(u_c)/d(x_e)
struct PostArgs {
    Geom g;
    Q5 q;
    double *vel[3];
    const double *d[3][3];
    double *vort, *qcrit;
};
cudaError_t launch_velocity(const PostArgs &a, cudaStream_t s);
cudaError_t launch_vort_q(const PostArgs &a, cudaStream_t s);
// allocation-free kinetic energy: kKeBlocks partials + the sum in a static
// device array whose address ke_scratch_address returns
constexpr int kKeBlocks = 1024;
cudaError_t ke_scratch_address(double **ptr);
cudaError_t launch_ke_noalloc(const double *rho, const double *ru, const double *rv, const double *rw,
                              long long npts, double *scratch, cudaStream_t s);
cudaError_t launch_wall_pre(const BCArgs &a, cudaStream_t s);
cudaError_t launch_cfl(const CflArgs &a, cudaStream_t s);
cudaError_t launch_nan_scan(const CflArgs &a, cudaStream_t s);
cudaError_t launch_finalize_dt(const DtArgs &a, cudaStream_t s);
cudaError_t launch_sponge_update(const SpongeArgs &a, cudaStream_t s);
cudaError_t launch_ic(const IcArgs &a, cudaStream_t s);
cudaError_t launch_ic_wall(const IcArgs &a, cudaStream_t s);
cudaError_t launch_ic_wall_eos(const IcArgs &a, cudaStream_t s);
cudaError_t launch_primitives(const PrimArgs &a, cudaStream_t s);
cudaError_t launch_shadow(const ShadowArgs &a, cudaStream_t s);

// ---------------------------------------------------------------------
// discrete adjoint of the stage (periodic boundaries)
// ---------------------------------------------------------------------
// k_apply: up to kApplyMax line operators along one direction on XYZ-layout
// fields; task k reads src (+ src2), applies op0 or op1, scales, and writes
// or adds the result to dst, and adds it to dst2.  Each tile reads and
// writes only its own points, so src and dst may be the same array.
constexpr int kApplyMax = 8;
template <typename T>
struct ApplyTask {
    const T *src, *src2;
    T *dst, *dst2;
    T scale;
    int op;   // 0: op0, 1: op1
    int acc;  // 1: dst += v, 0: dst = v
    // FP64 in / FP64 accumulate (ApplyArgs::f64io): v = op(narrowed src64),
    // dst64 += v in FP64 -- the FP32 correction form of a filter on an FP64 field
    const double *src64;
    double *dst64;
};
template <typename T>
struct ApplyArgs {
    Geom g;
    int L, lgL, P, threads;
    FastDiv divN;
    LineOp<T> op0, op1;
    int ntask;
    ApplyTask<T> t[kApplyMax];
    // merge[i]: tasks 2i and 2i+1 write one destination (t[2i].dst), the
    // second adding to the first's result; every other destination (dst and
    // dst2) appears once per launch (the host checks)
    signed char merge[kApplyMax / 2];
    int f64io;  // every task reads src64 and adds into dst64 (see ApplyTask)
};
// Threads per block of k_apply: 256 in FP32 (pair-interleaved tiles, as the
// sweeps), 128 in FP64 (the filter's solves use up to ~250 registers).
template <typename T>
__host__ __device__ constexpr int apply_threads() { return sizeof(T) == 4 ? 256 : 128; }
// primitives U V W T and the 15 Euler fluxes of the state q, in the work type
template <typename T>
struct TapePrepArgs {
    Geom g;
    GasParams gas;
    const T *qin[5];  // the state in the work type (FP64 q, or the FP32 shadow)
    T *prim[4];
    T *flux[15];  // x: rhoU, rhoU U + p, rhoV U, rhoW U, (rhoE + p) U; then y, z
};
template <typename T>
struct VjpArgs {
    Geom g;
    GasParams gas;
    const T *tape[48];
    const double *lam[5];
    // instead of lam (qb2 set): lam = ca qb2 + cb yt, yt optional -- the RK
    // weights of the adjoint stage, formed where they are used
    const double *qb2[5], *yt[5];
    double ca, cb;
    T *gbar[48];
};
// Transposed sweep of one direction (FP32-mixed adjoint): the direction's
// 16 / 15 / 13 transposed line operators (D1^T = -D1, D2^T = D2) on the
// cotangents of its derivative entries in gbar, accumulated into the
// cotangents of the values they were taken of, with the sweeps' tile shapes.
struct TSweepArgs {
    Geom g;
    int L, lgL, P, threads;
    FastDiv divN;
    LineOp<float> d1, d2;
    float *gbar[48];  // cotangents, indexed as the tape (kIn* of cs3d_rhs_adjoint.cuh)
};
cudaError_t launch_tsweep(int dir, const TSweepArgs &a, cudaStream_t s);

template <typename T>
struct ChainArgs {
    Geom g;
    GasParams gas;
    const T *qin[5];
    const T *gbar[48];
    double *out[5];
    double *acc[5];  // optional: acc = out (acc_set) or acc + out
    int acc_set;
};
template <typename T>
struct RhsEvalArgs {
    Geom g;
    GasParams gas;
    const T *tape[48];
    double *R[5];
};
// out = a x + b y (+ c z) on five fields; y, z may be null
struct Lin5Args {
    long long n;
    double *out[5];
    const double *x[5], *y[5], *z[5];
    double a, b, c;
};
// seed of J = mean over points of rho |u|^2 / 2, and per-block partial sums of J
struct KeSeedArgs {
    Geom g;
    Q5 q;
    double *seed[5];
    double *part;
};
template <typename T>
cudaError_t launch_apply(int dir, int H, const ApplyArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_tape_prep(const TapePrepArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_vjp(const VjpArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_chain(const ChainArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_rhs_eval(const RhsEvalArgs<T> &a, cudaStream_t s);
cudaError_t launch_lin5(const Lin5Args &a, cudaStream_t s);
constexpr int kKeSeedBlocks = 512;
cudaError_t launch_ke_seed(const KeSeedArgs &a, cudaStream_t s);

// shared memory of a sweep tile (pair-interleaved for prec_bytes 4) and of
// a planar tile (filter, single operators, adjoint operators)
size_t sweep_smem_bytes(int prec_bytes, int nbuf, int L, int P, int N);
size_t planar_smem_bytes(int prec_bytes, int nbuf, int L, int P, int N);
int sweep_nbuf(int dir, int prec_bytes);
int sweep_ntask(int dir);
int filter_ntask();

}  // namespace cs3d
