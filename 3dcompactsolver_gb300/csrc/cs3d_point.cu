// cs3d_point.cu -- pointwise and face kernels of the stage path (sm_103a):
// wall boundary conditions, CFL reduction, sponge update, initial conditions,
// diagnostics and the FP32 shadow of the state used by the mixed form.
#include <cstdio>
#include <cmath>
#include "cs3d_dev.cuh"
#include "cs3d_kernels.cuh"

namespace cs3d {

// ---------------------------------------------------------------------
// wall boundary conditions before the derivatives (CSolver_AWS.cpp:553-826)
// ---------------------------------------------------------------------
// One launch per face, in the reference's order.  Temperatures of interior
// points come from the current state; on stage 1, points of SPONGE faces that
// are not on a wall use the state saved before the previous step's sponge
// overwrite.  The state is FP64 (q), or only its FP32 shadow (qs) for the
// stage input qk of the mixed RK4 form; a shadow in qs_out is kept in step.
__device__ __forceinline__ double temp_at(const BCArgs &a, long long gi, int fc) {
    double q[5];
    const bool bk = a.use_backup && (fc & a.sponge_faces) && !(fc & a.wall_faces);
#pragma unroll
    for (int f = 0; f < 5; ++f)
        q[f] = bk ? a.backup.f[f][gi] : (a.q.f[0] ? a.q.f[f][gi] : widen(a.qs[f][gi]));
    const double r = q[0];
    const double U = q[1] / r, V = q[2] / r, W = q[3] / r;
    const double p = a.gas.gm1 * (q[4] - 0.5 * r * (U * U + V * V + W * W));
    return p / (r * a.gas.R);
}

// The same temperature in FP32 from the FP32 shadow (mixed form: the stage
// input's shadow is what the sweeps read; FP64 divisions are slow here).
__device__ __forceinline__ float temp_at32(const BCArgs &a, long long gi, int fc) {
    float q[5];
    const bool bk = a.use_backup && (fc & a.sponge_faces) && !(fc & a.wall_faces);
#pragma unroll
    for (int f = 0; f < 5; ++f) q[f] = bk ? narrow(a.backup.f[f][gi]) : a.qs[f][gi];
    const float r = q[0];
    const float U = q[1] / r, V = q[2] / r, W = q[3] / r;
    const float p = (float)a.gas.gm1 * (q[4] - 0.5f * r * (U * U + V * V + W * W));
    return p / (r * (float)a.gas.R);
}

__global__ void k_wall_pre(BCArgs a) {
    const Geom g = a.g;
    const int dir = a.face / 2, hi = a.face % 2;
    const int n1 = dir == 0 ? g.Ny : g.Nx, n2 = dir == 2 ? g.Ny : g.Nz;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n1 * n2) return;
    const int a1 = (int)(idx % n1), a2 = (int)(idx / n1);
    const int Nd = dir == 0 ? g.Nx : dir == 1 ? g.Ny : g.Nz;
    const int fix = hi ? Nd - 1 : 0, sg = hi ? -1 : 1;
    int i, j, k;
    if (dir == 0) { i = fix; j = a1; k = a2; }
    else if (dir == 1) { i = a1; j = fix; k = a2; }
    else { i = a1; j = a2; k = fix; }
    const long long nxy = (long long)g.Nx * g.Ny;
    const long long gi = (long long)k * nxy + (long long)j * g.Nx + i;
    const long long step = dir == 0 ? 1 : dir == 1 ? g.Nx : nxy;
    double Tw;
    if (a.qs[0]) {  // mixed form: FP32 from the shadow
        float Tn[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const long long nb = gi + sg * (m + 1) * step;
            int ii = i, jj = j, kk = k;
            if (dir == 0) ii += sg * (m + 1); else if (dir == 1) jj += sg * (m + 1); else kk += sg * (m + 1);
            Tn[m] = temp_at32(a, nb, faces_of(g, ii, jj, kk));
        }
        Tw = widen((Tn[0] * 360.f - Tn[1] * 450.f + Tn[2] * 400.f - Tn[3] * 225.f + Tn[4] * 72.f - Tn[5] * 10.f) /
                   147.f);
    } else {
        double Tn[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const long long nb = gi + sg * (m + 1) * step;
            int ii = i, jj = j, kk = k;
            if (dir == 0) ii += sg * (m + 1); else if (dir == 1) jj += sg * (m + 1); else kk += sg * (m + 1);
            Tn[m] = temp_at(a, nb, faces_of(g, ii, jj, kk));
        }
        // Utils.hpp:52-54
        Tw = (Tn[0] * 360.0 - Tn[1] * 450.0 + Tn[2] * 400.0 - Tn[3] * 225.0 + Tn[4] * 72.0 - Tn[5] * 10.0) / 147.0;
    }
    const double r = a.q.f[0] ? a.q.f[0][gi] : widen(a.qs[0][gi]);
    double nq[5];
    nq[0] = r;
    nq[1] = dir == 0 ? 0.0 : r * a.uw[0];
    nq[2] = dir == 1 ? 0.0 : r * a.uw[1];
    nq[3] = dir == 2 ? 0.0 : r * a.uw[2];
    const double p = r * a.gas.R * Tw;
    nq[4] = p / a.gas.gm1 + 0.5 * r * (a.uw[0] * a.uw[0] + a.uw[1] * a.uw[1] + a.uw[2] * a.uw[2]);
    if (a.q.f[0])
        for (int f = 1; f < 5; ++f) a.q.f[f][gi] = nq[f];
    if (a.qs_out[0])
        for (int f = 1; f < 5; ++f) a.qs_out[f][gi] = narrow(nq[f]);
}

// ---------------------------------------------------------------------
// CFL reduction (CSolver_AWS.cpp:507-525): max over points of
// (|u|+c)/dx + (|v|+c)/dy + (|w|+c)/dz, kept as the bit pattern of a
// positive double so atomicMax on 64-bit integers orders it.  FP64 from the
// state, or FP32 from its shadow in the mixed form.
// ---------------------------------------------------------------------
__device__ __forceinline__ void block_max_commit(double mx, double *out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = mx;
    __syncthreads();
    if (wid == 0) {
        mx = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) atomicMax(reinterpret_cast<unsigned long long *>(out), (unsigned long long)__double_as_longlong(mx));
    }
}

// kShadow: the mixed form's FP32 shadow, else the FP64 state (two instances:
// the FP64 branch's registers would otherwise cost the FP32 pass occupancy)
template <bool kShadow>
__global__ void k_cfl(CflArgs a) {
    double mx = 0.0;
    int bad = 0;
    if constexpr (kShadow) {
        // FP32 shadow: four consecutive points per thread (128-bit loads of
        // the 16-byte aligned arrays), one reciprocal of rho per point
        float fm = 0.f;
        const float gam = (float)a.gas.gamma, gm1 = (float)a.gas.gm1;
        const float idx = a.idx, idy = a.idy, idz = a.idz;
        auto point = [&](float r, float ru, float rv, float rw, float re) {
            const float ir = 1.0f / r;
            const float U = ru * ir, V = rv * ir, W = rw * ir;
            const float p = gm1 * (re - 0.5f * r * (U * U + V * V + W * W));
            const float c = sqrtf(gam * p * ir);
            const float v = (fabsf(U) + c) * idx + (fabsf(V) + c) * idy + (fabsf(W) + c) * idz;
            bad |= !(v == v) || isinf(v);
            fm = fmaxf(fm, v);
        };
        const long long n4 = a.g.npts >> 2;
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
             i += (long long)gridDim.x * blockDim.x) {
            float4 q[5];
#pragma unroll
            for (int f = 0; f < 5; ++f) q[f] = __ldg(reinterpret_cast<const float4 *>(a.qs[f]) + i);
            point(q[0].x, q[1].x, q[2].x, q[3].x, q[4].x);
            point(q[0].y, q[1].y, q[2].y, q[3].y, q[4].y);
            point(q[0].z, q[1].z, q[2].z, q[3].z, q[4].z);
            point(q[0].w, q[1].w, q[2].w, q[3].w, q[4].w);
        }
        for (long long gi = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
             gi += (long long)gridDim.x * blockDim.x)
            point(a.qs[0][gi], a.qs[1][gi], a.qs[2][gi], a.qs[3][gi], a.qs[4][gi]);
        mx = widen(fm);
    } else {
        for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
             gi += (long long)gridDim.x * blockDim.x) {
            // one reciprocal of rho and the host's 1/dx, 1/dy, 1/dz instead of
            // seven FP64 divisions (within an ulp of the quotients)
            const double r = a.q.f[0][gi], ir = __drcp_rn(r);
            const double U = a.q.f[1][gi] * ir, V = a.q.f[2][gi] * ir, W = a.q.f[3][gi] * ir;
            const double p = a.gas.gm1 * (a.q.f[4][gi] - 0.5 * r * (U * U + V * V + W * W));
            const double c = sqrt(a.gas.gamma * p * ir);
            const double v = (fabs(U) + c) * a.idx64 + (fabs(V) + c) * a.idy64 + (fabs(W) + c) * a.idz64;
            bad |= !(v == v) || isinf(v);
            mx = fmax(mx, v);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *a.nan_flag = 1;
    block_max_commit(mx, a.max_out);
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
    // the averaging weight, once per block (FP64 divisions are slow)
    __shared__ double eps_s;
    if (threadIdx.x == 0) eps_s = 1.0 / (a.avgT / *a.dt + 1.0);
    __syncthreads();
    const double eps = eps_s;
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
            const int k = (int)(gi / nxy);
            const long long rem = gi - k * nxy;
            const int j = (int)(rem / a.g.Nx), i = (int)(rem - (long long)j * a.g.Nx);
            if (faces_of(a.g, i, j, k) & a.sponge_kind_faces) {
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    a.backup.f[f][gi] = a.q1.f[f][gi];
                    a.q1.f[f][gi] = av[f];
                    if (a.q1s[0]) a.q1s[f][gi] = narrow(av[f]);
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

// FP32 shadow of an FP64 state (nf fields): out = narrow(q); or, when in is
// set, the reverse: q = widen(in).
__global__ void k_shadow(ShadowArgs a) {
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        for (int f = 0; f < a.nf; ++f) {
            if (a.in[0]) a.q.f[f][gi] = widen(a.in[f][gi]);
            else a.out[f][gi] = narrow(a.q.f[f][gi]);
        }
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
// launches
// ---------------------------------------------------------------------
static int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152 * 16) b = 152 * 16;
    if (b < 1) b = 1;
    return (int)b;
}

static long long face_points(const Geom &g, int face) {
    const int dir = face / 2;
    return dir == 0 ? (long long)g.Ny * g.Nz : dir == 1 ? (long long)g.Nx * g.Nz : (long long)g.Nx * g.Ny;
}

cudaError_t launch_wall_pre(const BCArgs &a, cudaStream_t s) {
    k_wall_pre<<<(unsigned)((face_points(a.g, a.face) + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_cfl(const CflArgs &a, cudaStream_t s) {
    if (a.qs[0]) k_cfl<true><<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    else k_cfl<false><<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
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
    k_ic_wall<<<(unsigned)((face_points(a.g, a.face) + 255) / 256), 256, 0, s>>>(a);
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
cudaError_t launch_shadow(const ShadowArgs &a, cudaStream_t s) {
    k_shadow<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------
// calcTurbulenceQuantities (CSolver_AWS.cpp:2033-2173): per-block partial
// sums, each term divided by the point count as the reference does; pass 0
// gives meanRho, meanMu, meanTurbDiss, uprime, uiprime, urms, meanSOS,
// taylor2_denom, meanKineticEng and the dilatation and vorticity sums, pass 1
// the density variance about meanRho.
// ---------------------------------------------------------------------
template <int NS>
__device__ __forceinline__ void block_sums(double (&s)[NS], double *out) {
    __shared__ double red[NS][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        double v = s[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[i][wid] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < NS) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
        out[threadIdx.x] = v;
    }
}

template <typename T>
__global__ void k_turb(DiagArgs<T> a, int pass) {
    const double n = (double)a.g.npts;
    double s[kTurbSums];
#pragma unroll
    for (int i = 0; i < kTurbSums; ++i) s[i] = 0.0;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        const double r = a.q.f[0][gi];
        if (pass == 1) {
            s[0] += ((r - a.meanRho) * (r - a.meanRho)) / n;
            continue;
        }
        const double Ux = to_f64(a.dx[0][gi]), Vx = to_f64(a.dx[1][gi]), Wx = to_f64(a.dx[2][gi]);
        const double Uy = to_f64(a.dy[0][gi]), Vy = to_f64(a.dy[1][gi]), Wy = to_f64(a.dy[2][gi]);
        const double Uz = to_f64(a.dz[0][gi]), Vz = to_f64(a.dz[1][gi]), Wz = to_f64(a.dz[2][gi]);
        const double U = a.q.f[1][gi] / r, V = a.q.f[2][gi] / r, W = a.q.f[3][gi] / r;
        const double p = a.gas.gm1 * (a.q.f[4][gi] - 0.5 * r * (U * U + V * V + W * W));
        const double mu = a.gas.mu_ref * pow(p / (r * a.gas.R), 0.76);
        const double sos = sqrt(a.gas.gamma * p / r);
        const double dv = Ux + Vy + Wz;
        const double S00 = 0.5 * (Ux + Ux) - (1.0 / 3.0) * dv, S11 = 0.5 * (Vy + Vy) - (1.0 / 3.0) * dv,
                     S22 = 0.5 * (Wz + Wz) - (1.0 / 3.0) * dv;
        const double S01 = 0.5 * (Uy + Vx), S02 = 0.5 * (Uz + Wx), S12 = 0.5 * (Vz + Wy);
        double td = S00 * Ux;
        td += S01 * Uy;
        td += S02 * Uz;
        td += S01 * Vx;
        td += S11 * Vy;
        td += S12 * Vz;
        td += S02 * Wx;
        td += S12 * Wy;
        td += S22 * Wz;
        td *= 2 * mu;
        const double uvar = (U * U + V * V + W * W);
        s[0] += r / n;
        s[1] += mu / n;
        s[2] += td / n;
        s[3] += uvar / 3.0 / n;
        s[4] += (Ux * Ux + Vy * Vy + Wz * Wz) / 3.0 / n;
        s[5] += uvar / n;
        s[6] += sos / n;
        s[7] += (Ux * Ux) / n;
        s[8] += r * uvar / n / 2.0;
        s[9] += (dv * dv) / n;
        const double wx = Wy - Vz, wy = Uz - Wx, wz = Vx - Uy;
        s[10] += ((wx * wx + wy * wy + wz * wz)) / n;
    }
    block_sums<kTurbSums>(s, a.out + (size_t)blockIdx.x * kTurbSums);
}

template <typename T>
cudaError_t launch_turb(const DiagArgs<T> &a, int blocks, int pass, cudaStream_t s) {
    k_turb<T><<<blocks, 256, 0, s>>>(a, pass);
    return cudaGetLastError();
}
template cudaError_t launch_turb<double>(const DiagArgs<double> &, int, int, cudaStream_t);
template cudaError_t launch_turb<float>(const DiagArgs<float> &, int, int, cudaStream_t);

// ---------------------------------------------------------------------
// shearLayerInfoCalc (CSolver_AWS.cpp:2259-2456): one block per y plane; the
// x-z means of rho, U, V, W, p, T, then the second moments about them.  The
// reference adds the v'w' sum into uwprime (:2318) and leaves vwprime at 0;
// rows 13 and 14 reproduce that, rows 15 and 16 hold u'w' and v'w'.
// ---------------------------------------------------------------------
__global__ void k_shear_info(DiagArgs<double> a) {
    const int j = blockIdx.x;
    const int Nx = a.g.Nx, Ny = a.g.Ny, Nz = a.g.Nz;
    const long long nxz = (long long)Nx * Nz;
    const double n = (double)nxz;
    __shared__ double mean[6];
    double s[6] = {0, 0, 0, 0, 0, 0};
    auto prims = [&](long long m, double v[6]) {
        const int i = (int)(m % Nx), k = (int)(m / Nx);
        const long long gi = ((long long)k * Ny + j) * Nx + i;
        const double r = a.q.f[0][gi];
        const double U = a.q.f[1][gi] / r, V = a.q.f[2][gi] / r, W = a.q.f[3][gi] / r;
        const double p = a.gas.gm1 * (a.q.f[4][gi] - 0.5 * r * (U * U + V * V + W * W));
        v[0] = r; v[1] = U; v[2] = V; v[3] = W; v[4] = p; v[5] = p / (r * a.gas.R);
    };
    for (long long m = threadIdx.x; m < nxz; m += blockDim.x) {
        double v[6];
        prims(m, v);
#pragma unroll
        for (int f = 0; f < 6; ++f) s[f] += v[f] / n;
    }
    double red6[6];
    block_sums<6>(s, red6);  // threads 0..5 hold the plane sums
    __syncthreads();
    if (threadIdx.x < 6) mean[threadIdx.x] = red6[threadIdx.x];
    __syncthreads();
    double t[11];
#pragma unroll
    for (int f = 0; f < 11; ++f) t[f] = 0.0;
    for (long long m = threadIdx.x; m < nxz; m += blockDim.x) {
        double v[6], d[6];
        prims(m, v);
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            d[f] = v[f] - mean[f];
            t[f] += d[f] * d[f] / n;
        }
        t[6] += d[1] * d[2] / n;
        t[7] += d[1] * d[3] / n;
        t[7] += d[2] * d[3] / n;
        t[9] += d[1] * d[3] / n;
        t[10] += d[2] * d[3] / n;
    }
    double red11[11];
    __syncthreads();
    block_sums<11>(t, red11);
    if (threadIdx.x < 6) a.out[(size_t)threadIdx.x * Ny + j] = mean[threadIdx.x];
    if (threadIdx.x < 11) a.out[(size_t)(6 + threadIdx.x) * Ny + j] = red11[threadIdx.x];
}

cudaError_t launch_shear_info(const DiagArgs<double> &a, cudaStream_t s) {
    k_shear_info<<<a.g.Ny, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------
// AeroOptics::computeAO (AeroOptics.cpp:45-93): trapezoidal integrals of the
// density along tilted rays, trilinear interpolation as linearInterpolation
// (Utils.cpp:261-331) with the base index kept at most N-2 (the reference
// reads one plane past its arrays for a point exactly on the last plane,
// where that plane's weight is 0).  Grid coordinates as Domain
// (x_i = i/(N-1) * L).  One warp per ray; the lanes take every 32nd sample.
// ---------------------------------------------------------------------
__device__ __forceinline__ double grid_coord(int i, int N, double L) { return ((double)i / ((double)N - 1.0)) * L; }

__device__ double aero_interp(const AeroArgs &a, const double xp[3]) {
    const int Nx = a.g.Nx, Ny = a.g.Ny, Nz = a.g.Nz;
    int b0 = min((int)(xp[0] / a.dx), Nx - 2);
    int b1 = min((int)(xp[1] / a.dy), Ny - 2);
    int b2 = min((int)(xp[2] / a.dz), Nz - 2);
    const double x0 = grid_coord(b0, Nx, a.Lx), x1 = grid_coord(b0 + 1, Nx, a.Lx);
    const double y0 = grid_coord(b1, Ny, a.Ly), y1 = grid_coord(b1 + 1, Ny, a.Ly);
    const double z0 = grid_coord(b2, Nz, a.Lz), z1 = grid_coord(b2 + 1, Nz, a.Lz);
    const double xd = (xp[0] - x0) / (x1 - x0), yd = (xp[1] - y0) / (y1 - y0), zd = (xp[2] - z0) / (z1 - z0);
    const long long sy = Nx, sz = (long long)Nx * Ny;
    const long long i000 = b2 * sz + b1 * sy + b0;
    const double *f = a.rho;
    const double c000 = f[i000], c001 = f[i000 + sz], c010 = f[i000 + sy], c011 = f[i000 + sy + sz];
    const double c100 = f[i000 + 1], c101 = f[i000 + 1 + sz], c110 = f[i000 + 1 + sy], c111 = f[i000 + 1 + sy + sz];
    const double c00 = c000 * (1 - xd) + c100 * xd;
    const double c01 = c001 * (1 - xd) + c101 * xd;
    const double c10 = c010 * (1 - xd) + c110 * xd;
    const double c11 = c011 * (1 - xd) + c111 * xd;
    const double c0 = c00 * (1 - yd) + c10 * yd;
    const double c1 = c01 * (1 - yd) + c11 * yd;
    return c0 * (1 - zd) + c1 * zd;
}

__global__ void k_aero(AeroArgs a) {
    const int lane = threadIdx.x & 31;
    const long long nray = (long long)a.nang * a.g.Nz * a.g.Nx;
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nray;
         r += ((long long)gridDim.x * blockDim.x) >> 5) {
        const int i = (int)(r % a.g.Nx);
        const int k = (int)((r / a.g.Nx) % a.g.Nz);
        const int ap = (int)(r / ((long long)a.g.Nx * a.g.Nz));
        const int nl = a.nline[ap];
        const double dsl = a.dsl[ap], dxl = a.dxl[ap], dyl = a.dyl[ap];
        const double xi = grid_coord(i, a.g.Nx, a.Lx), zk = grid_coord(k, a.g.Nz, a.Lz);
        double acc = 0.0;
        for (int sp = lane; sp < nl; sp += 32) {
            const double xp[3] = {fmod(xi + (double)(sp * dxl), a.Lx), a.lower + (double)(sp * dyl), zk};
            const double v = aero_interp(a, xp);
            acc += (sp == 0 || sp == nl - 1) ? v * dsl / 2.0 : v * dsl;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) a.out[r] = acc;
    }
}

cudaError_t launch_aero(const AeroArgs &a, cudaStream_t s) {
    const long long nray = (long long)a.nang * a.g.Nz * a.g.Nx;
    long long blocks = (nray * 32 + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_aero<<<(unsigned)blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------
// post-processor (PostProcess.cpp:190-310): U, V, W of q1, then per point the
// vorticity magnitude and Q = |W|^2/2 - |S|^2/2, S and W the symmetric and
// antisymmetric parts of the velocity gradient, summed in the reference's
// order
// ---------------------------------------------------------------------
__global__ void k_velocity(PostArgs a) {
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        const double r = a.q.f[0][gi];
        a.vel[0][gi] = a.q.f[1][gi] / r;
        a.vel[1][gi] = a.q.f[2][gi] / r;
        a.vel[2][gi] = a.q.f[3][gi] / r;
    }
}

__global__ void k_vort_q(PostArgs a) {
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < a.g.npts;
         gi += (long long)gridDim.x * blockDim.x) {
        const double Ux = a.d[0][0][gi], Uy = a.d[0][1][gi], Uz = a.d[0][2][gi];
        const double Vx = a.d[1][0][gi], Vy = a.d[1][1][gi], Vz = a.d[1][2][gi];
        const double Wx = a.d[2][0][gi], Wy = a.d[2][1][gi], Wz = a.d[2][2][gi];
        const double vx = Wy - Vz, vy = Uz - Wx, vz = Vx - Uy;
        a.vort[gi] = sqrt(vx * vx + vy * vy + vz * vz);
        const double s01 = 0.5 * (Uy + Vx), s12 = 0.5 * (Vz + Wy), s02 = 0.5 * (Uz + Wx);
        const double w01 = 0.5 * (Uy - Vx), w12 = 0.5 * (Vz - Wy), w02 = 0.5 * (Uz - Wx);
        // the nine products of each tensor in row order, as the reference sums them
        const double om2 = 0.5 * (0.0 * 0.0 + w01 * w01 + w02 * w02 + (-w01) * (-w01) + 0.0 * 0.0 + w12 * w12 +
                                  (-w02) * (-w02) + (-w12) * (-w12) + 0.0 * 0.0);
        const double st2 = 0.5 * (Ux * Ux + s01 * s01 + s02 * s02 + s01 * s01 + Vy * Vy + s12 * s12 + s02 * s02 +
                                  s12 * s12 + Wz * Wz);
        a.qcrit[gi] = om2 - st2;
    }
}

cudaError_t launch_velocity(const PostArgs &a, cudaStream_t s) {
    k_velocity<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_vort_q(const PostArgs &a, cudaStream_t s) {
    k_vort_q<<<grid_for(a.g.npts, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------
// Kinetic energy without any allocation: the KEsum column of the
// Taylor-Green diagnostics (CSolver_AWS.cpp:2175-2236) from four device
// arrays, with its partial sums in a fixed file-scope scratch array instead
// of handle memory.  Same launch shape, per-thread order and reduction tree
// as k_tgv, so the two agree.  Every call writes all kKeBlocks partials and
// the result before reading them: nothing in the scratch needs to start at
// zero, and two calls that overlap on one device race on it.
// ---------------------------------------------------------------------
static __device__ __align__(256) double g_ke_scratch[kKeBlocks + 1];

__global__ void k_ke_partials(const double *__restrict__ rho, const double *__restrict__ ru,
                              const double *__restrict__ rv, const double *__restrict__ rw,
                              long long npts, double *part) {
    double s = 0.0;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < npts;
         gi += (long long)gridDim.x * blockDim.x) {
        double r = rho[gi];
        double U = ru[gi] / r, V = rv[gi] / r, W = rw[gi] / r;
        s += r * (U * U + V * V + W * W) / 2.0;
    }
    __shared__ double red[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
        part[blockIdx.x] = v;
    }
}

// one thread adds the partials in block order, as the host does for k_tgv
__global__ void k_ke_final(double *part) {
    double s = 0.0;
    for (int b = 0; b < kKeBlocks; ++b) s += part[b];
    part[kKeBlocks] = s;
}

cudaError_t ke_scratch_address(double **ptr) {
    return cudaGetSymbolAddress((void **)ptr, g_ke_scratch);
}

cudaError_t launch_ke_noalloc(const double *rho, const double *ru, const double *rv, const double *rw,
                              long long npts, double *scratch, cudaStream_t s) {
    k_ke_partials<<<kKeBlocks, 256, 0, s>>>(rho, ru, rv, rw, npts, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_ke_final<<<1, 1, 0, s>>>(scratch);
    return cudaGetLastError();
}

}  // namespace cs3d
