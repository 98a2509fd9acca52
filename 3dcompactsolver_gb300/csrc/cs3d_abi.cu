// cs3d_abi.cu -- C ABI of the GB300 stage path: solver handle, device memory,
// precomputed line operators and the order of launches of one time step.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <cstdlib>
#include <initializer_list>

#include "../../include/cs3d.h"
#include "cs3d_dev.cuh"
#include "cs3d_kernels.cuh"
#include "cs3d_rhs_adjoint.cuh"  // kIn* slots of the adjoint tape

using namespace cs3d;

// ---------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------
static thread_local char g_err[512] = "";

static int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CS3D_CUDA(call)                                                                           \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(CS3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

extern "C" const char *cs3d_last_error(void) { return g_err; }

extern "C" int cs3d_version(int *major, int *minor, int *sm_arch) {
    if (major) *major = 1;
    if (minor) *minor = 0;
    if (sm_arch) *sm_arch = 103;
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// compact operator coefficients (Derivatives.hpp:79-161, Filter.hpp:54-104)
// ---------------------------------------------------------------------
namespace {

struct HostOp {
    std::vector<double> m, iw, c, z;
    std::vector<double> alo, aup;  // off-diagonals of A (unit diagonal), before any cyclic modification
    double taps[kTaps] = {0};
    double btaps[2 * kMaxH][kTaps] = {{0}};
    int boff[2 * kMaxH] = {0};
    double scale = 1.0, bog = 0.0, inv_den = 0.0;
    int N = 0, H = 2, periodic = 1;
};

// Thomas algorithm exactly as Utils.cpp:4-20, for the Sherman-Morrison vector.
void thomas(const std::vector<double> &a, const std::vector<double> &b, const std::vector<double> &c,
            const std::vector<double> &d, std::vector<double> &x) {
    int n = (int)b.size();
    std::vector<double> w(b);
    x = d;
    for (int i = 1; i < n; i++) {
        double mm = a[i] / w[i - 1];
        w[i] = w[i] - mm * c[i - 1];
        x[i] = x[i] - mm * x[i - 1];
    }
    x[n - 1] /= w[n - 1];
    for (int i = n - 2; i >= 0; i--) x[i] = (x[i] - c[i] * x[i + 1]) / w[i];
}

// kind: 1 = first derivative, 2 = second derivative, 3 = filter.
HostOp make_op(int kind, int N, int bc, double dh, double alphaF) {
    HostOp op;
    op.N = N;
    op.periodic = bc == CS3D_PERIODIC_SOLVE;
    op.H = kind == 3 ? 4 : 2;
    std::vector<double> lo(N), di(N, 1.0), up(N);
    double alpha;
    // interior coefficients
    const double a1 = 14.0 / 9.0, b1 = 1.0 / 9.0;                 // Derivatives.hpp:81-83
    const double a2 = 12.0 / 11.0, b2 = 3.0 / 11.0;               // :101-103
    double t[kTaps] = {0};
    if (kind == 1) {
        alpha = 1.0 / 3.0;
        t[2] = -b1 / 4.0; t[3] = -a1 / 2.0; t[5] = a1 / 2.0; t[6] = b1 / 4.0;  // Derivatives.cpp:121-124
        op.scale = 1.0 / dh;
    } else if (kind == 2) {
        alpha = 2.0 / 11.0;
        t[2] = b2 / 4.0; t[3] = a2; t[4] = -(b2 / 2.0 + 2.0 * a2); t[5] = a2; t[6] = b2 / 4.0;  // :155-159
        op.scale = 1.0 / (dh * dh);
    } else {
        alpha = alphaF;
        // Filter.hpp:54-58, Filter.cpp:7-11
        double a0_8 = (93.0 + 70.0 * alphaF) / 128.0, a1_8 = (7.0 + 18.0 * alphaF) / 16.0;
        double a2_8 = (-7.0 + 14.0 * alphaF) / 32.0, a3_8 = (1.0 - 2.0 * alphaF) / 16.0;
        double a4_8 = (-1.0 + 2.0 * alphaF) / 128.0;
        double cc[5] = {a0_8, a1_8 / 2.0, a2_8 / 2.0, a3_8 / 2.0, a4_8 / 2.0};
        for (int k = 0; k <= 4; k++) { t[4 + k] = cc[k]; t[4 - k] = cc[k]; }
        op.scale = 1.0;
    }
    for (int i = 0; i < N; i++) { lo[i] = alpha; up[i] = alpha; }
    std::memcpy(op.taps, t, sizeof(t));
    const int H = op.H;
    if (op.periodic) {
        for (int b = 0; b < 2 * H; b++) {
            int row = b < H ? b : N - 2 * H + b;
            std::memcpy(op.btaps[b], t, sizeof(t));
            op.boff[b] = row - kMaxH;
        }
        // cyclic system (Utils.cpp:22-46): gamma = -b0, modified corners
        double gamma = -di[0];
        std::vector<double> bb(di);
        bb[0] = di[0] - gamma;
        bb[N - 1] = di[N - 1] - alpha * alpha / gamma;
        std::vector<double> u(N, 0.0);
        u[0] = gamma;
        u[N - 1] = alpha;
        thomas(lo, bb, up, u, op.z);
        op.bog = alpha / gamma;
        op.inv_den = 1.0 / (1.0 + op.z[0] + alpha * op.z[N - 1] / gamma);
        di = bb;
    } else {
        auto set = [&](int b, int off, std::initializer_list<double> v) {
            int k = 0;
            for (double x : v) op.btaps[b][k++] = x;
            op.boff[b] = off;
        };
        if (kind == 1) {
            // Derivatives.hpp:85-97, Derivatives.cpp:191-205
            const double A1 = -197.0 / 60.0, B1 = -5.0 / 12.0, C1 = 5.0, D1 = -5.0 / 3.0, E1 = 5.0 / 12.0,
                         F1 = -1.0 / 20.0;
            const double A2 = -43.0 / 96.0, B2 = -5.0 / 6.0, C2 = 9.0 / 8.0, D2 = 1.0 / 6.0, E2 = -1.0 / 96.0;
            set(0, 0, {A1, B1, C1, D1, E1, F1});
            set(1, 0, {A2, B2, C2, D2, E2});
            set(2, N - 5, {-E2, -D2, -C2, -B2, -A2});
            set(3, N - 6, {-F1, -E1, -D1, -C1, -B1, -A1});
            up[0] = 5.0; up[1] = 3.0 / 4.0; lo[1] = 1.0 / 8.0;        // Derivatives.hpp:145-151
            lo[N - 1] = 5.0; lo[N - 2] = 3.0 / 4.0; up[N - 2] = 1.0 / 8.0;
        } else if (kind == 2) {
            // Derivatives.hpp:106-120, Derivatives.cpp:225-240
            const double A1 = 145.0 / 12.0, B1 = -76.0 / 3.0, C1 = 29.0 / 2.0, D1 = -4.0 / 3.0, E1 = 1.0 / 12.0;
            const double A2 = 177.0 / 88.0, B2 = -507.0 / 44.0, C2 = 783.0 / 44.0, D2 = -201.0 / 22.0,
                         E2 = 81.0 / 88.0, F2 = -3.0 / 44.0;
            set(0, 0, {A1, B1, C1, D1, E1});
            set(1, 0, {A2, B2, C2, D2, E2, F2});
            set(2, N - 6, {F2, E2, D2, C2, B2, A2});
            set(3, N - 5, {E1, D1, C1, B1, A1});
            up[0] = 10.0; up[1] = -131.0 / 22.0; lo[1] = 2.0 / 11.0;  // Derivatives.hpp:153-159
            lo[N - 1] = 10.0; lo[N - 2] = -131.0 / 22.0; up[N - 2] = 2.0 / 11.0;
        } else {
            // Filter.hpp:60-81, Filter.cpp:64-89
            double a0_6 = (11.0 + 10.0 * alphaF) / 16.0, a1_6 = (15.0 + 34.0 * alphaF) / 32.0;
            double a2_6 = (-3.0 + 6.0 * alphaF) / 16.0, a3_6 = (1.0 - 2.0 * alphaF) / 32.0;
            double aa0 = a0_6, aa1 = a1_6 / 2.0, aa2 = a2_6 / 2.0, aa3 = a3_6 / 2.0;
            const double A0 = 15.0 / 16.0, A1 = 4.0 / 16.0, A2 = -6.0 / 16.0, A3 = 4.0 / 16.0, A4 = -1.0 / 16.0;
            const double B0 = 1.0 / 16.0, B1 = 3.0 / 4.0, B2 = 6.0 / 16.0, B3 = -4.0 / 16.0, B4 = 1.0 / 16.0;
            const double C0 = -1.0 / 16.0, C1 = 4.0 / 16.0, C2 = 5.0 / 8.0, C3 = 4.0 / 16.0, C4 = -1.0 / 16.0;
            set(0, 0, {A0, A1, A2, A3, A4});
            set(1, 0, {B0, B1, B2, B3, B4});
            set(2, 0, {C0, C1, C2, C3, C4});
            set(3, 0, {aa3, aa2, aa1, aa0, aa1, aa2, aa3});
            set(4, N - 7, {aa3, aa2, aa1, aa0, aa1, aa2, aa3});
            set(5, N - 5, {C4, C3, C2, C1, C0});
            set(6, N - 5, {B4, B3, B2, B1, B0});
            set(7, N - 5, {A4, A3, A2, A1, A0});
            for (int r = 0; r < 3; r++) {  // Filter.hpp:89-104
                lo[r] = 0.0; up[r] = 0.0;
                lo[N - 1 - r] = 0.0; up[N - 1 - r] = 0.0;
            }
        }
    }
    op.alo = lo;
    op.aup = up;
    // Thomas factors of the (possibly corner-modified) matrix
    op.m.assign(N, 0.0);
    op.iw.assign(N, 0.0);
    op.c = up;
    std::vector<double> w(di);
    for (int i = 1; i < N; i++) {
        op.m[i] = lo[i] / w[i - 1];
        w[i] = w[i] - op.m[i] * up[i - 1];
    }
    for (int i = 0; i < N; i++) op.iw[i] = 1.0 / w[i];
    if (!op.periodic) op.z.assign(N, 0.0);
    return op;
}

// The filter's correction operator F - I = A^-1 (B - A): the same left-hand
// side, right-hand-side rows B - A.  Its taps are small and sum to zero, so in
// FP32 the rounding of the coefficients changes only the (small) correction
// and not the gain of the filter at the energy-carrying wavenumbers, which
// the FP32 form of F itself would (a drift of the kinetic energy by about
// 1e-8 per filter pass).
HostOp make_filter_correction(const HostOp &F) {
    HostOp d = F;
    const int H = F.H, N = F.N;
    d.taps[kMaxH] -= 1.0;  // interior rows of A: alpha, 1, alpha
    d.taps[kMaxH - 1] -= F.alo[N / 2];
    d.taps[kMaxH + 1] -= F.aup[N / 2];
    for (int b = 0; b < 2 * H; b++) {
        const int row = b < H ? b : N - 2 * H + b;
        const int col = row - F.boff[b];  // the row's own position among its taps
        d.btaps[b][col] -= 1.0;
        if (col > 0) d.btaps[b][col - 1] -= F.alo[row];
        if (col + 1 < kTaps) d.btaps[b][col + 1] -= F.aup[row];
    }
    return d;
}

// Device copy of an operator in precision T.
template <typename T>
struct DevOp {
    T *mem = nullptr;
    LineOp<T> op{};
};

template <typename T>
int upload_op(const HostOp &h, DevOp<T> &d, cudaStream_t s) {
    const int N = h.N;
    // seven arrays of S elements each (S a multiple of 4, with at least 8
    // elements of zero padding so chunked loads never leave an array)
    const size_t S = ((size_t)N + 8 + 3) & ~(size_t)3;
    std::vector<T> buf(7 * S, T(0));
    for (int i = 0; i < N; i++) {
        buf[i] = (T)h.m[i];
        buf[S + i] = (T)h.iw[i];
        buf[2 * S + i] = (T)h.c[i];
        buf[3 * S + i] = (T)h.z[i];
    }
    for (int k = 0; k + h.H < N; k++) buf[4 * S + k] = (T)h.m[k + h.H];
    for (int k = 0; k <= N - 2; k++) {
        buf[5 * S + k] = (T)h.c[N - 2 - k];
        buf[6 * S + k] = (T)h.iw[N - 2 - k];
    }
    CS3D_CUDA(cudaMalloc(&d.mem, sizeof(T) * buf.size()));
    CS3D_CUDA(cudaMemcpyAsync(d.mem, buf.data(), sizeof(T) * buf.size(), cudaMemcpyHostToDevice, s));
    CS3D_CUDA(cudaStreamSynchronize(s));
    LineOp<T> &o = d.op;
    o.m = d.mem;
    o.iw = d.mem + S;
    o.c = d.mem + 2 * S;
    o.z = d.mem + 3 * S;
    o.mf = d.mem + 4 * S;
    o.cbk = d.mem + 5 * S;
    o.ibk = d.mem + 6 * S;
    // the 1/h or 1/h^2 of the right-hand side is folded into the taps
    for (int k = 0; k < kTaps; k++) o.taps[k] = (T)(h.taps[k] * h.scale);
    for (int b = 0; b < 2 * kMaxH; b++) {
        for (int k = 0; k < kTaps; k++) o.btaps[b][k] = (T)(h.btaps[b][k] * h.scale);
        o.boff[b] = h.boff[b];
    }
    o.scale = (T)h.scale;
    // the run of rows around the middle with bitwise constant factors in T
    o.klo = o.khi = 1;
    if (N >= 8) {
        const int mid = N / 2;
        auto same = [&](int i) {
            return (T)h.m[i] == (T)h.m[mid] && (T)h.iw[i] == (T)h.iw[mid] && (T)h.c[i] == (T)h.c[mid];
        };
        int lo = mid, hi = mid + 1;
        while (lo > 1 && same(lo - 1)) --lo;
        while (hi < N - 1 && same(hi)) ++hi;
        // at least kU: a chunk of the back substitution inside the run then
        // reads ahead no row below 0
        o.klo = std::max(lo, kU);
        o.khi = hi;
    }
    o.km = (T)h.m[N / 2];
    o.kiw = (T)h.iw[N / 2];
    o.kc = (T)h.c[N / 2];
    o.bog = h.bog;
    o.inv_den = h.inv_den;
    o.N = N;
    o.H = h.H;
    o.periodic = h.periodic;
    return CS3D_OK;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

// ---------------------------------------------------------------------
// the handle
// ---------------------------------------------------------------------
// FP64 five-field groups of the adjoint workspace
enum AdjField { ADJ_Y2 = 0, ADJ_Y3, ADJ_Y4, ADJ_QB, ADJ_QB2, ADJ_LAM, ADJ_YS, ADJ_YT, ADJ_FIN, kAdjFields };

struct cs3d_handle {
    cs3d_config cfg;
    int dev = 0;
    cudaStream_t stream = nullptr;
    Geom g{};
    GasParams gas{};
    double dx = 0, dy = 0, dz = 0;
    int nstages = 4;
    int mixed = 0;
    size_t tb = 8;  // bytes of the work type
    // conserved state, and its FP32 shadows in the mixed form
    Q5 q1{}, qk{}, q2{};
    float *q1s[5] = {}, *qks[5] = {}, *q2s[5] = {};
    int mixed_rk4 = 0;  // mixed form with RK4: the stage input qk lives in qks only
    float *rfluct[5] = {};  // mixed RK4: q2 - fref in FP32 after a filtered step's last stage
    double *dq[5] = {};
    // work-precision fields (double or float, by tb)
    void *prim[5] = {}, *mu = nullptr, *amu = nullptr, *dx4[4] = {}, *dy4[4] = {}, *R[5] = {}, *diag[3] = {};
    // filter temporaries (work precision) and FP64 temporaries of the plain form
    void *ft1[5] = {}, *ft2[5] = {};
    double fref[5] = {0, 0, 0, 0, 0};
    // sponge
    int sponge = 0;
    double *sigma = nullptr;
    Q5 savg{}, backup{};
    int backup_valid = 0;
    int wall_faces = 0, sponge_kind_faces = 0;
    // scalars on device: dt, time, cfl max, nan flag
    double *scal = nullptr;
    int *flag = nullptr;
    // operators: [dir][kind-1]
    DevOp<double> op64[3][3];
    DevOp<float> op32[3][3];
    DevOp<float> op32fc[3];  // FP32 filter correction F - I (mixed form)
    // tiles
    int L[3] = {1, 1, 1}, Lf[3] = {1, 1, 1}, threads[3] = {128, 128, 128};
    // step state
    int timeStep = 0, filterTimeStep = 0;
    int ic_done = 0;
    int store_dq = 0, store_diag = 0;
    long long launches = 0;
    // optional per-kernel timing with CUDA events on the handle's stream
    int timing = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    double k_ms[CS3D_NUM_KERNEL_CLASSES] = {0};
    long long k_count[CS3D_NUM_KERNEL_CLASSES] = {0};
    int k_cur = -1;
    cudaEvent_t k_ev0 = nullptr;
    double *prim_out = nullptr;  // 7 FP64 fields for cs3d_get_field of primitives
    double *red = nullptr;       // reduction scratch
    double *shear_buf = nullptr; // 17 x Ny per-plane statistics
    double *post_buf = nullptr;  // 14 FP64 fields of the post-processor
    double *aero_buf = nullptr;  // optical path integrals
    size_t aero_cap = 0;
    std::vector<void *> allocs;
    // discrete adjoint: workspace (allocated on first use) and the record of
    // the forward steps (checkpoints every adj_every steps)
    std::vector<void *> adj_allocs, adj_rec_allocs;
    int adj_ws = 0;
    void *adj_tape[48] = {}, *adj_gbar[48] = {}, *adj_flux[15] = {};
    void *adj_tapes[4][48] = {};  // the tapes of a step's four stages (set 0 is adj_tape)
    void *tape_out[48] = {};      // where run_stage's sweeps write their tape (null: nowhere)
    double *adj_f[kAdjFields][5] = {};
    double *adj_part = nullptr;
    int adj_nsteps = 0, adj_every = 0;
    std::vector<double *> adj_ckpt;  // 5*npts each: the state before step k*adj_every
    std::vector<int> adj_ts, adj_fts;
    double *adj_seg = nullptr;       // adj_every states of the segment being reversed
    // segment mode (where the device has room): the tapes and stage inputs of
    // every step of a segment, written while the segment is replayed, so the
    // steps are not run a second time: [step][stage][48 tape / 5 input fields]
    int adj_segmode = 0, adj_recompute = 0;
    char *adj_segtape = nullptr, *adj_segyin = nullptr;
    int adj_end_ts = 0, adj_end_fts = 0;
    double adj_end_scal[2] = {0, 0};
};

static cudaEvent_t ev_get(cs3d_handle *h) {
    if (!h->ev_pool.empty()) {
        cudaEvent_t e = h->ev_pool.back();
        h->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Drain finished timing events into the per-class totals.
static int ev_drain(cs3d_handle *h) {
    for (auto &pe : h->ev_pending) {
        float ms = 0.f;
        CS3D_CUDA(cudaEventSynchronize(pe.second.second));
        CS3D_CUDA(cudaEventElapsedTime(&ms, pe.second.first, pe.second.second));
        h->k_ms[pe.first] += ms;
        h->k_count[pe.first] += 1;
        h->ev_pool.push_back(pe.second.first);
        h->ev_pool.push_back(pe.second.second);
    }
    h->ev_pending.clear();
    return CS3D_OK;
}

// Bracket one kernel launch of class cls with events (when timing is on).
static void tstart(cs3d_handle *h, int cls) {
    h->launches++;
    if (!h->timing) return;
    h->k_cur = cls;
    h->k_ev0 = ev_get(h);
    cudaEventRecord(h->k_ev0, h->stream);
}
static void tend(cs3d_handle *h) {
    if (!h->timing || h->k_cur < 0) return;
    cudaEvent_t e1 = ev_get(h);
    cudaEventRecord(e1, h->stream);
    h->ev_pending.push_back({h->k_cur, {h->k_ev0, e1}});
    h->k_cur = -1;
    if (h->ev_pending.size() > 4096) ev_drain(h);
}

static int dalloc(cs3d_handle *h, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(CS3D_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    h->allocs.push_back(*p);
    e = cudaMemsetAsync(*p, 0, bytes, h->stream);
    if (e != cudaSuccess) return fail(CS3D_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    return CS3D_OK;
}

static int ilog2(int v) {
    int r = 0;
    while ((1 << (r + 1)) <= v) ++r;
    return r;
}

static int face_band_flags(const cs3d_config *c, int *wall, int *spk) {
    *wall = 0;
    *spk = 0;
    for (int f = 0; f < 6; f++) {
        int k = c->bc_kind[f];
        if (k == CS3D_ADIABATIC_WALL || k == CS3D_MOVING_ADIABATIC_WALL) *wall |= 1 << f;
        if (k == CS3D_SPONGE) *spk |= 1 << f;
    }
    return 0;
}

// Wall velocity (U,V,W) of face f (CSolver_AWS.hpp:104-106).
static void wall_velocity(const cs3d_config *c, int f, double uw[3]) {
    uw[0] = uw[1] = uw[2] = 0.0;
    if (c->bc_kind[f] != CS3D_MOVING_ADIABATIC_WALL) return;
    const double *v = c->wall_vel;
    switch (f) {
    case 0: uw[1] = v[0]; uw[2] = v[1]; break;
    case 1: uw[1] = v[2]; uw[2] = v[3]; break;
    case 2: uw[0] = v[4]; uw[2] = v[5]; break;
    case 3: uw[0] = v[6]; uw[2] = v[7]; break;
    case 4: uw[0] = v[8]; uw[1] = v[9]; break;
    case 5: uw[0] = v[10]; uw[1] = v[11]; break;
    }
}

static int check_config(const cs3d_config *c) {
    if (!c) return fail(CS3D_ERR_ARG, "null config");
    int Nd[3] = {c->Nx, c->Ny, c->Nz};
    double Ld[3] = {c->Lx, c->Ly, c->Lz};
    for (int d = 0; d < 3; d++) {
        if (c->bc_type[d] != CS3D_PERIODIC_SOLVE && c->bc_type[d] != CS3D_DIRICHLET_SOLVE)
            return fail(CS3D_ERR_ARG, "bc_type[%d]=%d is not PERIODIC_SOLVE or DIRICHLET_SOLVE", d, c->bc_type[d]);
        // the filter's wall closure reaches phi[N-7] (Filter.cpp:77-87); the
        // periodic filter stencil spans 9 points
        if (Nd[d] < 8) return fail(CS3D_ERR_SHAPE, "N[%d]=%d: every direction needs at least 8 points", d, Nd[d]);
        if (Nd[d] > 4096) return fail(CS3D_ERR_SHAPE, "N[%d]=%d exceeds 4096 points per line", d, Nd[d]);
    }
    if ((long long)c->Nx * c->Ny * c->Nz >= (1ll << 31))
        return fail(CS3D_ERR_SHAPE, "Nx*Ny*Nz must stay below 2^31 points (32-bit indexing)");
    for (int d = 0; d < 3; d++) {
        if (!(Ld[d] > 0.0)) return fail(CS3D_ERR_ARG, "L[%d] must be positive", d);
    }
    for (int f = 0; f < 6; f++)
        if (c->bc_kind[f] < CS3D_PERIODIC || c->bc_kind[f] > CS3D_INLET)
            return fail(CS3D_ERR_ARG, "bc_kind[%d]=%d out of range", f, c->bc_kind[f]);
    if (c->rk != CS3D_RK4 && c->rk != CS3D_TVDRK3) return fail(CS3D_ERR_ARG, "rk=%d", c->rk);
    if (c->precision != CS3D_FP64 && c->precision != CS3D_FP32_MIXED)
        return fail(CS3D_ERR_ARG, "precision=%d", c->precision);
    if (c->filter_step < 1) return fail(CS3D_ERR_ARG, "filter_step must be >= 1");
    if (!(c->CFL > 0.0) && !(c->dt_fixed > 0.0)) return fail(CS3D_ERR_ARG, "CFL or dt_fixed must be positive");
    if (c->sponge_mode != CS3D_SPONGE_REFERENCE && c->sponge_mode != CS3D_SPONGE_BANDS)
        return fail(CS3D_ERR_ARG, "sponge_mode=%d", c->sponge_mode);
    return CS3D_OK;
}

// Tile width: the widest power of two (<= 32 lines) whose shared memory
// stays within a per-block budget (72 kB: three blocks per SM).  For the
// y and z sweeps of the mixed form at N = 128 this gives 8 lines: every
// global access is then a full 32-byte sector, which measured faster than
// narrower tiles with more blocks per SM.
// sweep: the sweeps' tile layout (pair-interleaved in FP32), else planar.
static int pick_L(size_t tb, int nbuf, int N, int pitch_plus, int budget_kb = 72, bool sweep = false) {
    const size_t budget = (size_t)budget_kb * 1024;
    int L = 32;
    auto bytes = [&](int l) {
        return sweep ? sweep_smem_bytes((int)tb, nbuf, l, l + pitch_plus, N)
                     : planar_smem_bytes((int)tb, nbuf, l, l + pitch_plus, N);
    };
    while (L > 1 && bytes(L) > budget) L /= 2;
    return L;
}

// The sweeps' shared-memory pitch beyond the tile width: one pad column in
// the mixed form's x tiles (their points walk along a line first), none in
// the FP64 x tiles (points across the lines first) nor in y and z.
static int x_pitch_plus(const cs3d_handle *h, int d) { return d == 0 && h->mixed ? 1 : 0; }

// Sponge strength sigma (SpongeBC.hpp:64-150) with sigma starting at zero.
static void build_sigma(const cs3d_config *c, std::vector<double> &sig, int *any) {
    const int Nx = c->Nx, Ny = c->Ny, Nz = c->Nz;
    sig.assign((size_t)Nx * Ny * Nz, 0.0);
    const double L[3] = {c->Lx, c->Ly, c->Lz};
    const double dflt[3] = {0.25, 0.125, 0.25};
    int Nd[3] = {Nx, Ny, Nz};
    *any = 0;
    for (int f = 0; f < 6; f++) {
        int dir = f / 2, hi = f % 2;
        double band = c->sponge_mode == CS3D_SPONGE_REFERENCE
                          ? (c->bc_kind[f] == CS3D_SPONGE ? dflt[dir] * L[dir] : 0.0)
                          : c->sponge_frac[f] * L[dir];
        if (band <= 0.0) continue;
        *any = 1;
        for (int a = 0; a < Nd[dir]; a++) {
            double xc = (((double)a) / ((double)Nd[dir] - 1.0)) * L[dir], s;
            if (!hi) { if (!(xc < band)) continue; s = (band - xc) / band; }
            else { if (!(xc > L[dir] - band)) continue; s = (xc - (L[dir] - band)) / band; }
            double val = 6.0 * (0.068 * std::pow(s, 2.0) + 0.845 * std::pow(s, 8.0));
            for (int k = 0; k < Nz; k++)
                for (int j = 0; j < Ny; j++)
                    for (int i = 0; i < Nx; i++) {
                        int id[3] = {i, j, k};
                        if (id[dir] != a) continue;
                        size_t ii = (size_t)k * Nx * Ny + (size_t)j * Nx + i;
                        sig[ii] = std::fmax(val, sig[ii]);
                    }
        }
    }
}

extern "C" int cs3d_create(const cs3d_config *cfg, cs3d_handle **out) {
    if (!out) return fail(CS3D_ERR_ARG, "null output pointer");
    *out = nullptr;
    int rc = check_config(cfg);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(CS3D_ERR_NODEV, "no CUDA device");
    cs3d_handle *h = new cs3d_handle();
    h->cfg = *cfg;
    CS3D_CUDA(cudaGetDevice(&h->dev));
    CS3D_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->g.Nx = cfg->Nx; h->g.Ny = cfg->Ny; h->g.Nz = cfg->Nz;
    h->g.npts = (long long)cfg->Nx * cfg->Ny * cfg->Nz;
    const size_t n = (size_t)h->g.npts;
    // Domain.hpp:31-45
    h->dx = (1.0 / ((double)cfg->Nx - 1.0)) * cfg->Lx - 0.0;
    h->dy = (1.0 / ((double)cfg->Ny - 1.0)) * cfg->Ly - 0.0;
    h->dz = (1.0 / ((double)cfg->Nz - 1.0)) * cfg->Lz - 0.0;
    h->gas.gamma = 1.4;
    h->gas.gm1 = h->gas.gamma - 1;
    double p_ref = 1.0 / h->gas.gamma;
    h->gas.R = p_ref / 1.0 / 1.0;
    double cp = h->gas.R * h->gas.gamma / (h->gas.gamma - 1.0);
    h->gas.cpPr = cp / 0.7;
    h->gas.mu_ref = cfg->mu_ref;
    h->nstages = cfg->rk == CS3D_TVDRK3 ? 3 : 4;
    h->mixed = cfg->precision == CS3D_FP32_MIXED;
    h->tb = h->mixed ? 4 : 8;
    face_band_flags(cfg, &h->wall_faces, &h->sponge_kind_faces);
    auto fail_free = [&](int code) {
        cs3d_destroy(h);
        return code;
    };
#define ALLOC(ptr, bytes)                                     \
    do {                                                      \
        int r_ = dalloc(h, (void **)&(ptr), (bytes));         \
        if (r_) return fail_free(r_);                         \
    } while (0)
    for (int f = 0; f < 5; f++) {
        ALLOC(h->q1.f[f], n * 8);
        ALLOC(h->qk.f[f], n * 8);
        ALLOC(h->q2.f[f], n * 8);
        ALLOC(h->prim[f], n * h->tb);
        ALLOC(h->R[f], n * h->tb);
        ALLOC(h->ft1[f], n * h->tb);
        ALLOC(h->ft2[f], n * h->tb);
    }
    for (int f = 0; f < 4; f++) {
        ALLOC(h->dx4[f], n * h->tb);
        ALLOC(h->dy4[f], n * h->tb);
    }
    if (h->mixed) {
        h->mixed_rk4 = cfg->rk == CS3D_RK4;
        for (int f = 0; f < 5; f++) {
            ALLOC(h->q1s[f], n * 4);
            ALLOC(h->qks[f], n * 4);
            ALLOC(h->q2s[f], n * 4);
            if (h->mixed_rk4) ALLOC(h->rfluct[f], n * 4);
        }
    }
    ALLOC(h->mu, n * h->tb);
    ALLOC(h->amu, n * h->tb);
    ALLOC(h->scal, 8 * sizeof(double));
    ALLOC(h->flag, 4 * sizeof(int));
    ALLOC(h->red, 1024 * 8 * sizeof(double));
    // sponge
    std::vector<double> sig;
    build_sigma(cfg, sig, &h->sponge);
    if (h->sponge) {
        ALLOC(h->sigma, n * 8);
        for (int f = 0; f < 5; f++) ALLOC(h->savg.f[f], n * 8);
        CS3D_CUDA(cudaMemcpyAsync(h->sigma, sig.data(), n * 8, cudaMemcpyHostToDevice, h->stream));
    }
    if (h->sponge_kind_faces) {
        for (int f = 0; f < 5; f++) ALLOC(h->backup.f[f], n * 8);
    }
    // operators
    const double dd[3] = {h->dx, h->dy, h->dz};
    const int Nd[3] = {cfg->Nx, cfg->Ny, cfg->Nz};
    for (int d = 0; d < 3; d++)
        for (int k = 1; k <= 3; k++) {
            HostOp ho = make_op(k, Nd[d], cfg->bc_type[d], dd[d], cfg->alphaF);
            int r = upload_op<double>(ho, h->op64[d][k - 1], h->stream);
            if (!r) r = upload_op<float>(ho, h->op32[d][k - 1], h->stream);
            if (!r && k == 3) r = upload_op<float>(make_filter_correction(ho), h->op32fc[d], h->stream);
            if (r) return fail_free(r);
        }
    for (int d = 0; d < 3; d++) {
        // Tile shape.  Default: the widest tile within 75 kB for the mixed
        // x sweep (3 blocks of 256 per SM), 72 kB for y and z (2 blocks of
        // 256).  A mixed-form y or z tile
        // narrower than 16 lines there (z rows of 32 bytes or less per field)
        // instead takes one block of 512 threads per SM and the widest tile
        // within 200 kB: measured at 128^3, z 0.79 -> 0.70 ms per step; where
        // the 72 kB tile is already 16 lines wide (N = 42) one block per SM was
        // slower, its phases no longer overlapping another block's.
        const int nb = sweep_nbuf(d, (int)h->tb);
        h->L[d] = pick_L(h->tb, nb, Nd[d], x_pitch_plus(h, d), d == 0 ? (h->mixed ? 75 : 115) : 72, true);
        // FP64 x: at most 4 lines within 115 kB (2 blocks per SM at N = 256,
        // 3 at 128, registers).  Against the former 75 kB tiles with a pad
        // column (1 line at N = 256): HIT 256^3 x 51.7 -> 26.3 ms per step,
        // shear layer 3.25 -> 1.84; 8 lines at 128^3 measured 4% slower.
        if (!h->mixed && d == 0 && h->L[d] > 4) h->L[d] = 4;
        h->threads[d] = h->mixed ? (d == 0 ? sweep_threads<float>(0) : 256) : sweep_threads<double>(d);
        if (h->mixed && d > 0 && h->L[d] < 16) {
            h->L[d] = pick_L(h->tb, nb, Nd[d], 0, 200, true);
            h->threads[d] = sweep_threads<float>(d);
        }
        h->Lf[d] = pick_L(h->tb, h->mixed ? 10 : 5, Nd[d], d == 0 ? 1 : 0);
        // a mixed filter tile narrower than 8 lines within 72 kB (N = 256: 4
        // lines, 16-byte rows) takes the widest within 110 kB instead (2
        // blocks per SM): HIT 256^3 filter 2.27 -> 1.81 ms per step; at
        // N = 128 the 8-line tile stays (16 lines measured slower)
        if (h->mixed && h->Lf[d] < 8) h->Lf[d] = pick_L(h->tb, 10, Nd[d], d == 0 ? 1 : 0, 110);
        if (sweep_smem_bytes((int)h->tb, nb, 1, 2, Nd[d]) > 200 * 1024)
            return fail_free(fail(CS3D_ERR_SHAPE, "N[%d]=%d: a line does not fit in shared memory", d, Nd[d]));
    }

    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    *out = h;
    return CS3D_OK;
#undef ALLOC
}

extern "C" int cs3d_destroy(cs3d_handle *h) {
    if (!h) return CS3D_OK;
    DeviceGuard dg(h->dev);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void *p : h->allocs) cudaFree(p);
    for (int d = 0; d < 3; d++)
        for (int k = 0; k < 3; k++) {
            if (h->op64[d][k].mem) cudaFree(h->op64[d][k].mem);
            if (h->op32[d][k].mem) cudaFree(h->op32[d][k].mem);
        }
    for (int d = 0; d < 3; d++)
        if (h->op32fc[d].mem) cudaFree(h->op32fc[d].mem);
    if (h->dq[0]) for (int f = 0; f < 5; f++) cudaFree(h->dq[f]);
    if (h->diag[0]) for (int f = 0; f < 3; f++) cudaFree(h->diag[f]);
    if (h->prim_out) cudaFree(h->prim_out);
    for (void *p : h->adj_allocs) cudaFree(p);
    for (void *p : h->adj_rec_allocs) cudaFree(p);
    for (auto &pe : h->ev_pending) { cudaEventDestroy(pe.second.first); cudaEventDestroy(pe.second.second); }
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------
static int launch_shadow_of(cs3d_handle *h, const Q5 &q, float *const out[5]) {
    ShadowArgs a{};
    a.g = h->g;
    a.q = q;
    for (int f = 0; f < 5; f++) a.out[f] = out[f];
    a.nf = 5;
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_shadow(a, h->stream));
    tend(h);
    return CS3D_OK;
}

static int launch_cfl_reduce(cs3d_handle *h) {
    CS3D_CUDA(cudaMemsetAsync(h->scal + 2, 0, sizeof(double), h->stream));
    CflArgs a{};
    a.g = h->g;
    a.gas = h->gas;
    a.q = h->q1;
    if (h->mixed)
        for (int f = 0; f < 5; f++) a.qs[f] = h->q1s[f];
    a.idx64 = 1.0 / h->dx; a.idy64 = 1.0 / h->dy; a.idz64 = 1.0 / h->dz;
    a.idx = (float)a.idx64; a.idy = (float)a.idy64; a.idz = (float)a.idz64;
    a.max_out = h->scal + 2;
    a.nan_flag = h->flag;
    tstart(h, CS3D_K_CFL);
    CS3D_CUDA(launch_cfl(a, h->stream));
    tend(h);
    return CS3D_OK;
}

static int init_after_state(cs3d_handle *h);

extern "C" int cs3d_set_initial_conditions(cs3d_handle *h, const double *rho0, const double *p0, const double *U0,
                                           const double *V0, const double *W0) {
    if (!h || !rho0 || !p0 || !U0 || !V0 || !W0) return fail(CS3D_ERR_ARG, "null argument");
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)h->g.npts;
    double *tmp = nullptr;
    CS3D_CUDA(cudaMalloc(&tmp, n * 8 * 6));
    double *d_rho = tmp, *d_p = tmp + n, *d_U = tmp + 2 * n, *d_V = tmp + 3 * n, *d_W = tmp + 4 * n, *d_T = tmp + 5 * n;
    CS3D_CUDA(cudaMemcpyAsync(d_rho, rho0, n * 8, cudaMemcpyHostToDevice, h->stream));
    CS3D_CUDA(cudaMemcpyAsync(d_p, p0, n * 8, cudaMemcpyHostToDevice, h->stream));
    CS3D_CUDA(cudaMemcpyAsync(d_U, U0, n * 8, cudaMemcpyHostToDevice, h->stream));
    CS3D_CUDA(cudaMemcpyAsync(d_V, V0, n * 8, cudaMemcpyHostToDevice, h->stream));
    CS3D_CUDA(cudaMemcpyAsync(d_W, W0, n * 8, cudaMemcpyHostToDevice, h->stream));
    IcArgs a{};
    a.g = h->g;
    a.gas = h->gas;
    a.rho0 = d_rho; a.p0 = d_p; a.U0 = d_U; a.V0 = d_V; a.W0 = d_W; a.T0 = d_T;
    a.q1 = h->q1;
    CS3D_CUDA(launch_ic(a, h->stream));
    h->launches++;
    if (h->wall_faces) {
        for (int pass = 0; pass < 2; pass++) {
            int kind = pass == 0 ? CS3D_ADIABATIC_WALL : CS3D_MOVING_ADIABATIC_WALL;
            for (int f = 0; f < 6; f++) {
                if (h->cfg.bc_kind[f] != kind) continue;
                a.face = f;
                wall_velocity(&h->cfg, f, a.uw);
                CS3D_CUDA(launch_ic_wall(a, h->stream));
                h->launches++;
            }
        }
        CS3D_CUDA(launch_ic_wall_eos(a, h->stream));
        h->launches++;
    }
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    CS3D_CUDA(cudaFree(tmp));
    return init_after_state(h);
}

// Everything that follows a new state q1: sponge averages (SpongeBC starts
// them at the state), the mixed filter's reference values (the state's field
// means), the FP32 shadow, counters, dt/time, the NaN flag and the CFL
// maximum for the first step.
static int init_after_state(cs3d_handle *h) {
    const size_t n = (size_t)h->g.npts;
    if (h->sponge)
        for (int f = 0; f < 5; f++)
            CS3D_CUDA(cudaMemcpyAsync(h->savg.f[f], h->q1.f[f], n * 8, cudaMemcpyDeviceToDevice, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    if (h->mixed) {
        std::vector<double> hb(n);
        for (int f = 0; f < 5; f++) {
            CS3D_CUDA(cudaMemcpy(hb.data(), h->q1.f[f], n * 8, cudaMemcpyDeviceToHost));
            long double s = 0;
            for (size_t i = 0; i < n; i++) s += hb[i];
            h->fref[f] = (double)(s / (long double)n);
        }
    }
    if (h->mixed) {
        int r = launch_shadow_of(h, h->q1, h->q1s);
        if (r) return r;
    }
    h->timeStep = 0;
    h->filterTimeStep = 0;
    h->backup_valid = 0;
    CS3D_CUDA(cudaMemsetAsync(h->scal, 0, 8 * sizeof(double), h->stream));
    CS3D_CUDA(cudaMemsetAsync(h->flag, 0, 4 * sizeof(int), h->stream));
    int rc = launch_cfl_reduce(h);
    if (rc) return rc;
    h->ic_done = 1;
    return CS3D_OK;
}

extern "C" int cs3d_pre_step(cs3d_handle *h) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    DeviceGuard dg(h->dev);
    DtArgs a{};
    a.max_in = h->scal + 2;
    a.dt = h->scal + 0;
    a.time = h->scal + 1;
    a.CFL = h->cfg.CFL;
    a.dt_fixed = h->cfg.dt_fixed;
    a.first = h->timeStep == 0;
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_finalize_dt(a, h->stream));
    tend(h);
    h->timeStep++;
    return CS3D_OK;
}

template <typename T>
static int run_stage(cs3d_handle *h, int st, int last) {
    // stage input q*: q1 on stage 1, qk afterwards (RK4.hpp:133-137); in the
    // mixed RK4 form qk exists only as its FP32 shadow
    const bool qk_shadow_only = h->mixed_rk4 && st > 1;
    const Q5 qin = st == 1 ? h->q1 : (qk_shadow_only ? Q5{} : h->qk);
    float *const *qin32 = st == 1 ? h->q1s : h->qks;
    const int use_backup = st == 1 && h->backup_valid;
    const bool filtered = h->timeStep % h->cfg.filter_step == 0;
    // walls before the derivatives
    if (h->wall_faces) {
        BCArgs b{};
        b.g = h->g;
        b.gas = h->gas;
        b.q = qin;
        for (int f = 0; f < 5; f++) {
            b.qs[f] = h->mixed ? qin32[f] : nullptr;
            b.qs_out[f] = h->mixed ? qin32[f] : nullptr;
        }
        b.backup = h->backup;
        b.use_backup = use_backup;
        b.wall_faces = h->wall_faces;
        b.sponge_faces = h->sponge_kind_faces;
        for (int pass = 0; pass < 2; pass++) {
            int kind = pass == 0 ? CS3D_ADIABATIC_WALL : CS3D_MOVING_ADIABATIC_WALL;
            for (int f = 0; f < 6; f++) {
                if (h->cfg.bc_kind[f] != kind) continue;
                b.face = f;
                wall_velocity(&h->cfg, f, b.uw);
                tstart(h, CS3D_K_BOUNDARY);
                CS3D_CUDA(launch_wall_pre(b, h->stream));
                tend(h);
            }
        }
    }
    SweepArgs<T> a{};
    a.g = h->g;
    a.gas = h->gas;
    a.q = qin;
    for (int f = 0; f < 5; f++) a.qs[f] = h->mixed ? (const T *)qin32[f] : (const T *)qin.f[f];
    a.backup = h->backup;
    a.use_backup = use_backup;
    a.wall_faces = h->wall_faces;
    a.sponge_kind_faces = h->sponge_kind_faces;
    for (int f = 0; f < 5; f++) {
        a.prim[f] = (T *)h->prim[f];
        a.R[f] = (T *)h->R[f];
        a.dq_out[f] = h->store_dq ? h->dq[f] : nullptr;
        a.q1s[f] = h->q1s[f];
    }
    a.mu = (T *)h->mu;
    a.amu = (T *)h->amu;
    for (int f = 0; f < 4; f++) {
        a.dx[f] = (T *)h->dx4[f];
        a.dy[f] = (T *)h->dy4[f];
    }
    for (int f = 0; f < 3; f++) a.diag[f] = h->store_diag ? (T *)h->diag[f] : nullptr;
    a.dt = h->scal;
    a.rk = h->cfg.rk == CS3D_TVDRK3 ? 1 : 0;
    a.rk_step = st;
    a.q1 = h->q1;
    a.q2 = h->q2;
    a.qk = h->qk;
    a.mixed_rk4 = h->mixed_rk4;
    for (int f = 0; f < 5; f++) {
        a.fluct[f] = h->rfluct[f];
        a.fref[f] = h->fref[f];
    }
    a.fluct_out = h->mixed_rk4 && last && filtered;
    // FP32 shadow written by the z sweep: the next stage's input, or -- after
    // the last stage of a step that is not filtered -- q2, which becomes q1
    a.shadow_target = SHADOW_NONE;
    if (h->mixed) {
        if (!last) a.shadow_target = SHADOW_QK;
        else if (!filtered) a.shadow_target = SHADOW_Q2;
        for (int f = 0; f < 5; f++) a.shadow_out[f] = last ? h->q2s[f] : h->qks[f];
    }
    a.sponge = h->sponge;
    a.sigma = h->sigma;
    a.savg = h->savg;
    for (int i = 0; i < 48; i++) a.tape[i] = (T *)h->tape_out[i];
    for (int d = 0; d < 3; d++) {
        a.threads = h->threads[d];
        a.L = h->L[d];
        a.lgL = ilog2(a.L);
        a.divN = make_fastdiv((unsigned)(d == 0 ? h->g.Nx : d == 1 ? h->g.Ny : h->g.Nz));
        a.P = a.L + x_pitch_plus(h, d);
        if (sizeof(T) == 8) {
            a.d1 = *reinterpret_cast<const LineOp<T> *>(&h->op64[d][0].op);
            a.d2 = *reinterpret_cast<const LineOp<T> *>(&h->op64[d][1].op);
        } else {
            a.d1 = *reinterpret_cast<const LineOp<T> *>(&h->op32[d][0].op);
            a.d2 = *reinterpret_cast<const LineOp<T> *>(&h->op32[d][1].op);
        }
        tstart(h, CS3D_K_SWEEP_X + d);
        CS3D_CUDA(launch_sweep<T>(d, a, h->stream));
        tend(h);
    }
    if (last) {
        if (filtered) {
            // filterConservedData round robin (CSolver_AWS.cpp:1690-1863)
            h->filterTimeStep++;
            int order[3];
            int m3 = h->filterTimeStep % 3;
            if (m3 == 1) { order[0] = 0; order[1] = 1; order[2] = 2; }
            else if (m3 == 2) { order[0] = 1; order[1] = 2; order[2] = 0; }
            else { order[0] = 2; order[1] = 0; order[2] = 1; }
            for (int pass = 0; pass < 3; pass++) {
                int d = order[pass];
                FilterArgs<T> fa{};
                fa.g = h->g;
                fa.L = h->Lf[d];
                fa.lgL = ilog2(h->Lf[d]);
                fa.divN = make_fastdiv((unsigned)(d == 0 ? h->g.Nx : d == 1 ? h->g.Ny : h->g.Nz));
                fa.P = h->Lf[d] + (d == 0 ? 1 : 0);
                fa.threads = sizeof(T) == 4 ? filter_threads<float>() : filter_threads<double>();
                if (sizeof(T) == 8) fa.op = *reinterpret_cast<const LineOp<T> *>(&h->op64[d][2].op);
                else fa.op = *reinterpret_cast<const LineOp<T> *>(&h->op32fc[d].op);
                void **src = pass == 1 ? h->ft1 : h->ft2;
                void **dst = pass == 0 ? h->ft1 : h->ft2;
                for (int f = 0; f < 5; f++) {
                    fa.ref[f] = h->mixed ? h->fref[f] : 0.0;
                    // first pass: q2 - fref, in FP32 from the last stage (mixed
                    // RK4) or formed here from FP64 q2
                    const bool fl = pass == 0 && h->mixed_rk4;
                    fa.src64.f[f] = pass == 0 && !fl ? h->q2.f[f] : nullptr;
                    fa.src32[f] = fl ? (T *)h->rfluct[f] : pass == 0 ? nullptr : (T *)src[f];
                    fa.dst64.f[f] = pass == 2 ? h->q1.f[f] : nullptr;
                    fa.dst32[f] = pass == 2 ? nullptr : (T *)dst[f];
                    fa.delta_from.f[f] = (pass == 2 && h->mixed) ? h->q2.f[f] : nullptr;
                    fa.unf[f] = (pass == 2 && h->mixed_rk4) ? h->rfluct[f] : nullptr;
                    fa.shadow_out[f] = (pass == 2 && h->mixed) ? h->q1s[f] : nullptr;
                }
                tstart(h, CS3D_K_FILTER);
                CS3D_CUDA(launch_filter<T>(d, fa, h->stream));
                tend(h);
            }
        } else {
            // not a filter step: q1 takes q2's values (:1866-1880) by exchange
            std::swap(h->q1, h->q2);
            for (int f = 0; f < 5; f++) std::swap(h->q1s[f], h->q2s[f]);
        }
        int rc = launch_cfl_reduce(h);
        if (rc) return rc;
    }
    return CS3D_OK;
}

extern "C" int cs3d_sub_step(cs3d_handle *h, int rk_step, int rk_last) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    if (h->timeStep < 1) return fail(CS3D_ERR_STATE, "cs3d_pre_step must precede the first sub-step");
    if (rk_step < 1 || rk_step > h->nstages) return fail(CS3D_ERR_ARG, "rk_step=%d", rk_step);
    DeviceGuard dg(h->dev);
    return h->mixed ? run_stage<float>(h, rk_step, rk_last) : run_stage<double>(h, rk_step, rk_last);
}

extern "C" int cs3d_post_step(cs3d_handle *h) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    if (!h->sponge) return CS3D_OK;
    DeviceGuard dg(h->dev);
    SpongeArgs a{};
    a.g = h->g;
    a.dt = h->scal;
    a.avgT = 15.0;         // SpongeBC.hpp:56-58
    a.epsP = 0.005;
    a.spongeP = 1.0 / h->gas.gamma;
    a.gm1 = h->gas.gamma - 1.0;
    a.q1 = h->q1;
    a.savg = h->savg;
    a.backup = h->backup;
    for (int f = 0; f < 5; f++) a.q1s[f] = h->mixed ? h->q1s[f] : nullptr;
    a.sponge_kind_faces = h->sponge_kind_faces;
    tstart(h, CS3D_K_SPONGE);
    CS3D_CUDA(launch_sponge_update(a, h->stream));
    tend(h);
    if (h->sponge_kind_faces) h->backup_valid = 1;
    return CS3D_OK;
}

extern "C" int cs3d_step(cs3d_handle *h) {
    int rc = cs3d_pre_step(h);
    if (rc) return rc;
    for (int s = 1; s <= h->nstages; s++) {
        rc = cs3d_sub_step(h, s, s == h->nstages);
        if (rc) return rc;
    }
    return cs3d_post_step(h);
}

extern "C" int cs3d_run(cs3d_handle *h, int n) {
    for (int i = 0; i < n; i++) {
        int rc = cs3d_step(h);
        if (rc) return rc;
    }
    return CS3D_OK;
}

extern "C" int cs3d_sync(cs3d_handle *h) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    DeviceGuard dg(h->dev);
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    CflArgs a{};
    a.g = h->g;
    a.q = h->q1;
    a.nan_flag = h->flag;
    CS3D_CUDA(launch_nan_scan(a, h->stream));
    h->launches++;
    int flag = 0;
    CS3D_CUDA(cudaMemcpyAsync(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    if (flag) {
        CS3D_CUDA(cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream));
        return fail(CS3D_ERR_NAN, "a non-finite value reached the conserved state");
    }
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// field access
// ---------------------------------------------------------------------
static int field_ptr(cs3d_handle *h, int field, double **p) {
    *p = nullptr;
    if (field >= CS3D_F_RHO1 && field < CS3D_F_RHO1 + 5) *p = h->q1.f[field - CS3D_F_RHO1];
    else if (field >= CS3D_F_RHOK && field < CS3D_F_RHOK + 5) {
        *p = h->qk.f[field - CS3D_F_RHOK];
        if (h->mixed_rk4) {
            // the mixed RK4 form keeps the stage input qk as an FP32 shadow only
            ShadowArgs a{};
            a.g = h->g;
            a.q.f[0] = *p;
            a.in[0] = h->qks[field - CS3D_F_RHOK];
            a.nf = 1;
            CS3D_CUDA(launch_shadow(a, h->stream));
            h->launches++;
        }
    }
    else if (field >= CS3D_F_RHO2 && field < CS3D_F_RHO2 + 5) *p = h->q2.f[field - CS3D_F_RHO2];
    else if (field >= CS3D_F_RHOK2 && field < CS3D_F_RHOK2 + 5) {
        if (!h->store_dq) return fail(CS3D_ERR_STATE, "increments are kept only with CS3D_OPT_STORE_INCREMENTS");
        *p = h->dq[field - CS3D_F_RHOK2];
    } else if (field >= CS3D_F_U && field < CS3D_F_U + 7) {
        if (!h->prim_out) CS3D_CUDA(cudaMalloc(&h->prim_out, (size_t)h->g.npts * 8 * 7));
        PrimArgs a{};
        a.g = h->g;
        a.gas = h->gas;
        a.q = h->q1;
        for (int f = 0; f < 7; f++) a.out[f] = h->prim_out + (size_t)f * h->g.npts;
        CS3D_CUDA(launch_primitives(a, h->stream));
        h->launches++;
        *p = h->prim_out + (size_t)(field - CS3D_F_U) * h->g.npts;
    } else if (field >= CS3D_F_SPONGE_AVG && field < CS3D_F_SPONGE_AVG + 5) {
        if (!h->sponge) return fail(CS3D_ERR_STATE, "no sponge in this configuration");
        *p = h->savg.f[field - CS3D_F_SPONGE_AVG];
    } else if (field == CS3D_F_SIGMA) {
        if (!h->sponge) return fail(CS3D_ERR_STATE, "no sponge in this configuration");
        *p = h->sigma;
    } else {
        return fail(CS3D_ERR_ARG, "field index %d out of range", field);
    }
    return CS3D_OK;
}

extern "C" int cs3d_get_field(cs3d_handle *h, int field, double *host_out) {
    if (!h || !host_out) return fail(CS3D_ERR_ARG, "null argument");
    DeviceGuard dg(h->dev);
    double *p;
    int rc = field_ptr(h, field, &p);
    if (rc) return rc;
    CS3D_CUDA(cudaMemcpyAsync(host_out, p, (size_t)h->g.npts * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

extern "C" int cs3d_set_field(cs3d_handle *h, int field, const double *host_in) {
    if (!h || !host_in) return fail(CS3D_ERR_ARG, "null argument");
    if (field >= CS3D_F_U && field < CS3D_F_U + 7)
        return fail(CS3D_ERR_ARG, "primitive fields are derived from the conserved state and cannot be set");
    DeviceGuard dg(h->dev);
    double *p;
    int rc = field_ptr(h, field, &p);
    if (rc) return rc;
    CS3D_CUDA(cudaMemcpyAsync(p, host_in, (size_t)h->g.npts * 8, cudaMemcpyHostToDevice, h->stream));
    if (h->mixed && field < CS3D_F_RHOK2) {
        // keep the FP32 shadow of the written state in step
        const int grp = field / 5, f = field % 5;
        float *out = (grp == 0 ? h->q1s : grp == 1 ? h->qks : h->q2s)[f];
        ShadowArgs a{};
        a.g = h->g;
        a.q.f[0] = p;
        a.out[0] = out;
        a.nf = 1;
        CS3D_CUDA(launch_shadow(a, h->stream));
        h->launches++;
    }
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

extern "C" int cs3d_get_conserved(cs3d_handle *h, double *const host_out[5]) {
    if (!h || !host_out) return fail(CS3D_ERR_ARG, "null argument");
    for (int f = 0; f < 5; f++)
        if (!host_out[f]) return fail(CS3D_ERR_ARG, "null field %d", f);
    DeviceGuard dg(h->dev);
    const size_t bytes = (size_t)h->g.npts * 8;
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(host_out[f], h->q1.f[f], bytes, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

extern "C" int cs3d_set_conserved(cs3d_handle *h, const double *const host_in[5]) {
    if (!h || !host_in) return fail(CS3D_ERR_ARG, "null argument");
    for (int f = 0; f < 5; f++)
        if (!host_in[f]) return fail(CS3D_ERR_ARG, "null field %d", f);
    DeviceGuard dg(h->dev);
    const size_t bytes = (size_t)h->g.npts * 8;
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(h->q1.f[f], host_in[f], bytes, cudaMemcpyHostToDevice, h->stream));
    if (h->mixed) {
        // the FP32 shadow of q1, all five fields in one launch
        ShadowArgs a{};
        a.g = h->g;
        for (int f = 0; f < 5; f++) {
            a.q.f[f] = h->q1.f[f];
            a.out[f] = h->q1s[f];
        }
        a.nf = 5;
        CS3D_CUDA(launch_shadow(a, h->stream));
        h->launches++;
    }
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

extern "C" int cs3d_field_ptr(cs3d_handle *h, int field, double **dev_ptr) {
    if (!h || !dev_ptr) return fail(CS3D_ERR_ARG, "null argument");
    DeviceGuard dg(h->dev);
    return field_ptr(h, field, dev_ptr);
}

extern "C" int cs3d_get_scalars(cs3d_handle *h, double *dt, double *time, int *time_step) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    DeviceGuard dg(h->dev);
    double s[2];
    CS3D_CUDA(cudaMemcpyAsync(s, h->scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    if (dt) *dt = s[0];
    if (time) *time = s[1];
    if (time_step) *time_step = h->timeStep;
    return CS3D_OK;
}

extern "C" int cs3d_get_stream(cs3d_handle *h, void **stream) {
    if (!h || !stream) return fail(CS3D_ERR_ARG, "null argument");
    *stream = (void *)h->stream;
    return CS3D_OK;
}

extern "C" int cs3d_launch_count(cs3d_handle *h, long long *count) {
    if (!h || !count) return fail(CS3D_ERR_ARG, "null argument");
    *count = h->launches;
    return CS3D_OK;
}

extern "C" int cs3d_set_option(cs3d_handle *h, int option, int value) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)h->g.npts;
    if (option == CS3D_OPT_STORE_INCREMENTS) {
        if (value && !h->dq[0])
            for (int f = 0; f < 5; f++) {
                CS3D_CUDA(cudaMalloc(&h->dq[f], n * 8));
                CS3D_CUDA(cudaMemsetAsync(h->dq[f], 0, n * 8, h->stream));
            }
        h->store_dq = value != 0;
    } else if (option == CS3D_OPT_STORE_DIAGNOSTICS) {
        if (value && !h->diag[0])
            for (int f = 0; f < 3; f++) {
                CS3D_CUDA(cudaMalloc(&h->diag[f], n * h->tb));
                CS3D_CUDA(cudaMemsetAsync(h->diag[f], 0, n * h->tb, h->stream));
            }
        h->store_diag = value != 0;
    } else if (option == CS3D_OPT_KERNEL_TIMING) {
        h->timing = value != 0;
    } else if (option == CS3D_OPT_ADJ_RECOMPUTE) {
        h->adj_recompute = value != 0;
    } else {
        return fail(CS3D_ERR_ARG, "unknown option %d", option);
    }
    return CS3D_OK;
}

extern "C" int cs3d_kernel_times(cs3d_handle *h, double *ms, long long *count, int n, int reset) {
    if (!h || (!ms && !count)) return fail(CS3D_ERR_ARG, "null argument");
    DeviceGuard dg(h->dev);
    int rc = ev_drain(h);
    if (rc) return rc;
    for (int i = 0; i < n && i < CS3D_NUM_KERNEL_CLASSES; i++) {
        if (ms) ms[i] = h->k_ms[i];
        if (count) count[i] = h->k_count[i];
    }
    if (reset)
        for (int i = 0; i < CS3D_NUM_KERNEL_CLASSES; i++) { h->k_ms[i] = 0; h->k_count[i] = 0; }
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// single operators
// ---------------------------------------------------------------------
static int line_op(cs3d_handle *h, int kind, int dir, const double *in, double *out) {
    if (!h || !in || !out) return fail(CS3D_ERR_ARG, "null argument");
    if (dir < 0 || dir > 2) return fail(CS3D_ERR_ARG, "dir=%d", dir);
    if (in == out) return fail(CS3D_ERR_ARG, "in and out must not overlap");
    DeviceGuard dg(h->dev);
    LineOpArgs a{};
    a.op = h->op64[dir][kind - 1].op;
    const int N = a.op.N;
    a.nlines = h->g.npts / N;
    a.L = 32;
    while (a.L > 1 && planar_smem_bytes(8, 1, a.L, a.L + 1, N) > 72 * 1024) a.L /= 2;
    a.P = a.L + 1;
    a.threads = 128;
    a.in = in;
    a.out = out;
    CS3D_CUDA(launch_line_op(a, h->stream));
    h->launches++;
    return CS3D_OK;
}

extern "C" int cs3d_deriv1(cs3d_handle *h, int dir, const double *in_dev, double *out_dev) {
    return line_op(h, 1, dir, in_dev, out_dev);
}
extern "C" int cs3d_deriv2(cs3d_handle *h, int dir, const double *in_dev, double *out_dev) {
    return line_op(h, 2, dir, in_dev, out_dev);
}
extern "C" int cs3d_filter(cs3d_handle *h, int dir, const double *in_dev, double *out_dev) {
    return line_op(h, 3, dir, in_dev, out_dev);
}

// ---------------------------------------------------------------------
// operator-only handles: one direction's three compact operators
// ---------------------------------------------------------------------
struct cs3d_op {
    int dev = 0;
    cudaStream_t stream = nullptr;
    long long npts = 0;
    DevOp<double> ops[3];
    double *stage = nullptr;  // 2 * npts doubles for the host-array calls (allocated on first use)
};

extern "C" int cs3d_op_create(const cs3d_config *cfg, int dir, cs3d_op **out) {
    if (!out) return fail(CS3D_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!cfg) return fail(CS3D_ERR_ARG, "null config");
    if (dir < 0 || dir > 2) return fail(CS3D_ERR_ARG, "dir=%d", dir);
    const int Nd[3] = {cfg->Nx, cfg->Ny, cfg->Nz};
    const double Ld[3] = {cfg->Lx, cfg->Ly, cfg->Lz};
    for (int d = 0; d < 3; d++)
        if (Nd[d] < 1) return fail(CS3D_ERR_SHAPE, "N[%d]=%d", d, Nd[d]);
    if (Nd[dir] < 8) return fail(CS3D_ERR_SHAPE, "N[%d]=%d: a line needs at least 8 points", dir, Nd[dir]);
    if (Nd[dir] > 4096) return fail(CS3D_ERR_SHAPE, "N[%d]=%d exceeds 4096 points per line", dir, Nd[dir]);
    if ((long long)Nd[0] * Nd[1] * Nd[2] >= (1ll << 31))
        return fail(CS3D_ERR_SHAPE, "Nx*Ny*Nz must stay below 2^31 points (32-bit indexing)");
    if (!(Ld[dir] > 0.0)) return fail(CS3D_ERR_ARG, "L[%d] must be positive", dir);
    const int bc = cfg->bc_type[dir];
    if (bc != CS3D_PERIODIC_SOLVE && bc != CS3D_DIRICHLET_SOLVE)
        return fail(CS3D_ERR_ARG, "bc_type[%d]=%d is not PERIODIC_SOLVE or DIRICHLET_SOLVE", dir, bc);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(CS3D_ERR_NODEV, "no CUDA device");
    cs3d_op *o = new cs3d_op();
    o->npts = (long long)Nd[0] * Nd[1] * Nd[2];
    auto fail_free = [&](int code) {
        cs3d_op_destroy(o);
        return code;
    };
    if (cudaGetDevice(&o->dev) != cudaSuccess ||
        cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail_free(fail(CS3D_ERR_CUDA, "stream creation failed"));
    // Domain.hpp:31-45: dx = x[1] - x[0]
    const double dh = (1.0 / ((double)Nd[dir] - 1.0)) * Ld[dir] - 0.0;
    for (int k = 1; k <= 3; k++) {
        int r = upload_op<double>(make_op(k, Nd[dir], bc, dh, cfg->alphaF), o->ops[k - 1], o->stream);
        if (r) return fail_free(r);
    }
    if (cudaStreamSynchronize(o->stream) != cudaSuccess)
        return fail_free(fail(CS3D_ERR_CUDA, "operator upload failed"));
    *out = o;
    return CS3D_OK;
}

extern "C" int cs3d_op_destroy(cs3d_op *o) {
    if (!o) return CS3D_OK;
    DeviceGuard dg(o->dev);
    if (o->stream) cudaStreamSynchronize(o->stream);
    for (auto &d : o->ops)
        if (d.mem) cudaFree(d.mem);
    if (o->stage) cudaFree(o->stage);
    if (o->stream) cudaStreamDestroy(o->stream);
    delete o;
    return CS3D_OK;
}

static int op_launch(cs3d_op *o, int kind, const double *in, double *out) {
    LineOpArgs a{};
    a.op = o->ops[kind - 1].op;
    const int N = a.op.N;
    a.nlines = o->npts / N;
    a.L = 32;
    while (a.L > 1 && planar_smem_bytes(8, 1, a.L, a.L + 1, N) > 72 * 1024) a.L /= 2;
    a.P = a.L + 1;
    a.threads = 128;
    a.in = in;
    a.out = out;
    CS3D_CUDA(launch_line_op(a, o->stream));
    return CS3D_OK;
}

extern "C" int cs3d_op_apply(cs3d_op *o, int kind, const double *in_dev, double *out_dev) {
    if (!o || !in_dev || !out_dev) return fail(CS3D_ERR_ARG, "null argument");
    if (kind < CS3D_OP_DERIV1 || kind > CS3D_OP_FILTER) return fail(CS3D_ERR_ARG, "kind=%d", kind);
    if (in_dev == out_dev) return fail(CS3D_ERR_ARG, "in and out must not overlap");
    DeviceGuard dg(o->dev);
    return op_launch(o, kind, in_dev, out_dev);
}

extern "C" int cs3d_op_apply_host(cs3d_op *o, int kind, const double *in_host, double *out_host) {
    if (!o || !in_host || !out_host) return fail(CS3D_ERR_ARG, "null argument");
    if (kind < CS3D_OP_DERIV1 || kind > CS3D_OP_FILTER) return fail(CS3D_ERR_ARG, "kind=%d", kind);
    DeviceGuard dg(o->dev);
    const size_t bytes = (size_t)o->npts * 8;
    if (!o->stage) {
        cudaError_t e = cudaMalloc(&o->stage, 2 * bytes);
        if (e != cudaSuccess) {
            o->stage = nullptr;
            return fail(CS3D_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", 2 * bytes, cudaGetErrorString(e));
        }
    }
    CS3D_CUDA(cudaMemcpyAsync(o->stage, in_host, bytes, cudaMemcpyHostToDevice, o->stream));
    int rc = op_launch(o, kind, o->stage, o->stage + o->npts);
    if (rc) return rc;
    CS3D_CUDA(cudaMemcpyAsync(out_host, o->stage + o->npts, bytes, cudaMemcpyDeviceToHost, o->stream));
    CS3D_CUDA(cudaStreamSynchronize(o->stream));
    return CS3D_OK;
}

extern "C" int cs3d_op_get_stream(cs3d_op *o, void **stream) {
    if (!o || !stream) return fail(CS3D_ERR_ARG, "null argument");
    *stream = (void *)o->stream;
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// Taylor-Green diagnostics
// ---------------------------------------------------------------------
template <typename T>
static int tgv_launch(cs3d_handle *h, int blocks) {
    TgvArgs<T> a{};
    a.g = h->g;
    a.gas = h->gas;
    a.q = h->q1;
    for (int f = 0; f < 3; f++) {
        a.dx[f] = (const T *)h->dx4[f];
        a.dy[f] = (const T *)h->dy4[f];
        a.dz[f] = (const T *)h->diag[f];
    }
    a.out = h->red;
    CS3D_CUDA(launch_tgv<T>(a, blocks, h->stream));
    h->launches++;
    return CS3D_OK;
}

extern "C" int cs3d_tgv_quantities(cs3d_handle *h, double out[7]) {
    if (!h || !out) return fail(CS3D_ERR_ARG, "null argument");
    if (!h->store_diag || h->timeStep < 1)
        return fail(CS3D_ERR_STATE, "run a step with CS3D_OPT_STORE_DIAGNOSTICS on first");
    DeviceGuard dg(h->dev);
    const int blocks = 1024;
    int rc = h->mixed ? tgv_launch<float>(h, blocks) : tgv_launch<double>(h, blocks);
    if (rc) return rc;
    std::vector<double> part((size_t)blocks * 6);
    double t[2];
    CS3D_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaMemcpyAsync(t, h->scal, 2 * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int b = 0; b < blocks; b++)
        for (int i = 0; i < 6; i++) s[i] += part[(size_t)b * 6 + i];
    out[0] = t[1];
    out[1] = s[3];
    out[2] = s[2];
    out[3] = s[0];
    out[4] = s[1];
    out[5] = s[5];
    out[6] = std::sqrt(s[4]);
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// calcTurbulenceQuantities and shearLayerInfoCalc
// ---------------------------------------------------------------------
template <typename T>
static DiagArgs<T> diag_args(cs3d_handle *h) {
    DiagArgs<T> a{};
    a.g = h->g;
    a.gas = h->gas;
    a.q = h->q1;
    for (int f = 0; f < 3; f++) {
        a.dx[f] = (const T *)h->dx4[f];
        a.dy[f] = (const T *)h->dy4[f];
        a.dz[f] = (const T *)h->diag[f];
    }
    a.out = h->red;
    return a;
}

template <typename T>
static int turb_sums(cs3d_handle *h, int blocks, int pass, double meanRho, double *sums) {
    DiagArgs<T> a = diag_args<T>(h);
    a.meanRho = meanRho;
    CS3D_CUDA(launch_turb<T>(a, blocks, pass, h->stream));
    h->launches++;
    std::vector<double> part((size_t)blocks * kTurbSums);
    CS3D_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < kTurbSums; i++) sums[i] = 0.0;
    for (int b = 0; b < blocks; b++)
        for (int i = 0; i < kTurbSums; i++) sums[i] += part[(size_t)b * kTurbSums + i];
    return CS3D_OK;
}

extern "C" int cs3d_turbulence_quantities(cs3d_handle *h, double out[11]) {
    if (!h || !out) return fail(CS3D_ERR_ARG, "null argument");
    if (!h->store_diag || h->timeStep < 1)
        return fail(CS3D_ERR_STATE, "run a step with CS3D_OPT_STORE_DIAGNOSTICS on first");
    DeviceGuard dg(h->dev);
    const int blocks = 512;  // 512 x 11 partial sums fit the reduction scratch
    double s[kTurbSums], r2[kTurbSums], t[2];
    int rc = h->mixed ? turb_sums<float>(h, blocks, 0, 0.0, s) : turb_sums<double>(h, blocks, 0, 0.0, s);
    if (rc) return rc;
    const double meanRho = s[0];
    rc = h->mixed ? turb_sums<float>(h, blocks, 1, meanRho, r2) : turb_sums<double>(h, blocks, 1, meanRho, r2);
    if (rc) return rc;
    CS3D_CUDA(cudaMemcpyAsync(t, h->scal, 2 * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    // the derived quantities of CSolver_AWS.cpp:2119-2147, in its order
    const double rhoprime = std::sqrt(r2[0]), dilprime = std::sqrt(s[9]), vortprime = std::sqrt(s[10]);
    const double meanNu = s[1] / meanRho;
    const double meanTurbDiss = s[2] / meanRho;
    const double uprime = std::sqrt(s[3]), uiprime = std::sqrt(s[4]), urms = std::sqrt(s[5]);
    const double turbMach = urms / s[6];
    const double taylorMicro2 = uprime / uiprime;
    const double taylorReyn3 = uprime * taylorMicro2 / meanNu;
    const double pi = 3.14159265358979323846;
    const double tau = std::sqrt(2.0 * pi) / 8.0 / uprime;
    const double kolNu = std::pow(std::pow(meanNu, 3.0) / meanTurbDiss, 0.25);
    const double row[11] = {t[1], tau, taylorReyn3, turbMach, meanTurbDiss, uprime, kolNu,
                            rhoprime, dilprime, vortprime, s[8]};
    for (int i = 0; i < 11; i++) out[i] = row[i];
    return CS3D_OK;
}

extern "C" int cs3d_shear_layer_info(cs3d_handle *h, double *out) {
    if (!h || !out) return fail(CS3D_ERR_ARG, "null argument");
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    DeviceGuard dg(h->dev);
    const size_t n = 17 * (size_t)h->g.Ny;
    if (!h->shear_buf) {
        int rc = dalloc(h, (void **)&h->shear_buf, n * 8);
        if (rc) return rc;
    }
    DiagArgs<double> a{};
    a.g = h->g;
    a.gas = h->gas;
    a.q = h->q1;
    a.out = h->shear_buf;
    CS3D_CUDA(launch_shear_info(a, h->stream));
    h->launches++;
    CS3D_CUDA(cudaMemcpyAsync(out, h->shear_buf, n * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// AeroOptics::computeAO with generateBaseBeamDiff (AeroOptics.cpp:3-93)
// ---------------------------------------------------------------------
extern "C" int cs3d_aero_optics(cs3d_handle *h, int num_angles, double max_angle, double *opl) {
    if (!h || !opl) return fail(CS3D_ERR_ARG, "null argument");
    if (num_angles < 2 || num_angles > kAeroMaxAngles)
        return fail(CS3D_ERR_ARG, "num_angles = %d (2 .. %d)", num_angles, kAeroMaxAngles);
    if (!(max_angle >= 0.0 && max_angle < 90.0)) return fail(CS3D_ERR_ARG, "max_angle = %g degrees", max_angle);
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)num_angles * h->g.Nx * h->g.Nz;
    if (n > h->aero_cap) {
        void *p = nullptr;
        int rc = dalloc(h, &p, n * 8);
        if (rc) return rc;
        h->aero_buf = (double *)p;
        h->aero_cap = n;
    }
    AeroArgs a{};
    a.g = h->g;
    a.rho = h->q1.f[0];
    a.Lx = h->cfg.Lx; a.Ly = h->cfg.Ly; a.Lz = h->cfg.Lz;
    a.dx = h->dx; a.dy = h->dy; a.dz = h->dz;
    // AeroOptics.hpp:56-63 and generateBaseBeamDiff
    a.lower = 0.2 * h->cfg.Ly;
    const double upper = 0.8 * h->cfg.Ly, totalDY = upper - a.lower;
    const double ds = std::fmin(h->dx, std::fmin(h->dy, h->dz));
    const double pi = 3.14159265358979323846;
    a.nang = num_angles;
    for (int ap = 0; ap < num_angles; ap++) {
        double minAngle = 0.0;
        double ang = minAngle + ((double)ap / ((double)(num_angles - 1))) * (max_angle - minAngle);
        ang *= pi / 180.0;
        const double Ldiag = totalDY / std::cos(ang);
        const double totalDX = Ldiag * std::sin(ang);
        const int nl = (int)std::ceil(Ldiag / ds) + 1;
        a.nline[ap] = nl;
        a.dsl[ap] = Ldiag / (double)(nl - 1);
        a.dxl[ap] = totalDX / (double)(nl - 1);
        a.dyl[ap] = totalDY / (double)(nl - 1);
    }
    a.out = h->aero_buf;
    CS3D_CUDA(launch_aero(a, h->stream));
    h->launches++;
    CS3D_CUDA(cudaMemcpyAsync(opl, h->aero_buf, n * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// allocation-free kinetic energy (no handle, no cudaMalloc, no host heap)
// ---------------------------------------------------------------------
extern "C" int cs3d_kinetic_energy_noalloc(const double *rho_dev, const double *rhoU_dev,
                                           const double *rhoV_dev, const double *rhoW_dev,
                                           long long npts, void *stream, double *ke) {
    if (!rho_dev || !rhoU_dev || !rhoV_dev || !rhoW_dev || !ke) return fail(CS3D_ERR_ARG, "null argument");
    if (npts < 1 || npts > 2147483647LL)
        return fail(CS3D_ERR_SHAPE, "npts = %lld: the allocation-free kinetic energy takes 1 .. 2^31-1 points",
                    npts);
    int dev = -1;
    CS3D_CUDA(cudaGetDevice(&dev));
    const double *ptrs[4] = {rho_dev, rhoU_dev, rhoV_dev, rhoW_dev};
    for (int f = 0; f < 4; ++f) {
        cudaPointerAttributes at{};
        CS3D_CUDA(cudaPointerGetAttributes(&at, ptrs[f]));
        if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || at.device != dev)
            return fail(CS3D_ERR_ARG, "array %d is not device memory of the current device %d", f, dev);
    }
    // the static scratch array's address on the current device, looked up on
    // every call: a device reset reloads the device code and can move it
    double *scratch = nullptr;
    CS3D_CUDA(ke_scratch_address(&scratch));
    cudaStream_t s = (cudaStream_t)stream;
    CS3D_CUDA(launch_ke_noalloc(rho_dev, rhoU_dev, rhoV_dev, rhoW_dev, npts, scratch, s));
    CS3D_CUDA(cudaMemcpyAsync(ke, scratch + kKeBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    CS3D_CUDA(cudaStreamSynchronize(s));
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// discrete adjoint of the time step (periodic boundaries, RK4, fixed dt)
// ---------------------------------------------------------------------
static int adj_check(cs3d_handle *h) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    for (int d = 0; d < 3; d++)
        if (h->cfg.bc_type[d] != CS3D_PERIODIC_SOLVE)
            return fail(CS3D_ERR_STATE, "the adjoint is built for periodic boundaries only (direction %d)", d);
    if (h->sponge || h->wall_faces) return fail(CS3D_ERR_STATE, "the adjoint is built for periodic boundaries only");
    return CS3D_OK;
}

static int adj_alloc(cs3d_handle *h, std::vector<void *> &list, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(CS3D_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    list.push_back(*p);
    return CS3D_OK;
}

static int adj_workspace(cs3d_handle *h) {
    if (h->adj_ws) return CS3D_OK;
    const size_t n = (size_t)h->g.npts;
    int rc;
    for (int i = 0; i < 48; i++) {
        if ((rc = adj_alloc(h, h->adj_allocs, &h->adj_tape[i], n * h->tb))) return rc;
        if ((rc = adj_alloc(h, h->adj_allocs, &h->adj_gbar[i], n * h->tb))) return rc;
        h->adj_tapes[0][i] = h->adj_tape[i];
        for (int st = 1; st < 4; st++)
            if ((rc = adj_alloc(h, h->adj_allocs, &h->adj_tapes[st][i], n * h->tb))) return rc;
    }
    for (int i = 0; i < 15; i++)
        if ((rc = adj_alloc(h, h->adj_allocs, &h->adj_flux[i], n * h->tb))) return rc;
    for (int g = 0; g < kAdjFields; g++)
        for (int f = 0; f < 5; f++)
            if ((rc = adj_alloc(h, h->adj_allocs, (void **)&h->adj_f[g][f], n * 8))) return rc;
    if ((rc = adj_alloc(h, h->adj_allocs, (void **)&h->adj_part, kKeSeedBlocks * 8))) return rc;
    h->adj_ws = 1;
    return CS3D_OK;
}

// one launch of k_apply along d: tasks {src, src2, dst, dst2, scale, op, acc}
// (or, f64io, {.., src64, dst64}); operator kinds 0 d1, 1 d2, 2 filter, 3 the
// FP32 filter correction F - I
template <typename T>
static int adj_apply(cs3d_handle *h, int d, int kind0, int kind1, std::initializer_list<ApplyTask<T>> tasks,
                     int f64io = 0) {
    ApplyArgs<T> a{};
    a.g = h->g;
    const int N = d == 0 ? h->g.Nx : d == 1 ? h->g.Ny : h->g.Nz;
    a.ntask = (int)tasks.size();
    const int nbuf = sizeof(T) == 4 ? 2 * ((a.ntask + 1) / 2) : a.ntask;
    a.L = pick_L(sizeof(T), nbuf, N, d == 0 ? 1 : 0, 72, true);
    a.lgL = ilog2(a.L);
    a.P = a.L + (d == 0 ? 1 : 0);
    a.threads = apply_threads<T>();
    a.divN = make_fastdiv((unsigned)N);
    const DevOp<T> *ops = sizeof(T) == 8 ? reinterpret_cast<const DevOp<T> *>(h->op64[d])
                                         : reinterpret_cast<const DevOp<T> *>(h->op32[d]);
    auto opk = [&](int kind) {
        if (kind == 3) return *reinterpret_cast<const LineOp<T> *>(&h->op32fc[d].op);
        return ops[kind].op;
    };
    a.op0 = opk(kind0);
    a.op1 = opk(kind1);
    a.f64io = f64io;
    int k = 0;
    for (const ApplyTask<T> &t : tasks) a.t[k++] = t;
    // pairs (2i, 2i+1) that write one destination are merged; every other
    // destination must occur once in the launch (the kernel reads each
    // destination it adds to before any store)
    std::vector<const void *> dsts;
    for (int i = 0; i < a.ntask; i++) {
        const bool second = (i & 1) && a.t[i].dst && a.t[i].dst == a.t[i - 1].dst;
        if (second) a.merge[i / 2] = 1;
        if (a.t[i].dst && !second) dsts.push_back(a.t[i].dst);
        if (a.t[i].dst2) dsts.push_back(a.t[i].dst2);
        if (a.t[i].dst64) dsts.push_back(a.t[i].dst64);
    }
    for (size_t i = 0; i < dsts.size(); i++)
        for (size_t j = i + 1; j < dsts.size(); j++)
            if (dsts[i] == dsts[j]) return fail(CS3D_ERR_STATE, "adjoint operator launch with a repeated destination");
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_apply<T>(d, a.op0.H, a, h->stream));
    tend(h);
    return CS3D_OK;
}

// tape G(q): primitives and the 44 derivative values of the right-hand side
template <typename T>
static int adj_tape(cs3d_handle *h, const T *const qin[5]) {
    T **G = reinterpret_cast<T **>(h->adj_tape);
    T **F = reinterpret_cast<T **>(h->adj_flux);
    TapePrepArgs<T> pa{};
    pa.g = h->g;
    pa.gas = h->gas;
    for (int f = 0; f < 5; f++) pa.qin[f] = qin[f];
    for (int i = 0; i < 4; i++) pa.prim[i] = G[i];
    for (int i = 0; i < 15; i++) pa.flux[i] = F[i];
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_tape_prep<T>(pa, h->stream));
    tend(h);
    const T one = T(1);
    int rc;
    // first and second derivatives of U V W T along d into slots b1.., b2..
    auto derivs = [&](int d, int b1, int b2) {
        return adj_apply<T>(h, d, 0, 1,
                            {{G[0], nullptr, G[b1 + 0], nullptr, one, 0, 0}, {G[0], nullptr, G[b2 + 0], nullptr, one, 1, 0},
                             {G[1], nullptr, G[b1 + 1], nullptr, one, 0, 0}, {G[1], nullptr, G[b2 + 1], nullptr, one, 1, 0},
                             {G[2], nullptr, G[b1 + 2], nullptr, one, 0, 0}, {G[2], nullptr, G[b2 + 2], nullptr, one, 1, 0},
                             {G[3], nullptr, G[b1 + 3], nullptr, one, 0, 0}, {G[3], nullptr, G[b2 + 3], nullptr, one, 1, 0}});
    };
    if ((rc = derivs(0, kInUx, kInUxx))) return rc;
    if ((rc = adj_apply<T>(h, 0, 0, 1,
                           {{F[0], nullptr, G[kInCEx], nullptr, one, 0, 0}, {F[1], nullptr, G[kInF1x], nullptr, one, 0, 0},
                            {F[2], nullptr, G[kInF2x], nullptr, one, 0, 0}, {F[3], nullptr, G[kInF3x], nullptr, one, 0, 0},
                            {F[4], nullptr, G[kInF4x], nullptr, one, 0, 0}})))
        return rc;
    if ((rc = derivs(1, kInUy, kInUyy))) return rc;
    if ((rc = adj_apply<T>(h, 1, 0, 1,
                           {{G[kInUx], nullptr, G[kInUxy], nullptr, one, 0, 0}, {G[kInVx], nullptr, G[kInVxy], nullptr, one, 0, 0},
                            {F[5], nullptr, G[kInCEy], nullptr, one, 0, 0}, {F[6], nullptr, G[kInG1y], nullptr, one, 0, 0},
                            {F[7], nullptr, G[kInG2y], nullptr, one, 0, 0}, {F[8], nullptr, G[kInG3y], nullptr, one, 0, 0},
                            {F[9], nullptr, G[kInG4y], nullptr, one, 0, 0}})))
        return rc;
    if ((rc = derivs(2, kInUz, kInUzz))) return rc;
    if ((rc = adj_apply<T>(h, 2, 0, 1,
                           {{G[kInUx], G[kInVy], G[kInS], nullptr, one, 0, 0}, {G[kInWx], nullptr, G[kInWxz], nullptr, one, 0, 0},
                            {G[kInWy], nullptr, G[kInWyz], nullptr, one, 0, 0}, {F[10], nullptr, G[kInCEz], nullptr, one, 0, 0},
                            {F[11], nullptr, G[kInH1z], nullptr, one, 0, 0}, {F[12], nullptr, G[kInH2z], nullptr, one, 0, 0},
                            {F[13], nullptr, G[kInH3z], nullptr, one, 0, 0}, {F[14], nullptr, G[kInH4z], nullptr, one, 0, 0}})))
        return rc;
    return CS3D_OK;
}

// out = J(q)^T lam for the right-hand side R(q) of one stage whose tape
// (primitives and derivative values at q) is G
// Optional fusions of the RK combination of the adjoint stage: the
// cotangent lam = ca qb2 + cb yt formed inside the pointwise VJP (qb2 set;
// yt optional), and acc = out (acc_set) or acc + out inside the chain rule.
struct VjpFuse {
    double *const *qb2 = nullptr, *const *yt = nullptr;
    double ca = 0.0, cb = 0.0;
    double *const *acc = nullptr;
    int acc_set = 0;
};

template <typename T>
static int adj_vjp_tape(cs3d_handle *h, const T *const qin[5], void *const Gv[48], double *const lam[5],
                        double *const out[5], const VjpFuse &fz = VjpFuse{}) {
    int rc;
    T *const *G = reinterpret_cast<T *const *>(Gv);
    T **B = reinterpret_cast<T **>(h->adj_gbar);
    VjpArgs<T> va{};
    va.g = h->g;
    va.gas = h->gas;
    for (int i = 0; i < 48; i++) {
        va.tape[i] = G[i];
        va.gbar[i] = B[i];
    }
    for (int f = 0; f < 5; f++) {
        va.lam[f] = lam ? lam[f] : nullptr;
        va.qb2[f] = fz.qb2 ? fz.qb2[f] : nullptr;
        va.yt[f] = fz.yt ? fz.yt[f] : nullptr;
    }
    va.ca = fz.ca;
    va.cb = fz.cb;
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_vjp<T>(va, h->stream));
    tend(h);
    // transposed operators, z then y then x: D1^T = -D1, D2^T = D2
    if constexpr (sizeof(T) == 4) {
        // one transposed sweep per direction, in the forward sweeps' tile shapes
        for (int d = 2; d >= 0; d--) {
            TSweepArgs ta{};
            ta.g = h->g;
            ta.L = h->L[d];
            ta.lgL = ilog2(h->L[d]);
            ta.P = h->L[d] + (d == 0 ? 1 : 0);
            ta.threads = h->threads[d];
            ta.divN = make_fastdiv((unsigned)(d == 0 ? h->g.Nx : d == 1 ? h->g.Ny : h->g.Nz));
            ta.d1 = h->op32[d][0].op;
            ta.d2 = h->op32[d][1].op;
            for (int q = 0; q < 48; q++) ta.gbar[q] = reinterpret_cast<float *>(B[q]);
            tstart(h, CS3D_K_OTHER);
            CS3D_CUDA(launch_tsweep(d, ta, h->stream));
            tend(h);
        }
    } else {
        const T m1 = T(-1), p1 = T(1);
        auto derivsT = [&](int d, int b1, int b2) {
            return adj_apply<T>(h, d, 0, 1,
                                {{B[b1 + 0], nullptr, B[kInU], nullptr, m1, 0, 1}, {B[b2 + 0], nullptr, B[kInU], nullptr, p1, 1, 1},
                                 {B[b1 + 1], nullptr, B[kInV], nullptr, m1, 0, 1}, {B[b2 + 1], nullptr, B[kInV], nullptr, p1, 1, 1},
                                 {B[b1 + 2], nullptr, B[kInW], nullptr, m1, 0, 1}, {B[b2 + 2], nullptr, B[kInW], nullptr, p1, 1, 1},
                                 {B[b1 + 3], nullptr, B[kInT], nullptr, m1, 0, 1}, {B[b2 + 3], nullptr, B[kInT], nullptr, p1, 1, 1}});
        };
        if ((rc = derivsT(2, kInUz, kInUzz))) return rc;
        if ((rc = adj_apply<T>(h, 2, 0, 1,
                               {{B[kInS], nullptr, B[kInUx], B[kInVy], m1, 0, 1}, {B[kInWxz], nullptr, B[kInWx], nullptr, m1, 0, 1},
                                {B[kInWyz], nullptr, B[kInWy], nullptr, m1, 0, 1}, {B[kInCEz], nullptr, B[kInCEz], nullptr, m1, 0, 0},
                                {B[kInH1z], nullptr, B[kInH1z], nullptr, m1, 0, 0}, {B[kInH2z], nullptr, B[kInH2z], nullptr, m1, 0, 0},
                                {B[kInH3z], nullptr, B[kInH3z], nullptr, m1, 0, 0}, {B[kInH4z], nullptr, B[kInH4z], nullptr, m1, 0, 0}})))
            return rc;
        if ((rc = derivsT(1, kInUy, kInUyy))) return rc;
        if ((rc = adj_apply<T>(h, 1, 0, 1,
                               {{B[kInUxy], nullptr, B[kInUx], nullptr, m1, 0, 1}, {B[kInVxy], nullptr, B[kInVx], nullptr, m1, 0, 1},
                                {B[kInCEy], nullptr, B[kInCEy], nullptr, m1, 0, 0}, {B[kInG1y], nullptr, B[kInG1y], nullptr, m1, 0, 0},
                                {B[kInG2y], nullptr, B[kInG2y], nullptr, m1, 0, 0}, {B[kInG3y], nullptr, B[kInG3y], nullptr, m1, 0, 0},
                                {B[kInG4y], nullptr, B[kInG4y], nullptr, m1, 0, 0}})))
            return rc;
        if ((rc = derivsT(0, kInUx, kInUxx))) return rc;
        if ((rc = adj_apply<T>(h, 0, 0, 1,
                               {{B[kInCEx], nullptr, B[kInCEx], nullptr, m1, 0, 0}, {B[kInF1x], nullptr, B[kInF1x], nullptr, m1, 0, 0},
                                {B[kInF2x], nullptr, B[kInF2x], nullptr, m1, 0, 0}, {B[kInF3x], nullptr, B[kInF3x], nullptr, m1, 0, 0},
                                {B[kInF4x], nullptr, B[kInF4x], nullptr, m1, 0, 0}})))
            return rc;
    }
    ChainArgs<T> ca{};
    ca.g = h->g;
    ca.gas = h->gas;
    for (int f = 0; f < 5; f++) {
        ca.qin[f] = qin[f];
        ca.out[f] = out[f];
        ca.acc[f] = fz.acc ? fz.acc[f] : nullptr;
    }
    ca.acc_set = fz.acc_set;
    for (int i = 0; i < 48; i++) ca.gbar[i] = B[i];
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_chain<T>(ca, h->stream));
    tend(h);
    return CS3D_OK;
}

// out = J(q)^T lam at a state q given on its own: the tape by the generic
// line operators, then the transposed Jacobian
template <typename T>
static int adj_rhs_vjp(cs3d_handle *h, const T *const qin[5], double *const lam[5], double *const out[5]) {
    int rc = adj_tape<T>(h, qin);
    if (rc) return rc;
    return adj_vjp_tape<T>(h, qin, h->adj_tape, lam, out);
}

// out = a x + b y + c z on five-field groups (y, z may be null)
static int adj_lin(cs3d_handle *h, double *const out[5], double a, double *const x[5], double b,
                   double *const y[5], double c = 0.0, double *const z[5] = nullptr) {
    Lin5Args la{};
    la.n = h->g.npts;
    la.a = a; la.b = b; la.c = c;
    for (int f = 0; f < 5; f++) {
        la.out[f] = out[f];
        la.x[f] = x[f];
        la.y[f] = y ? y[f] : nullptr;
        la.z[f] = z ? z[f] : nullptr;
    }
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_lin5(la, h->stream));
    tend(h);
    return CS3D_OK;
}

static int copy5(cs3d_handle *h, double *const dst[5], double *const src[5]) {
    const size_t bytes = (size_t)h->g.npts * 8;
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(dst[f], src[f], bytes, cudaMemcpyDeviceToDevice, h->stream));
    return CS3D_OK;
}

static void slab5(cs3d_handle *h, double *base, double *out[5]) {
    for (int f = 0; f < 5; f++) out[f] = base + (size_t)f * (size_t)h->g.npts;
}

// the filter order of filterConservedData for filter step number fts
static void filter_order(int fts, int order[3]) {
    const int m3 = fts % 3;
    if (m3 == 1) { order[0] = 0; order[1] = 1; order[2] = 2; }
    else if (m3 == 2) { order[0] = 1; order[1] = 2; order[2] = 0; }
    else { order[0] = 2; order[1] = 0; order[2] = 1; }
}

// The solver's state q1 := q (and, in the mixed form, its FP32 shadow).
static int adj_set_state(cs3d_handle *h, double *const q[5]) {
    int rc = copy5(h, h->q1.f, q);
    if (rc) return rc;
    return h->mixed ? launch_shadow_of(h, h->q1, h->q1s) : CS3D_OK;
}

// The backward part of one time step from the state's filter step count fts
// before it, whether it filtered, its stage inputs yin and its stage tapes:
// adj_f[ADJ_QB] holds dJ/dq after the step on entry and dJ/dq before it on
// return.
template <typename T>
static int adj_back(cs3d_handle *h, int fts, bool filtered, const T *const yin[4][5], void *const tapes[4][48]) {
    int rc;
    double **QB = h->adj_f[ADJ_QB], **QB2 = h->adj_f[ADJ_QB2];
    double **YS = h->adj_f[ADJ_YS], **YT = h->adj_f[ADJ_YT];
    const double dt = h->cfg.dt_fixed;
    // the filter's transpose: F = F_o2 F_o1 F_o0, F^T = F_o0 F_o1 F_o2 (each symmetric)
    if ((rc = copy5(h, QB2, QB))) return rc;
    if (filtered) {
        int order[3];
        filter_order(fts + 1, order);
        for (int pass = 2; pass >= 0; pass--) {
            const int d = order[pass];
            if (sizeof(T) == 4) {
                // mixed handle: F^T qbar = qbar + (F - I) qbar with the
                // correction in FP32 and the sum in FP64, the form of the
                // mixed forward filter
                if ((rc = adj_apply<float>(h, d, 3, 3,
                                           {{nullptr, nullptr, nullptr, nullptr, 1.f, 0, 0, QB2[0], QB2[0]},
                                            {nullptr, nullptr, nullptr, nullptr, 1.f, 0, 0, QB2[1], QB2[1]},
                                            {nullptr, nullptr, nullptr, nullptr, 1.f, 0, 0, QB2[2], QB2[2]},
                                            {nullptr, nullptr, nullptr, nullptr, 1.f, 0, 0, QB2[3], QB2[3]},
                                            {nullptr, nullptr, nullptr, nullptr, 1.f, 0, 0, QB2[4], QB2[4]}},
                                           1)))
                    return rc;
                continue;
            }
            if ((rc = adj_apply<double>(h, d, 2, 2,
                                        {{QB2[0], nullptr, QB2[0], nullptr, 1.0, 0, 0},
                                         {QB2[1], nullptr, QB2[1], nullptr, 1.0, 0, 0},
                                         {QB2[2], nullptr, QB2[2], nullptr, 1.0, 0, 0},
                                         {QB2[3], nullptr, QB2[3], nullptr, 1.0, 0, 0},
                                         {QB2[4], nullptr, QB2[4], nullptr, 1.0, 0, 0}})))
                return rc;
        }
    }
    if (h->cfg.rk == CS3D_TVDRK3) {
        // TVD-RK3 (TVDRK3.hpp:38-96) in reverse: y2 = y1 + dt R(y1),
        // y3 = 3/4 y1 + 1/4 y2 + 1/4 dt R(y2), q+ = 1/3 y1 + 2/3 y3 + 2/3 dt R(y3)
        // with y1 = q.  ybar3 = 2/3 qbar+ + J(y3)^T (2/3 dt qbar+) in YS,
        // ybar2 = 1/4 ybar3 + J(y2)^T (dt/4 ybar3) in LAM, and
        // qbar = 1/3 qbar+ + 3/4 ybar3 + ybar2 + J(y1)^T (dt ybar2); each
        // cotangent lam is formed in the VJP kernel, the last VJP added into
        // qbar by the chain-rule kernel.
        double **LAM = h->adj_f[ADJ_LAM];
        VjpFuse f3;
        f3.qb2 = QB2;
        f3.ca = 2.0 * dt / 3.0;
        if ((rc = adj_vjp_tape<T>(h, yin[2], tapes[2], nullptr, YT, f3))) return rc;
        if ((rc = adj_lin(h, YS, 2.0 / 3.0, QB2, 1.0, YT))) return rc;
        VjpFuse f2;
        f2.qb2 = YS;
        f2.ca = 0.25 * dt;
        if ((rc = adj_vjp_tape<T>(h, yin[1], tapes[1], nullptr, YT, f2))) return rc;
        if ((rc = adj_lin(h, LAM, 0.25, YS, 1.0, YT))) return rc;
        if ((rc = adj_lin(h, QB, 1.0 / 3.0, QB2, 0.75, YS, 1.0, LAM))) return rc;
        VjpFuse f1;
        f1.qb2 = LAM;
        f1.ca = dt;
        f1.acc = QB;
        return adj_vjp_tape<T>(h, yin[0], tapes[0], nullptr, YT, f1);
    }
    // RK4 (RK4.hpp:35-118) in reverse: q+ = q + dt/6 (k1 + 2 k2 + 2 k3 + k4),
    // y2 = q + dt/2 k1, y3 = q + dt/2 k2, y4 = q + dt k3, k_s = R(y_s)
    const double ca[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};  // weight of k_s in q+
    const double cb[4] = {dt / 2.0, dt / 2.0, dt, 0.0};             // weight of k_s in y_{s+1}
    for (int s = 3; s >= 0; s--) {
        // lam_s = ca_s qbar+ + cb_s ybar_{s+1} (formed in the VJP kernel);
        // ybar_s = J(y_s)^T lam_s into YT, and YS = sum of the ybar_s (in the
        // chain-rule kernel)
        VjpFuse fz;
        fz.qb2 = QB2;
        fz.yt = s == 3 ? nullptr : YT;
        fz.ca = ca[s];
        fz.cb = cb[s];
        fz.acc = YS;
        fz.acc_set = s == 3;
        if ((rc = adj_vjp_tape<T>(h, yin[s], tapes[s], nullptr, YT, fz))) return rc;
    }
    return adj_lin(h, QB, 1.0, QB2, 1.0, YS);
}

// Adjoint of one time step taken from the state q0 with counters (ts, fts):
// the stages run again with their sweeps writing the stage tapes, then
// adj_back.  T is the work type: the stage Jacobians are transposed in T at
// the stage inputs the forward used (FP64 q1, qk; or, in the mixed form, the
// FP32 shadows q1s, qks); the adjoint state and the filter transpose stay FP64.
template <typename T>
static int adj_step(cs3d_handle *h, int ts, int fts, double *const q0[5]) {
    int rc;
    double **Y[3] = {h->adj_f[ADJ_Y2], h->adj_f[ADJ_Y3], h->adj_f[ADJ_Y4]};
    const size_t n = (size_t)h->g.npts;
    // stage inputs y1 = q0, y2, y3 (, y4) of the forward step, in T
    const T *yin[4][5];
    h->timeStep = ts;
    h->filterTimeStep = fts;
    if ((rc = adj_set_state(h, q0))) return rc;
    for (int f = 0; f < 5; f++) yin[0][f] = sizeof(T) == 8 ? (const T *)q0[f] : (const T *)h->q1s[f];
    if ((rc = cs3d_pre_step(h))) return rc;
    // the stages again: their sweeps write the stage tapes (the values the
    // stage's right-hand side was formed from), and every stage but the last
    // gives the input of the next
    for (int st = 1; st <= h->nstages; st++) {
        for (int i = 0; i < 48; i++) h->tape_out[i] = h->adj_tapes[st - 1][i];
        rc = run_stage<T>(h, st, 0);
        for (int i = 0; i < 48; i++) h->tape_out[i] = nullptr;
        if (rc) return rc;
        if (st == h->nstages) break;
        for (int f = 0; f < 5; f++) {
            const void *src = sizeof(T) == 8 ? (const void *)h->qk.f[f] : (const void *)h->qks[f];
            CS3D_CUDA(cudaMemcpyAsync(Y[st - 1][f], src, n * sizeof(T), cudaMemcpyDeviceToDevice, h->stream));
            yin[st][f] = (const T *)Y[st - 1][f];
        }
    }
    const bool filtered = h->timeStep % h->cfg.filter_step == 0;
    return adj_back<T>(h, fts, filtered, yin, h->adj_tapes);
}

// Segment mode: one full time step from the current state (as cs3d_step)
// with the sweeps writing the tapes of its stages, and the stage inputs
// copied, into slot j of the segment storage (four stage slots a step).
template <typename T>
static int adj_taped_step(cs3d_handle *h, int j) {
    int rc;
    const size_t fb = (size_t)h->g.npts * sizeof(T);
    if ((rc = cs3d_pre_step(h))) return rc;
    for (int st = 1; st <= h->nstages; st++) {
        char *yb = h->adj_segyin + (size_t)((j * 4 + st - 1) * 5) * fb;
        for (int f = 0; f < 5; f++) {
            const void *src = st == 1 ? (sizeof(T) == 8 ? (const void *)h->q1.f[f] : (const void *)h->q1s[f])
                                      : (sizeof(T) == 8 ? (const void *)h->qk.f[f] : (const void *)h->qks[f]);
            CS3D_CUDA(cudaMemcpyAsync(yb + f * fb, src, fb, cudaMemcpyDeviceToDevice, h->stream));
        }
        char *tb = h->adj_segtape + (size_t)((j * 4 + st - 1) * 48) * fb;
        for (int i = 0; i < 48; i++) h->tape_out[i] = tb + i * fb;
        rc = run_stage<T>(h, st, st == h->nstages);
        for (int i = 0; i < 48; i++) h->tape_out[i] = nullptr;
        if (rc) return rc;
    }
    return cs3d_post_step(h);
}

// Segment mode: the backward part of step j of the segment, from the storage.
template <typename T>
static int adj_back_stored(cs3d_handle *h, int j, int ts, int fts) {
    const size_t fb = (size_t)h->g.npts * sizeof(T);
    const T *yin[4][5];
    void *tapes[4][48];
    for (int st = 0; st < 4; st++) {
        for (int f = 0; f < 5; f++)
            yin[st][f] = reinterpret_cast<const T *>(h->adj_segyin + (size_t)((j * 4 + st) * 5 + f) * fb);
        for (int i = 0; i < 48; i++) tapes[st][i] = h->adj_segtape + (size_t)((j * 4 + st) * 48 + i) * fb;
    }
    return adj_back<T>(h, fts, (ts + 1) % h->cfg.filter_step == 0, yin, tapes);
}

extern "C" int cs3d_adjoint_record(cs3d_handle *h, int nsteps, int checkpoint_every) {
    int rc = adj_check(h);
    if (rc) return rc;
    if (!(h->cfg.dt_fixed > 0.0)) return fail(CS3D_ERR_STATE, "the adjoint needs a fixed time step (cfg.dt_fixed > 0)");
    if (nsteps < 1) return fail(CS3D_ERR_ARG, "nsteps = %d", nsteps);
    if (checkpoint_every < 0) return fail(CS3D_ERR_ARG, "checkpoint_every = %d", checkpoint_every);
    DeviceGuard dg(h->dev);
    int every = checkpoint_every;
    if (every == 0) every = (int)std::ceil(std::sqrt((double)nsteps));
    if (every > nsteps) every = nsteps;
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    for (void *p : h->adj_rec_allocs) cudaFree(p);
    h->adj_rec_allocs.clear();
    h->adj_ckpt.clear();
    h->adj_ts.clear();
    h->adj_fts.clear();
    h->adj_nsteps = 0;
    if ((rc = adj_workspace(h))) return rc;
    const size_t n5 = (size_t)h->g.npts * 5;
    const int nseg = (nsteps + every - 1) / every;
    for (int k = 0; k < nseg; k++) {
        void *p = nullptr;
        if ((rc = adj_alloc(h, h->adj_rec_allocs, &p, n5 * 8))) return rc;
        h->adj_ckpt.push_back((double *)p);
    }
    if ((rc = adj_alloc(h, h->adj_rec_allocs, (void **)&h->adj_seg, n5 * 8 * (size_t)every))) return rc;
    // segment mode where the tapes and stage inputs of one segment (212 fields
    // in the work precision per step) fit in half of the free device memory
    h->adj_segmode = 0;
    h->adj_segtape = h->adj_segyin = nullptr;
    {
        const size_t fb = (size_t)h->g.npts * h->tb;
        const size_t tape_b = (size_t)every * 4 * 48 * fb, yin_b = (size_t)every * 4 * 5 * fb;
        size_t free_b = 0, total_b = 0;
        CS3D_CUDA(cudaMemGetInfo(&free_b, &total_b));
        if (!h->adj_recompute && tape_b + yin_b <= free_b / 2) {
            if ((rc = adj_alloc(h, h->adj_rec_allocs, (void **)&h->adj_segtape, tape_b))) return rc;
            if ((rc = adj_alloc(h, h->adj_rec_allocs, (void **)&h->adj_segyin, yin_b))) return rc;
            h->adj_segmode = 1;
        }
    }
    for (int k = 0; k < nsteps; k++) {
        if (k % every == 0) {
            double *ck[5];
            slab5(h, h->adj_ckpt[k / every], ck);
            if ((rc = copy5(h, ck, h->q1.f))) return rc;
            h->adj_ts.push_back(h->timeStep);
            h->adj_fts.push_back(h->filterTimeStep);
        }
        if ((rc = cs3d_step(h))) return rc;
    }
    h->adj_end_ts = h->timeStep;
    h->adj_end_fts = h->filterTimeStep;
    CS3D_CUDA(cudaMemcpyAsync(h->adj_end_scal, h->scal, 2 * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    h->adj_nsteps = nsteps;
    h->adj_every = every;
    return CS3D_OK;
}

extern "C" int cs3d_adjoint_backward(cs3d_handle *h, int objective, const double *seed_host, double *grad_host,
                                     double *J) {
    int rc = adj_check(h);
    if (rc) return rc;
    if (!h->adj_nsteps) return fail(CS3D_ERR_STATE, "call cs3d_adjoint_record first");
    if (!grad_host) return fail(CS3D_ERR_ARG, "null gradient");
    if (objective != CS3D_ADJ_SEED && objective != CS3D_ADJ_KE_MEAN)
        return fail(CS3D_ERR_ARG, "objective = %d", objective);
    if (objective == CS3D_ADJ_SEED && !seed_host) return fail(CS3D_ERR_ARG, "null seed");
    if (h->timeStep != h->adj_end_ts) return fail(CS3D_ERR_STATE, "the solver has stepped since the record");
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)h->g.npts;
    double **QB = h->adj_f[ADJ_QB], **FIN = h->adj_f[ADJ_FIN];
    // dJ/dq at the final state
    if (objective == CS3D_ADJ_KE_MEAN) {
        KeSeedArgs ka{};
        ka.g = h->g;
        ka.q = h->q1;
        for (int f = 0; f < 5; f++) ka.seed[f] = QB[f];
        ka.part = h->adj_part;
        tstart(h, CS3D_K_OTHER);
        CS3D_CUDA(launch_ke_seed(ka, h->stream));
        tend(h);
        double part[kKeSeedBlocks];
        CS3D_CUDA(cudaMemcpyAsync(part, h->adj_part, sizeof(part), cudaMemcpyDeviceToHost, h->stream));
        CS3D_CUDA(cudaStreamSynchronize(h->stream));
        double s = 0.0;
        for (int b = 0; b < kKeSeedBlocks; b++) s += part[b];
        if (J) *J = s / (double)h->g.npts;
    } else {
        for (int f = 0; f < 5; f++)
            CS3D_CUDA(cudaMemcpyAsync(QB[f], seed_host + (size_t)f * n, n * 8, cudaMemcpyHostToDevice, h->stream));
        if (J) *J = 0.0;
    }
    if ((rc = copy5(h, FIN, h->q1.f))) return rc;
    // segments in reverse: replay the segment's states from its checkpoint,
    // then take the steps back one by one
    const int every = h->adj_every, nsteps = h->adj_nsteps;
    const int nseg = (nsteps + every - 1) / every;
    std::vector<int> tsv(every), ftsv(every);
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int s0 = sg * every, m = std::min(nsteps, s0 + every) - s0;
        double *st[5];
        slab5(h, h->adj_seg, st);
        double *ck[5];
        slab5(h, h->adj_ckpt[sg], ck);
        if ((rc = copy5(h, st, ck))) return rc;
        h->timeStep = h->adj_ts[sg];
        h->filterTimeStep = h->adj_fts[sg];
        if (h->adj_segmode) {
            // replay the segment once, its steps keeping their tapes and stage
            // inputs; then take the steps back from that storage.  Each step
            // starts from its FP64 state, as in the per-step recompute.
            for (int j = 0; j < m; j++) {
                double *cur[5];
                slab5(h, h->adj_seg, cur);
                tsv[j] = h->timeStep;
                ftsv[j] = h->filterTimeStep;
                if ((rc = adj_set_state(h, cur))) return rc;
                rc = h->mixed ? adj_taped_step<float>(h, j) : adj_taped_step<double>(h, j);
                if (rc) return rc;
                if (j + 1 < m && (rc = copy5(h, cur, h->q1.f))) return rc;
            }
            for (int j = m - 1; j >= 0; j--) {
                rc = h->mixed ? adj_back_stored<float>(h, j, tsv[j], ftsv[j])
                              : adj_back_stored<double>(h, j, tsv[j], ftsv[j]);
                if (rc) return rc;
            }
            continue;
        }
        for (int j = 0; j < m; j++) {
            tsv[j] = h->timeStep;
            ftsv[j] = h->filterTimeStep;
            if (j + 1 < m) {
                double *cur[5], *nxt[5];
                slab5(h, h->adj_seg + (size_t)j * 5 * n, cur);
                slab5(h, h->adj_seg + (size_t)(j + 1) * 5 * n, nxt);
                if ((rc = adj_set_state(h, cur))) return rc;
                if ((rc = cs3d_step(h))) return rc;
                if ((rc = copy5(h, nxt, h->q1.f))) return rc;
            }
        }
        for (int j = m - 1; j >= 0; j--) {
            double *cur[5];
            slab5(h, h->adj_seg + (size_t)j * 5 * n, cur);
            rc = h->mixed ? adj_step<float>(h, tsv[j], ftsv[j], cur) : adj_step<double>(h, tsv[j], ftsv[j], cur);
            if (rc) return rc;
        }
    }
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(grad_host + (size_t)f * n, QB[f], n * 8, cudaMemcpyDeviceToHost, h->stream));
    // back to the recorded final state
    if ((rc = adj_set_state(h, FIN))) return rc;
    h->timeStep = h->adj_end_ts;
    h->filterTimeStep = h->adj_end_fts;
    CS3D_CUDA(cudaMemcpyAsync(h->scal, h->adj_end_scal, 2 * 8, cudaMemcpyHostToDevice, h->stream));
    if ((rc = launch_cfl_reduce(h))) return rc;
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

// R(q) from the tape, and J(q)^T lam, for one state given on the host
static int adj_upload_state(cs3d_handle *h, const double *q_host, double *const dst[5]) {
    const size_t n = (size_t)h->g.npts;
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(dst[f], q_host + (size_t)f * n, n * 8, cudaMemcpyHostToDevice, h->stream));
    return CS3D_OK;
}

// FP32 copy of five FP64 fields, in the ADJ_Y3 group's storage
static int adj_narrow(cs3d_handle *h, double *const q[5], float *out[5]) {
    Q5 src{};
    for (int f = 0; f < 5; f++) {
        src.f[f] = q[f];
        out[f] = (float *)h->adj_f[ADJ_Y3][f];
    }
    return launch_shadow_of(h, src, out);
}

template <typename T>
static int adj_rhs_eval(cs3d_handle *h, double *const Q[5], double *const R[5]) {
    const T *qin[5];
    int rc;
    if (sizeof(T) == 4) {
        float *qs[5];
        if ((rc = adj_narrow(h, Q, qs))) return rc;
        for (int f = 0; f < 5; f++) qin[f] = (const T *)qs[f];
    } else {
        for (int f = 0; f < 5; f++) qin[f] = (const T *)Q[f];
    }
    if ((rc = adj_tape<T>(h, qin))) return rc;
    RhsEvalArgs<T> ra{};
    ra.g = h->g;
    ra.gas = h->gas;
    for (int i = 0; i < 48; i++) ra.tape[i] = (const T *)h->adj_tape[i];
    for (int f = 0; f < 5; f++) ra.R[f] = R[f];
    tstart(h, CS3D_K_OTHER);
    CS3D_CUDA(launch_rhs_eval<T>(ra, h->stream));
    tend(h);
    return CS3D_OK;
}

extern "C" int cs3d_rhs_eval(cs3d_handle *h, const double *q_host, double *R_host) {
    int rc = adj_check(h);
    if (rc) return rc;
    if (!q_host || !R_host) return fail(CS3D_ERR_ARG, "null argument");
    DeviceGuard dg(h->dev);
    if ((rc = adj_workspace(h))) return rc;
    double **Q = h->adj_f[ADJ_Y2], **R = h->adj_f[ADJ_YT];
    if ((rc = adj_upload_state(h, q_host, Q))) return rc;
    rc = h->mixed ? adj_rhs_eval<float>(h, Q, R) : adj_rhs_eval<double>(h, Q, R);
    if (rc) return rc;
    const size_t n = (size_t)h->g.npts;
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(R_host + (size_t)f * n, R[f], n * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

extern "C" int cs3d_rhs_vjp(cs3d_handle *h, const double *q_host, const double *lam_host, double *out_host) {
    int rc = adj_check(h);
    if (rc) return rc;
    if (!q_host || !lam_host || !out_host) return fail(CS3D_ERR_ARG, "null argument");
    DeviceGuard dg(h->dev);
    if ((rc = adj_workspace(h))) return rc;
    double **Q = h->adj_f[ADJ_Y2], **LAM = h->adj_f[ADJ_LAM], **OUT = h->adj_f[ADJ_YT];
    if ((rc = adj_upload_state(h, q_host, Q))) return rc;
    if ((rc = adj_upload_state(h, lam_host, LAM))) return rc;
    if (h->mixed) {
        float *qs[5];
        if ((rc = adj_narrow(h, Q, qs))) return rc;
        rc = adj_rhs_vjp<float>(h, qs, LAM, OUT);
    } else {
        rc = adj_rhs_vjp<double>(h, Q, LAM, OUT);
    }
    if (rc) return rc;
    const size_t n = (size_t)h->g.npts;
    for (int f = 0; f < 5; f++)
        CS3D_CUDA(cudaMemcpyAsync(out_host + (size_t)f * n, OUT[f], n * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// dumpSolution format (CSolver_AWS.cpp:2493-2535): q1 as five raw FP64
// files in XYZ order, no header, named rho.out.<step> ... rhoE.out.<step>
// ---------------------------------------------------------------------
static const char *const kDumpNames[5] = {"rho", "rhoU", "rhoV", "rhoW", "rhoE"};

static std::string dump_path(const char *prefix, int f, int step) {
    return std::string(prefix ? prefix : "") + kDumpNames[f] + ".out." + std::to_string(step);
}

extern "C" int cs3d_dump_solution(cs3d_handle *h, const char *prefix) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)h->g.npts;
    std::vector<double> buf(n);
    for (int f = 0; f < 5; f++) {
        CS3D_CUDA(cudaMemcpyAsync(buf.data(), h->q1.f[f], n * 8, cudaMemcpyDeviceToHost, h->stream));
        CS3D_CUDA(cudaStreamSynchronize(h->stream));
        const std::string path = dump_path(prefix, f, h->timeStep);
        FILE *fp = fopen(path.c_str(), "wb");
        if (!fp) return fail(CS3D_ERR_IO, "cannot open %s for writing", path.c_str());
        const size_t w = fwrite(buf.data(), sizeof(double), n, fp);
        const int c = fclose(fp);
        if (w != n || c != 0) return fail(CS3D_ERR_IO, "short write to %s", path.c_str());
    }
    return CS3D_OK;
}

extern "C" int cs3d_load_solution(cs3d_handle *h, const char *prefix, int time_step, double time) {
    if (!h) return fail(CS3D_ERR_ARG, "null handle");
    if (time_step < 0) return fail(CS3D_ERR_ARG, "time_step = %d", time_step);
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)h->g.npts;
    std::vector<double> buf(n);
    for (int f = 0; f < 5; f++) {
        const std::string path = dump_path(prefix, f, time_step);
        FILE *fp = fopen(path.c_str(), "rb");
        if (!fp) return fail(CS3D_ERR_IO, "cannot open %s", path.c_str());
        const size_t r = fread(buf.data(), sizeof(double), n, fp);
        const int extra = fgetc(fp);
        fclose(fp);
        if (r != n || extra != EOF)
            return fail(CS3D_ERR_SHAPE, "%s does not hold %zu doubles (%d x %d x %d)", path.c_str(), n, h->g.Nx,
                        h->g.Ny, h->g.Nz);
        CS3D_CUDA(cudaMemcpyAsync(h->q1.f[f], buf.data(), n * 8, cudaMemcpyHostToDevice, h->stream));
        CS3D_CUDA(cudaStreamSynchronize(h->stream));
    }
    int rc = init_after_state(h);
    if (rc) return rc;
    h->timeStep = time_step;
    h->filterTimeStep = time_step / h->cfg.filter_step;  // filtered steps so far
    double sc[2] = {0.0, time};
    CS3D_CUDA(cudaMemcpyAsync(h->scal, sc, 2 * 8, cudaMemcpyHostToDevice, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}

// ---------------------------------------------------------------------
// post-processor: vorticity magnitude and Q-criterion (PostProcess.cpp:190-310)
// ---------------------------------------------------------------------
extern "C" int cs3d_vorticity_q(cs3d_handle *h, double *vort, double *qcrit) {
    if (!h || !vort || !qcrit) return fail(CS3D_ERR_ARG, "null argument");
    if (!h->ic_done) return fail(CS3D_ERR_STATE, "cs3d_set_initial_conditions has not been called");
    DeviceGuard dg(h->dev);
    const size_t n = (size_t)h->g.npts;
    if (!h->post_buf) {
        int rc = dalloc(h, (void **)&h->post_buf, 14 * n * 8);
        if (rc) return rc;
    }
    PostArgs a{};
    a.g = h->g;
    a.q = h->q1;
    double *d[3][3];
    for (int c = 0; c < 3; c++) {
        a.vel[c] = h->post_buf + (size_t)c * n;
        for (int e = 0; e < 3; e++) {
            d[c][e] = h->post_buf + (size_t)(3 + 3 * c + e) * n;
            a.d[c][e] = d[c][e];
        }
    }
    a.vort = h->post_buf + 12 * n;
    a.qcrit = h->post_buf + 13 * n;
    CS3D_CUDA(launch_velocity(a, h->stream));
    h->launches++;
    // the nine first derivatives with the solver's FP64 operators, one launch per direction
    for (int e = 0; e < 3; e++) {
        int rc = adj_apply<double>(h, e, 0, 1,
                                   {{a.vel[0], nullptr, d[0][e], nullptr, 1.0, 0, 0},
                                    {a.vel[1], nullptr, d[1][e], nullptr, 1.0, 0, 0},
                                    {a.vel[2], nullptr, d[2][e], nullptr, 1.0, 0, 0}});
        if (rc) return rc;
    }
    CS3D_CUDA(launch_vort_q(a, h->stream));
    h->launches++;
    CS3D_CUDA(cudaMemcpyAsync(vort, a.vort, n * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaMemcpyAsync(qcrit, a.qcrit, n * 8, cudaMemcpyDeviceToHost, h->stream));
    CS3D_CUDA(cudaStreamSynchronize(h->stream));
    return CS3D_OK;
}
