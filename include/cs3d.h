/*
 * cs3d.h -- C ABI of the GB300 implementation of the per-Runge-Kutta-stage
 * path of 3DCompactSolver (compact derivatives, compact filter, Euler and
 * viscous right-hand side, RK4 / TVD-RK3 stage update).
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (CS3D_OK on success).  Host pointers are caller-owned; device pointers
 * ("_dev") must point to memory on the handle's GPU.  One handle owns one CUDA
 * stream; calls on one handle must come from one host thread at a time, as
 * with the reference's single-threaded driver loop.
 *
 * Citations are to files of the reference project (emathew1/3DCompactSolver).
 */
#ifndef CS3D_H
#define CS3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define CS3D_OK          0
#define CS3D_ERR_ARG     1  /* null pointer, bad enum, bad index            */
#define CS3D_ERR_SHAPE   2  /* grid too small for the requested closure     */
#define CS3D_ERR_CUDA    3  /* a CUDA call failed (cs3d_last_error says which) */
#define CS3D_ERR_NAN     4  /* a non-finite value reached the state         */
#define CS3D_ERR_ALLOC   5  /* device or host allocation failed             */
#define CS3D_ERR_STATE   6  /* call made in the wrong order                 */
#define CS3D_ERR_NODEV   7  /* no CUDA device visible                       */
#define CS3D_ERR_IO      8  /* a file could not be opened, read or written  */

/* ---- enumerations (values equal the reference's enums) ---------------- */
/* BC::BCType, BC.hpp:10 */
#define CS3D_PERIODIC_SOLVE   0
#define CS3D_DIRICHLET_SOLVE  1
/* BC::BCKind, BC.hpp:11 */
#define CS3D_PERIODIC               0
#define CS3D_SPONGE                 1
#define CS3D_ADIABATIC_WALL         2
#define CS3D_MOVING_ADIABATIC_WALL  3
#define CS3D_INLET                  4
/* Derivatives::Direct, Derivatives.hpp:48 */
#define CS3D_DIRX 0
#define CS3D_DIRY 1
#define CS3D_DIRZ 2
/* time integrators: RK4.hpp, TVDRK3.hpp */
#define CS3D_RK4     0
#define CS3D_TVDRK3  1
/* arithmetic of the stage */
#define CS3D_FP64        0  /* plain form: every operation in FP64        */
#define CS3D_FP32_MIXED  1  /* RHS, flux, derivative and filter arithmetic in
                               FP32; conserved state q1/q2, the RK
                               accumulation q2 += a_s dq of every stage and
                               the cyclic Sherman-Morrison factor in FP64;
                               the RK4 stage input qk = q1 + b_s dq is kept
                               as an FP32 shadow only                       */
/* sponge construction */
#define CS3D_SPONGE_REFERENCE 0 /* sigma built only on SPONGE faces with the
                                   reference's band widths 0.25Lx, 0.125Ly,
                                   0.25Lz (SpongeBC.hpp:56-62)             */
#define CS3D_SPONGE_BANDS     1 /* sigma built on every face whose entry of
                                   sponge_frac is > 0, band = frac * L      */

/* Solver configuration.  Mirrors the constructor arguments of Domain
 * (Domain.hpp:16), BC (BC.hpp:16), TimeStepping (TimeStepping.hpp:20) and
 * CSolver_AWS (CSolver_AWS.hpp:119), plus the choice of integrator. */
typedef struct cs3d_config {
    int    Nx, Ny, Nz;          /* grid points per direction                */
    double Lx, Ly, Lz;          /* x_i = i*L/(N-1), Domain.hpp:31-41        */
    int    bc_type[3];          /* CS3D_PERIODIC_SOLVE / CS3D_DIRICHLET_SOLVE */
    int    bc_kind[6];          /* faces X0,X1,Y0,Y1,Z0,Z1: CS3D_PERIODIC..  */
    double alphaF;              /* compact filter coefficient               */
    double mu_ref;              /* reference viscosity, IdealGas.hpp:40     */
    double CFL;                 /* constant-CFL time step                   */
    double dt_fixed;            /* > 0: frozen dt (adjoint); else CFL rule  */
    int    filter_step;         /* filter when timeStep % filter_step == 0  */
    int    rk;                  /* CS3D_RK4 / CS3D_TVDRK3                   */
    int    precision;           /* CS3D_FP64 / CS3D_FP32_MIXED              */
    int    sponge_mode;         /* CS3D_SPONGE_REFERENCE / CS3D_SPONGE_BANDS */
    double sponge_frac[6];      /* band fraction per face (SPONGE_BANDS)    */
    /* moving-wall velocities, CSolver_AWS.hpp:104-106, in the order
     * X0V X0W X1V X1W Y0U Y0W Y1U Y1W Z0U Z0V Z1U Z1V */
    double wall_vel[12];
} cs3d_config;

/* Fields addressable by cs3d_get_field / cs3d_set_field.  Conserved fields
 * follow AbstractCSolver.hpp:19-26; primitives CSolver_AWS.hpp:40-48. */
#define CS3D_F_RHO1   0
#define CS3D_F_RHOU1  1
#define CS3D_F_RHOV1  2
#define CS3D_F_RHOW1  3
#define CS3D_F_RHOE1  4
#define CS3D_F_RHOK   5   /* rhok..rhoEk: stage input (qk)      5..9  */
#define CS3D_F_RHO2   10  /* rho2..rhoE2: RK accumulator (q2)  10..14 */
#define CS3D_F_RHOK2  15  /* rhok2..rhoEk2: last increment dq  15..19 */
#define CS3D_F_U      20  /* U V W p T mu sos from q1 (the solver's
                             primitives after the last stage)  20..26 */
#define CS3D_F_SPONGE_AVG 27 /* sponge running averages        27..31 */
#define CS3D_F_SIGMA  32
#define CS3D_NUM_FIELDS 33

typedef struct cs3d_handle cs3d_handle;

/* Last error message of the calling thread (static storage). */
const char *cs3d_last_error(void);

/* Library version and the CUDA architecture it was built for. */
int cs3d_version(int *major, int *minor, int *sm_arch);

/* Create / destroy a solver on the current CUDA device.  Replaces
 * `new CSolver_AWS(dom, bc, ts, alphaF, mu_ref, blocksize, useTiming)`
 * (CSolver_AWS.hpp:119-185) plus initializeSolverData (CSolver_AWS.cpp:3-196).
 * Device memory is allocated here and nowhere else. */
int cs3d_create(const cs3d_config *cfg, cs3d_handle **out);
int cs3d_destroy(cs3d_handle *h);

/* Initial conditions from host arrays (XYZ layout, Nx*Ny*Nz doubles each).
 * Replaces writing cs->rho0,p0,U0,V0,W0 and calling setInitialConditions
 * (CSolver_AWS.cpp:199-504), including the wall overwrite, the sponge
 * average initialisation and the primitive update. */
int cs3d_set_initial_conditions(cs3d_handle *h, const double *rho0, const double *p0,
                                const double *U0, const double *V0, const double *W0);

/* One time step: calcDtFromCFL (CSolver_AWS.cpp:507-551), every RK stage
 * (RK4.hpp:120-170 / TVDRK3.hpp:98-139) and updateSponge
 * (CSolver_AWS.cpp:1937-2031).  Diagnostics and file output of postStep are
 * not part of the path. */
int cs3d_step(cs3d_handle *h);
/* Run n steps back to back with no host synchronisation in between. */
int cs3d_run(cs3d_handle *h, int n);

/* The pieces of cs3d_step, for drivers that call the reference's virtuals
 * one by one (AbstractCSolver.hpp:36-43, AbstractRK.hpp:13-14). */
int cs3d_pre_step(cs3d_handle *h);                            /* preStep      */
int cs3d_sub_step(cs3d_handle *h, int rk_step, int rk_last);  /* preSubStep + solveEqnSet
                                                                 + postSubStep
                                                                 + updateConservedData
                                                                 + updateData */
int cs3d_post_step(cs3d_handle *h);                           /* updateSponge */

/* Wait for all queued work; returns CS3D_ERR_NAN if the device status flag
 * saw a non-finite value in the state since the last call. */
int cs3d_sync(cs3d_handle *h);

/* Copy a field (Nx*Ny*Nz doubles, XYZ layout) between host and device. */
int cs3d_get_field(cs3d_handle *h, int field, double *host_out);
int cs3d_set_field(cs3d_handle *h, int field, const double *host_in);
/* The conserved state q1 (rho1, rhoU1, rhoV1, rhoW1, rhoE1; AbstractCSolver.hpp:
 * 19-26) between host and device in one call: the five copies are queued
 * together and waited for once.  Same result as cs3d_get_field /
 * cs3d_set_field on fields 0..4.  Setting the state leaves the CFL maximum
 * of the state the last step ended with, from which the next cs3d_pre_step
 * takes dt -- as the reference's calcDtFromCFL reads the primitive arrays of
 * its last updateNonConservedData (CSolver_AWS.cpp:507-525, 1895-1935), not
 * arrays written since; cs3d_set_initial_conditions and cs3d_load_solution
 * form it from the new state. */
int cs3d_get_conserved(cs3d_handle *h, double *const host_out[5]);
int cs3d_set_conserved(cs3d_handle *h, const double *const host_in[5]);
/* Device pointer of a field (XYZ layout, FP64), valid until destroy. */
int cs3d_field_ptr(cs3d_handle *h, int field, double **dev_ptr);

/* Scalars: time step dt, simulated time, time-step counter
 * (CSolver_AWS.hpp:28-31, TimeStepping.hpp:15). */
int cs3d_get_scalars(cs3d_handle *h, double *dt, double *time, int *time_step);
/* The CUDA stream the handle launches on (a cudaStream_t). */
int cs3d_get_stream(cs3d_handle *h, void **stream);
/* Number of kernels the handle has launched so far. */
int cs3d_launch_count(cs3d_handle *h, long long *count);

/* Options (value 0 = off, the default):
 *  CS3D_OPT_STORE_INCREMENTS  keep the stage increments dt*RHS (rhok2..rhoEk2,
 *                             CSolver_AWS.cpp:1246-1504) in device memory;
 *  CS3D_OPT_STORE_DIAGNOSTICS keep Uz, Vz, Wz of the last stage so that
 *                             cs3d_tgv_quantities can run. */
#define CS3D_OPT_STORE_INCREMENTS  1
#define CS3D_OPT_STORE_DIAGNOSTICS 2
#define CS3D_OPT_KERNEL_TIMING     3  /* bracket every launch with CUDA events */
#define CS3D_OPT_ADJ_RECOMPUTE     4  /* adjoint: recompute each step's stages (see below) */
int cs3d_set_option(cs3d_handle *h, int option, int value);

/* Kernel classes of cs3d_kernel_times. */
#define CS3D_K_SWEEP_X  0
#define CS3D_K_SWEEP_Y  1
#define CS3D_K_SWEEP_Z  2   /* z sweep + RHS + RK update */
#define CS3D_K_FILTER   3
#define CS3D_K_BOUNDARY 4
#define CS3D_K_CFL      5
#define CS3D_K_SPONGE   6
#define CS3D_K_OTHER    7
#define CS3D_NUM_KERNEL_CLASSES 8
/* Accumulated device time (ms, from CUDA events on the handle's stream) and
 * launch count per kernel class while CS3D_OPT_KERNEL_TIMING was on; waits
 * for the recorded work.  reset != 0 clears the totals afterwards.  No
 * counterpart in the reference (its useTiming flag prints host wall time per
 * phase, CSolver_AWS.cpp:1237-1240). */
int cs3d_kernel_times(cs3d_handle *h, double *ms, long long *count, int n, int reset);

/* ---- single operators on device arrays --------------------------------
 * Replace Derivatives::calc1stDerivField / calc2ndDerivField
 * (Derivatives.hpp:167-168, Derivatives.cpp:3-96) and Filter::filterField
 * (Filter.hpp:115, Filter.cpp:129-171).  As in the reference, `in` holds the
 * field in the direction's contiguous layout (DIRX: XYZ, DIRY: YZX,
 * DIRZ: ZXY, Macros.hpp:8-10): lines of length N_dir, one after another.
 * FP64 in and out; `in` and `out` must not overlap. */
int cs3d_deriv1(cs3d_handle *h, int dir, const double *in_dev, double *out_dev);
int cs3d_deriv2(cs3d_handle *h, int dir, const double *in_dev, double *out_dev);
int cs3d_filter(cs3d_handle *h, int dir, const double *in_dev, double *out_dev);

/* ---- operator-only handles ----------------------------------------------
 * One direction's three compact operators with no solver state: replaces
 * `new Derivatives(dom, bcType, dir)` (Derivatives.hpp:54-161) and
 * `new Filter(alphaF, dom, bcType, dir)` (Filter.hpp:31-110), which build
 * only the tridiagonal factors of their direction.  cs3d_op_create reads
 * Nx, Ny, Nz, Lx, Ly, Lz, bc_type[dir] and alphaF from cfg; it allocates the
 * operators' factors only (a few kB).  Fields are in the direction's
 * contiguous layout (DIRX: XYZ, DIRY: YZX, DIRZ: ZXY, Macros.hpp:8-10).
 *   cs3d_op_apply       device arrays, queued on the handle's stream
 *                       (cs3d_op_get_stream); in and out must not overlap;
 *   cs3d_op_apply_host  host arrays, synchronous, as the reference's
 *                       calc1stDerivField(in, out) / filterField(in, out):
 *                       the first call allocates 2*Nx*Ny*Nz doubles of device
 *                       staging, kept until cs3d_op_destroy. */
#define CS3D_OP_DERIV1 1  /* Derivatives::calc1stDerivField (Derivatives.cpp:3-49)  */
#define CS3D_OP_DERIV2 2  /* Derivatives::calc2ndDerivField (Derivatives.cpp:51-96) */
#define CS3D_OP_FILTER 3  /* Filter::filterField (Filter.cpp:129-171)               */
typedef struct cs3d_op cs3d_op;
int cs3d_op_create(const cs3d_config *cfg, int dir, cs3d_op **out);
int cs3d_op_destroy(cs3d_op *op);
int cs3d_op_apply(cs3d_op *op, int kind, const double *in_dev, double *out_dev);
int cs3d_op_apply_host(cs3d_op *op, int kind, const double *in_host, double *out_host);
int cs3d_op_get_stream(cs3d_op *op, void **stream);

/* Kinetic energy and dissipation diagnostics of the Taylor-Green case,
 * the columns of calcTaylorGreenQuantities (CSolver_AWS.cpp:2175-2257):
 * out[0..6] = time, KEsum, dissSum, enstrophySum, enstrophy*2mu, meanMu,
 * dilprime.  Derivatives are those of the last stage, as in the reference;
 * requires CS3D_OPT_STORE_DIAGNOSTICS to have been on during that stage. */
int cs3d_tgv_quantities(cs3d_handle *h, double out[7]);

/* calcTurbulenceQuantities (CSolver_AWS.cpp:2033-2173): out[0..10] = the
 * turbdata.out row -- time, tau, taylorReyn3, turbMach, meanTurbDiss, uprime,
 * kolNu, rhoprime, dilprime, vortprime, meanKineticEng.  Derivatives of the
 * last stage as in the reference; requires CS3D_OPT_STORE_DIAGNOSTICS. */
int cs3d_turbulence_quantities(cs3d_handle *h, double out[11]);

/* shearLayerInfoCalc (CSolver_AWS.cpp:2259-2456): per y plane j, x-z means
 * and second moments of rho, U, V, W, p, T of the current state; out holds
 * 17*Ny doubles, out[k*Ny + j] with k = 0 rhoAvg, 1 uAvg, 2 vAvg, 3 wAvg,
 * 4 pAvg, 5 tAvg, 6 rhoprime2, 7 uprime2, 8 vprime2, 9 wprime2, 10 pprime2,
 * 11 tprime2, 12 uvprime, 13 uwprime and 14 vwprime as the reference writes
 * them (it adds the v'w' sum into uwprime and leaves vwprime 0, :2317-2318),
 * 15 u'w' and 16 v'w' each on its own.  The reference evaluates it in
 * postStep before the sponge update: call it between the last cs3d_sub_step
 * and cs3d_post_step to see the same state; it runs on every call (the
 * reference only on steps that are multiples of 25). */
int cs3d_shear_layer_info(cs3d_handle *h, double *out);

/* AeroOptics::computeAO (AeroOptics.cpp:3-93, Utils.cpp:242-331): for
 * num_angles beam angles 0 .. max_angle degrees (the reference uses 5 and
 * 70) and every x-z position, the trapezoidal integral of the density along
 * a ray from y = 0.2 Ly to 0.8 Ly tilted by the angle in x (periodic in x),
 * trilinear interpolation at spacing about min(dx, dy, dz).
 * opl[ap*Nx*Nz + k*Nx + i] (the contents of the reference's <angle>.OPL
 * rows).  The density is that of the current state q1; the reference
 * integrates rho2, which equals it on steps without filtering and holds
 * filterConservedData's transposition scratch after filtered steps
 * (CSolver_AWS.cpp:1697-1710). */
int cs3d_aero_optics(cs3d_handle *h, int num_angles, double max_angle, double *opl);

/* The post-processor's vorticity magnitude and Q-criterion
 * (PostProcess.cpp:190-310) for the current state q1 (load a dump with
 * cs3d_load_solution first to post-process one): U = rhoU/rho, ..., the nine
 * first derivatives with the solver's FP64 compact operators, then per point
 * vort = |curl u| and qcrit = |W|^2/2 - |S|^2/2 (S, W: symmetric and
 * antisymmetric parts of grad u).  vort and qcrit: npts host doubles each. */
int cs3d_vorticity_q(cs3d_handle *h, double *vort, double *qcrit);

/* ---- restart files ------------------------------------------------------
 * dumpSolution's format (CSolver_AWS.cpp:2493-2535): the conserved state q1
 * as five raw FP64 files in XYZ order with no header, named
 * <prefix>rho.out.<step>, rhoU, rhoV, rhoW, rhoE (prefix may be a directory
 * ending in '/', or ""); <step> is the solver's step count.
 * cs3d_load_solution reads such files (the reference's own or ours) into q1,
 * sets the step count and the time (the format stores neither; pass the
 * time the run had), and prepares the handle as cs3d_set_initial_conditions
 * does.  In the FP64 form without SPONGE faces or bands the run then
 * continues bit for bit as if it had not stopped; otherwise the sponge
 * averages restart from the loaded state and the mixed form's filter
 * reference values are the loaded state's field means. */
int cs3d_dump_solution(cs3d_handle *h, const char *prefix);
int cs3d_load_solution(cs3d_handle *h, const char *prefix, int time_step, double time);

/* ---- discrete adjoint of the time steps --------------------------------
 * No counterpart in the reference.  Gradient of an objective J of the state
 * after n steps with respect to the state before them, by the transposed
 * (discrete adjoint) step: filter^T, then the RK stages in reverse,
 * each J^T lam of the stage right-hand side through the transposed compact
 * operators (D1^T = -D1, D2^T = D2, F^T = F on periodic grids), the
 * generated pointwise adjoint of the flux and viscous terms and the chain
 * rule through the ideal-gas primitives.  Scope: periodic boundaries, RK4
 * or TVD-RK3, and a fixed time step (cfg.dt_fixed > 0).  On a CS3D_FP64 handle every
 * operation is FP64; on a CS3D_FP32_MIXED handle the stage Jacobians are
 * transposed in FP32 at the FP32 stage inputs of the mixed forward, while
 * the adjoint state, the RK combination and the filter transpose are FP64.
 *
 * cs3d_adjoint_record runs n steps from the current state, keeping the state
 * at every checkpoint_every-th step (0: ceil(sqrt(n))); memory is
 * (n/checkpoint_every + checkpoint_every) states plus a workspace of about
 * 150 fields.  cs3d_adjoint_backward replays each segment from its
 * checkpoint and takes its steps back.  Where it fits in half of the free
 * device memory at record time, the replay keeps the stage tapes and stage
 * inputs of the whole segment (212 work-precision fields per step, e.g.
 * 3.5 GB per step at 128^3 FP64), so that no step runs forward twice; else,
 * or with CS3D_OPT_ADJ_RECOMPUTE on when cs3d_adjoint_record is called, each
 * step's stages run again just before that step is taken back.  Both give the
 * same bits.  cs3d_adjoint_backward writes dJ/dq0 to grad (5*npts, field-major rho, rhoU, rhoV, rhoW,
 * rhoE) and returns the solver to the recorded final state.  objective
 * CS3D_ADJ_KE_MEAN: J = mean over points of rho |u|^2 / 2 of the final
 * state (returned in *J); CS3D_ADJ_SEED: seed = dJ/dq of the final state
 * (5*npts host doubles). */
#define CS3D_ADJ_SEED     0
#define CS3D_ADJ_KE_MEAN  1
int cs3d_adjoint_record(cs3d_handle *h, int nsteps, int checkpoint_every);
int cs3d_adjoint_backward(cs3d_handle *h, int objective, const double *seed, double *grad, double *J);

/* Building blocks of the adjoint, on a state q given on the host (5*npts):
 * R(q), the stage right-hand side evaluated from its 48 pointwise inputs
 * (unfused: primitives, fluxes and derivative fields stored, then combined),
 * and out = (dR/dq)^T lam. */
int cs3d_rhs_eval(cs3d_handle *h, const double *q, double *R);
int cs3d_rhs_vjp(cs3d_handle *h, const double *q, const double *lam, double *out);

/* ---- allocation-free kinetic energy -------------------------------------
 * No counterpart in the reference.  The KEsum column of
 * cs3d_tgv_quantities (sum over points of rho |u|^2 / 2, CSolver_AWS.cpp:
 * 2175-2236) from four FP64 device arrays of npts points, without a handle.
 * For callers that may not allocate device memory: code whose device memory
 * is all owned by another allocator (a caching pool), or that must not pay
 * the device-wide synchronisation of cudaMalloc/cudaFree, or that has no
 * solver handle (cs3d_create allocates).  This call allocates nothing, on the
 * device or the host: its 1025 doubles (8200 bytes) of partial sums live in a
 * fixed static device array.  The arrays must be device memory of the
 * current device; the kernels run on `stream` (a cudaStream_t, NULL for the
 * default stream) and the call returns after the result is in *ke.
 * Every call looks up the static array's address on the current device
 * (cudaGetSymbolAddress), so a device reset between calls does no harm; the
 * first call on a device may load the library's device code, so make it
 * before any stream capture starts.  Nothing has to be zeroed beforehand.
 * Two calls that overlap in time on one device share the array and race.
 * npts must be 1 .. 2^31-1 (CS3D_ERR_SHAPE otherwise). */
int cs3d_kinetic_energy_noalloc(const double *rho_dev, const double *rhoU_dev, const double *rhoV_dev,
                                const double *rhoW_dev, long long npts, void *stream, double *ke);

#ifdef __cplusplus
}
#endif
#endif /* CS3D_H */
