// cs3d_solver.hpp -- C++ host classes over the C ABI of include/cs3d.h that
// keep the names and call sequence of the reference's interfaces for the
// per-stage path:
//
//   Domain(Nx, Ny, Nz, Lx, Ly, Lz)                           Domain.hpp:16
//   BC(bcXType, bcX0, bcX1, bcYType, ..., bcZ1)              BC.hpp:16
//   TimeStepping(type, CFL, maxTimeStep, maxTime, filterStep, checkStep, dumpStep)
//                                                            TimeStepping.hpp:20
//   CSolver_GB300(dom, bc, ts, alphaF, mu_ref, blocksize, useTiming)
//       the eight virtuals of AbstractCSolver.hpp:36-43 and its public
//       state (rkStep, rkLast, endFlag, rho0..W0, rho1..rhoE2)
//   RK4(cs), TVDRK3(cs): executeSolverLoop(), updateConservedData()
//                                                            AbstractRK.hpp:13-14
//   Derivatives_GB300(dom, bcType, dir).calc1stDerivField / calc2ndDerivField
//   Filter_GB300(alphaF, dom, bcType, dir).filterField      (host arrays, as
//       the reference's; *_dev forms on device arrays)
//
// These classes stand alone (no reference headers needed).  For the
// reference's own AbstractCSolver / RK4 / TVDRK3 classes see
// cs3d_ref_binding.hpp.
//
// The five stage virtuals of the reference (preSubStep, solveEqnSet,
// postSubStep, updateConservedData, updateData) run on the GPU as one fused
// launch sequence, issued by updateData(), the last of them.  The public
// state arrays rho1..rhoE2 are host mirrors filled by syncToHost(); writes to
// them reach the device through syncToDevice().  Errors throw cs3d_gb300::Error
// carrying the ABI status code.
#pragma once
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cs3d.h"

namespace cs3d_gb300 {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const char *what) {
    if (rc != CS3D_OK) throw Error(rc, std::string(what) + ": " + cs3d_last_error());
}

class Domain {
  public:
    int Nx, Ny, Nz, N;
    double Lx, Ly, Lz, dx, dy, dz;
    std::vector<double> x, y, z;
    Domain(int Nx_, int Ny_, int Nz_, double Lx_, double Ly_, double Lz_)
        : Nx(Nx_), Ny(Ny_), Nz(Nz_), N(Nx_ * Ny_ * Nz_), Lx(Lx_), Ly(Ly_), Lz(Lz_) {
        // x_i = i*L/(N-1) (Domain.hpp:31-41)
        for (int i = 0; i < Nx; i++) x.push_back((((double)i) / ((double)Nx - 1.0)) * Lx);
        for (int j = 0; j < Ny; j++) y.push_back((((double)j) / ((double)Ny - 1.0)) * Ly);
        for (int k = 0; k < Nz; k++) z.push_back((((double)k) / ((double)Nz - 1.0)) * Lz);
        dx = x[1] - x[0];
        dy = y[1] - y[0];
        dz = z[1] - z[0];
    }
};

class BC {
  public:
    enum BCType { PERIODIC_SOLVE = CS3D_PERIODIC_SOLVE, DIRICHLET_SOLVE = CS3D_DIRICHLET_SOLVE };
    enum BCKind {
        PERIODIC = CS3D_PERIODIC,
        SPONGE = CS3D_SPONGE,
        ADIABATIC_WALL = CS3D_ADIABATIC_WALL,
        MOVING_ADIABATIC_WALL = CS3D_MOVING_ADIABATIC_WALL,
        INLET = CS3D_INLET
    };
    BCType bcXType, bcYType, bcZType;
    BCKind bcX0, bcX1, bcY0, bcY1, bcZ0, bcZ1;
    BC(BCType xt, BCKind x0, BCKind x1, BCType yt, BCKind y0, BCKind y1, BCType zt, BCKind z0, BCKind z1)
        : bcXType(xt), bcYType(yt), bcZType(zt), bcX0(x0), bcX1(x1), bcY0(y0), bcY1(y1), bcZ0(z0), bcZ1(z1) {}
};

class TimeStepping {
  public:
    enum TimeSteppingType { CONST_DT, CONST_CFL };
    TimeSteppingType timeSteppingType;
    double CFL, dt = 0.0, maxTime;
    int maxTimeStep, filterStep, checkStep, dumpStep;
    TimeStepping(TimeSteppingType t, double CFL_, int maxTimeStep_, double maxTime_, int filterStep_,
                 int checkStep_, int dumpStep_)
        : timeSteppingType(t), CFL(CFL_), maxTime(maxTime_), maxTimeStep(maxTimeStep_), filterStep(filterStep_),
          checkStep(checkStep_), dumpStep(dumpStep_) {}
};

// The drop-in for CSolver_AWS (CSolver_AWS.hpp:119).
class CSolver_GB300 {
  public:
    int rkStep = 1;
    bool rkLast = false, endFlag = false, useTiming = false;
    // initial conditions, written by the case program before setInitialConditions()
    std::vector<double> rho0v, p0v, U0v, V0v, W0v;
    double *rho0, *p0, *U0, *V0, *W0;
    // host mirrors of the conserved state (AbstractCSolver.hpp:19-26)
    std::vector<double> mirror[20];
    double *rho1, *rhoU1, *rhoV1, *rhoW1, *rhoE1;
    double *rhok, *rhoUk, *rhoVk, *rhoWk, *rhoEk;
    double *rho2, *rhoU2, *rhoV2, *rhoW2, *rhoE2;
    double *rhok2, *rhoUk2, *rhoVk2, *rhoWk2, *rhoEk2;
    Domain *dom;
    BC *bc;
    TimeStepping *ts;
    int timeStep = 0;
    double time = 0.0;
    cs3d_handle *h = nullptr;
    cs3d_config cfg;

    CSolver_GB300(Domain *dom_, BC *bc_, TimeStepping *ts_, double alphaF, double mu_ref, int blocksize,
                  bool useTiming_, int rk = CS3D_RK4, int precision = CS3D_FP64)
        : useTiming(useTiming_), dom(dom_), bc(bc_), ts(ts_) {
        (void)blocksize;  // the reference's transpose block size; no transposes here
        std::memset(&cfg, 0, sizeof(cfg));
        cfg.Nx = dom->Nx; cfg.Ny = dom->Ny; cfg.Nz = dom->Nz;
        cfg.Lx = dom->Lx; cfg.Ly = dom->Ly; cfg.Lz = dom->Lz;
        cfg.bc_type[0] = bc->bcXType; cfg.bc_type[1] = bc->bcYType; cfg.bc_type[2] = bc->bcZType;
        cfg.bc_kind[0] = bc->bcX0; cfg.bc_kind[1] = bc->bcX1; cfg.bc_kind[2] = bc->bcY0;
        cfg.bc_kind[3] = bc->bcY1; cfg.bc_kind[4] = bc->bcZ0; cfg.bc_kind[5] = bc->bcZ1;
        cfg.alphaF = alphaF;
        cfg.mu_ref = mu_ref;
        cfg.CFL = ts->CFL;
        cfg.filter_step = ts->filterStep;
        cfg.rk = rk;
        cfg.precision = precision;
        cfg.sponge_mode = CS3D_SPONGE_REFERENCE;
        check(cs3d_create(&cfg, &h), "cs3d_create");
        const size_t n = (size_t)dom->N;
        rho0v.assign(n, 1.0); p0v.assign(n, 1.0); U0v.assign(n, 0.0); V0v.assign(n, 0.0); W0v.assign(n, 0.0);
        rho0 = rho0v.data(); p0 = p0v.data(); U0 = U0v.data(); V0 = V0v.data(); W0 = W0v.data();
        for (auto &m : mirror) m.assign(n, 0.0);
        double **ptrs[20] = {&rho1, &rhoU1, &rhoV1, &rhoW1, &rhoE1, &rhok, &rhoUk, &rhoVk, &rhoWk, &rhoEk,
                             &rho2, &rhoU2, &rhoV2, &rhoW2, &rhoE2, &rhok2, &rhoUk2, &rhoVk2, &rhoWk2, &rhoEk2};
        for (int f = 0; f < 20; f++) *ptrs[f] = mirror[f].data();
    }
    CSolver_GB300(const CSolver_GB300 &) = delete;
    CSolver_GB300 &operator=(const CSolver_GB300 &) = delete;
    virtual ~CSolver_GB300() { cs3d_destroy(h); }

    // AbstractCSolver.hpp:36-43
    virtual void initializeSolverData() {}  // device arrays are allocated by the constructor
    virtual void setInitialConditions() {
        check(cs3d_set_initial_conditions(h, rho0, p0, U0, V0, W0), "cs3d_set_initial_conditions");
    }
    virtual void preStep() {
        check(cs3d_pre_step(h), "cs3d_pre_step");
        timeStep++;
    }
    virtual void preSubStep() {}
    virtual void solveEqnSet() {}
    virtual void postSubStep() {}
    virtual void updateData() { check(cs3d_sub_step(h, rkStep, rkLast ? 1 : 0), "cs3d_sub_step"); }
    virtual void postStep() {
        check(cs3d_post_step(h), "cs3d_post_step");
        // checkEnd (CSolver_AWS.cpp:2764-2790) without the dump
        if (timeStep >= ts->maxTimeStep) endFlag = true;
        if (!endFlag && ts->maxTime < 1e300) {
            int ts_ = 0;
            check(cs3d_get_scalars(h, &ts->dt, &time, &ts_), "cs3d_get_scalars");
            if (time >= ts->maxTime) endFlag = true;
        }
    }

    // Copy the device state into the public host arrays (q1, qk, q2).
    void syncToHost() {
        for (int f = 0; f < 15; f++) check(cs3d_get_field(h, f, mirror[f].data()), "cs3d_get_field");
        int ts_ = 0;
        check(cs3d_get_scalars(h, &ts->dt, &time, &ts_), "cs3d_get_scalars");
    }
    // Copy the public host arrays of q1 back to the device.
    void syncToDevice() {
        for (int f = 0; f < 5; f++) check(cs3d_set_field(h, f, mirror[f].data()), "cs3d_set_field");
    }
};

// AbstractRK (AbstractRK.hpp:6-16) and its two implementations.
class AbstractRK_GB300 {
  public:
    CSolver_GB300 *cs;
    int nstages;
    AbstractRK_GB300(CSolver_GB300 *cs_, int n) : cs(cs_), nstages(n) {}
    virtual ~AbstractRK_GB300() {}
    virtual void updateConservedData() {}  // fused into the stage issued by updateData()
    // RK4.hpp:120-170 / TVDRK3.hpp:98-139
    virtual void executeSolverLoop() {
        cs->setInitialConditions();
        while (!cs->endFlag) {
            cs->rkLast = false;
            cs->preStep();
            for (int s = 1; s <= nstages; s++) {
                cs->rkStep = s;
                cs->rkLast = s == nstages;
                cs->preSubStep();
                cs->solveEqnSet();
                cs->postSubStep();
                updateConservedData();
                cs->updateData();
            }
            cs->postStep();
        }
    }
};

class RK4 : public AbstractRK_GB300 {
  public:
    explicit RK4(CSolver_GB300 *cs_) : AbstractRK_GB300(cs_, 4) {}
};

class TVDRK3 : public AbstractRK_GB300 {
  public:
    explicit TVDRK3(CSolver_GB300 *cs_) : AbstractRK_GB300(cs_, 3) {}
};

// Derivatives (Derivatives.hpp:54) and Filter (Filter.hpp:31): the three
// operators of one direction on an operator-only handle (cs3d_op_create), no
// solver state.  calc1stDerivField / calc2ndDerivField / filterField take
// host arrays in the direction's contiguous layout and return when the
// result is there, as the reference's do (Derivatives.hpp:167-168,
// Filter.hpp:115); the *_dev forms take device arrays and queue the work on
// the handle's stream (stream()).
class Derivatives_GB300 {
  public:
    enum Direct { DIRX = CS3D_DIRX, DIRY = CS3D_DIRY, DIRZ = CS3D_DIRZ };
    cs3d_op *op = nullptr;
    Direct currentDir;
    Derivatives_GB300(Domain *dom, BC::BCType bcType, Direct dir, double alphaF = 0.49) : currentDir(dir) {
        cs3d_config c;
        std::memset(&c, 0, sizeof(c));
        c.Nx = dom->Nx; c.Ny = dom->Ny; c.Nz = dom->Nz;
        c.Lx = dom->Lx; c.Ly = dom->Ly; c.Lz = dom->Lz;
        c.bc_type[dir] = bcType;
        c.alphaF = alphaF;
        check(cs3d_op_create(&c, dir, &op), "cs3d_op_create");
    }
    Derivatives_GB300(const Derivatives_GB300 &) = delete;
    Derivatives_GB300 &operator=(const Derivatives_GB300 &) = delete;
    virtual ~Derivatives_GB300() { cs3d_op_destroy(op); }
    void calc1stDerivField(const double *dataIn, double *dataOut) {
        check(cs3d_op_apply_host(op, CS3D_OP_DERIV1, dataIn, dataOut), "calc1stDerivField");
    }
    void calc2ndDerivField(const double *dataIn, double *dataOut) {
        check(cs3d_op_apply_host(op, CS3D_OP_DERIV2, dataIn, dataOut), "calc2ndDerivField");
    }
    void calc1stDerivField_dev(const double *in_dev, double *out_dev) {
        check(cs3d_op_apply(op, CS3D_OP_DERIV1, in_dev, out_dev), "cs3d_op_apply");
    }
    void calc2ndDerivField_dev(const double *in_dev, double *out_dev) {
        check(cs3d_op_apply(op, CS3D_OP_DERIV2, in_dev, out_dev), "cs3d_op_apply");
    }
    void *stream() {
        void *s = nullptr;
        check(cs3d_op_get_stream(op, &s), "cs3d_op_get_stream");
        return s;
    }
};

class Filter_GB300 : public Derivatives_GB300 {
  public:
    Filter_GB300(double alphaF, Domain *dom, BC::BCType bcType, Direct dir)
        : Derivatives_GB300(dom, bcType, dir, alphaF) {}
    void filterField(const double *dataIn, double *dataOut) {
        check(cs3d_op_apply_host(op, CS3D_OP_FILTER, dataIn, dataOut), "filterField");
    }
    void filterField_dev(const double *in_dev, double *out_dev) {
        check(cs3d_op_apply(op, CS3D_OP_FILTER, in_dev, out_dev), "cs3d_op_apply");
    }
};

}  // namespace cs3d_gb300
