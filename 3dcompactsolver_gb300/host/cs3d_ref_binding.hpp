// cs3d_ref_binding.hpp -- the GB300 stage path behind the reference's own
// C++ interfaces.  Compile with the reference's headers on the include path
// (AbstractCSolver.hpp, RK4.hpp, TVDRK3.hpp, Domain.hpp, BC.hpp,
// TimeStepping.hpp and what they include) and link libcs3d_gb300.so plus the
// reference's Utils.cpp (RK4.hpp / TVDRK3.hpp call its tic/toc).
//
//   cs3d_ref::CSolver_GB300 : public AbstractCSolver   (AbstractCSolver.hpp:9-45)
//       constructor as CSolver_AWS(dom, bc, ts, alphaF, mu_ref, blocksize,
//       useTiming) (CSolver_AWS.hpp:119), plus the integrator and precision
//   cs3d_ref::RK4_GB300    : public RK4     (RK4.hpp:9-33)
//   cs3d_ref::TVDRK3_GB300 : public TVDRK3  (TVDRK3.hpp:7-36)
//       override updateConservedData() only, so the reference's unmodified
//       executeSolverLoop() (RK4.hpp:120-170, TVDRK3.hpp:98-139) drives the GPU
//   cs3d_ref::Derivatives_GB300(dom, bcType, dir)   calc1stDerivField /
//   cs3d_ref::Filter_GB300(alphaF, dom, bcType, dir) calc2ndDerivField /
//       filterField on host arrays, same signatures as Derivatives.hpp:167-168
//       and Filter.hpp:115 (those methods are not virtual, so these are
//       separate classes with the same interface, not subclasses)
//
// Call mapping of one RK stage (the reference's loop calls the five in this
// order): preSubStep() nothing; solveEqnSet() issues the whole stage on the
// GPU -- walls, derivatives, right-hand side, boundary fix-up, the RK update
// and, on the last stage, the filter (cs3d_sub_step); postSubStep() nothing;
// RK*_GB300::updateConservedData() nothing (done by the stage); updateData()
// nothing.  preStep() is calcDtFromCFL (cs3d_pre_step), postStep() is
// updateSponge (cs3d_post_step) plus the reference's checkSolution /
// dumpSolution / checkEnd cadence.
//
// State: the public arrays rho1..rhoEk2 of AbstractCSolver are host mirrors
// of the device state.  syncToHost() fills q1, qk and q2 (rho1.., rhok..,
// rho2..); it runs after setInitialConditions(), on every checkStep-th step
// (when the reference's checkSolution reads them) and when the run ends.
// syncToDevice() writes q1 back after the case program has changed it.  rho0..W0 are
// allocated by initializeSolverData() for the case program to fill and freed by
// setInitialConditions(), as the reference does (CSolver_AWS.cpp:124-128,
// 219-224).  derivX..filtZ stay null: the reference's CPU operators are not
// built; use Derivatives_GB300 / Filter_GB300.  Errors throw
// cs3d_ref::Error with the C ABI status code (the reference has no error
// reporting).
#pragma once
#include <cstring>
#include <stdexcept>
#include <string>

#include "AbstractCSolver.hpp"
#include "BC.hpp"
#include "Domain.hpp"
#include "RK4.hpp"
#include "TVDRK3.hpp"
#include "TimeStepping.hpp"
#include "cs3d.h"

namespace cs3d_ref {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const char *what) {
    if (rc != CS3D_OK) throw Error(rc, std::string(what) + ": " + cs3d_last_error());
}

class CSolver_GB300 : public AbstractCSolver {
  public:
    // CSolver_AWS's own counters (CSolver_AWS.hpp:28-31)
    int timeStep = 0;
    double time = 0.0;
    double alphaF, mu_ref;
    int blocksize;
    int rk, precision, nstages;
    int N = 0;
    cs3d_handle *h = nullptr;
    cs3d_config cfg;
    // dumpSolution's files (CSolver_AWS.cpp:2493-2535) go to dumpPrefix
    // ("" = the working directory, as the reference writes them)
    bool writeDumps = true;
    std::string dumpPrefix;

    CSolver_GB300(Domain *dom_, BC *bc_, TimeStepping *ts_, double alphaF_, double mu_ref_, int blocksize_,
                  bool useTiming_, int rk_ = CS3D_RK4, int precision_ = CS3D_FP64)
        : alphaF(alphaF_), mu_ref(mu_ref_), blocksize(blocksize_), rk(rk_), precision(precision_),
          nstages(rk_ == CS3D_TVDRK3 ? 3 : 4) {
        dom = dom_;
        bc = bc_;
        ts = ts_;
        useTiming = useTiming_;
        rkStep = 1;
        rkLast = false;
        endFlag = false;
        ig = new IdealGas(dom, mu_ref);
        derivX = derivY = derivZ = nullptr;
        filtX = filtY = filtZ = nullptr;
        rho0 = p0 = U0 = V0 = W0 = nullptr;
        double **st[20] = {&rho1, &rhoU1, &rhoV1, &rhoW1, &rhoE1, &rhok, &rhoUk, &rhoVk, &rhoWk, &rhoEk,
                           &rho2, &rhoU2, &rhoV2, &rhoW2, &rhoE2, &rhok2, &rhoUk2, &rhoVk2, &rhoWk2, &rhoEk2};
        for (auto p : st) *p = nullptr;
        try {
            initializeSolverData();
        } catch (...) {
            release();
            throw;
        }
    }
    CSolver_GB300(const CSolver_GB300 &) = delete;
    CSolver_GB300 &operator=(const CSolver_GB300 &) = delete;
    virtual ~CSolver_GB300() { release(); }

    // ---- AbstractCSolver.hpp:36-43 ---------------------------------------
    void initializeSolverData() override {
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
        N = dom->N;
        rho0 = new double[N]; p0 = new double[N];
        U0 = new double[N]; V0 = new double[N]; W0 = new double[N];
        double **st[20] = {&rho1, &rhoU1, &rhoV1, &rhoW1, &rhoE1, &rhok, &rhoUk, &rhoVk, &rhoWk, &rhoEk,
                           &rho2, &rhoU2, &rhoV2, &rhoW2, &rhoE2, &rhok2, &rhoUk2, &rhoVk2, &rhoWk2, &rhoEk2};
        for (auto p : st) *p = new double[N]();
    }
    void setInitialConditions() override {
        check(cs3d_set_initial_conditions(h, rho0, p0, U0, V0, W0), "cs3d_set_initial_conditions");
        double **ic[5] = {&rho0, &p0, &U0, &V0, &W0};
        for (auto p : ic) {
            delete[] *p;
            *p = nullptr;
        }
        syncToHost();
    }
    void preStep() override {
        if (timeStep == 0) dumpSolution();  // CSolver_AWS.cpp:2897-2903
        check(cs3d_pre_step(h), "cs3d_pre_step");
        timeStep++;
    }
    void preSubStep() override {}
    void solveEqnSet() override {
        if (rkLast != (rkStep == nstages))
            throw Error(CS3D_ERR_STATE, "the solver was built for " + std::string(nstages == 4 ? "RK4" : "TVD-RK3") +
                                            ": pair it with the matching RK*_GB300 loop");
        check(cs3d_sub_step(h, rkStep, rkLast ? 1 : 0), "cs3d_sub_step");
    }
    void postSubStep() override {}
    void updateData() override {}
    void postStep() override {
        check(cs3d_post_step(h), "cs3d_post_step");
        if (ts->checkStep > 0 && timeStep % ts->checkStep == 0) syncToHost();
        dumpSolution();
        checkEnd();
    }

    // ---- the rest of CSolver_AWS's postStep cadence ------------------------
    void dumpSolution() {
        if (writeDumps && ts->dumpStep > 0 && timeStep % ts->dumpStep == 0)
            check(cs3d_dump_solution(h, dumpPrefix.c_str()), "cs3d_dump_solution");
    }
    // CSolver_AWS.cpp:2764-2790; `time` is read back only when maxTime can end the run
    void checkEnd() {
        if (ts->maxTime < 1e300) {
            int step = 0;
            check(cs3d_get_scalars(h, &ts->dt, &time, &step), "cs3d_get_scalars");
            if (time >= ts->maxTime) endFlag = true;
        }
        if (timeStep >= ts->maxTimeStep) endFlag = true;
        if (endFlag) syncToHost();
    }

    // ---- host mirrors -------------------------------------------------------
    void syncToHost() {
        double **st = state();
        for (int f = 0; f < 15; f++) check(cs3d_get_field(h, f, st[f]), "cs3d_get_field");
        int step = 0;
        check(cs3d_get_scalars(h, &ts->dt, &time, &step), "cs3d_get_scalars");
    }
    void syncToDevice() {
        double **st = state();
        for (int f = 0; f < 5; f++) check(cs3d_set_field(h, f, st[f]), "cs3d_set_field");
    }

  private:
    void release() {
        cs3d_destroy(h);
        h = nullptr;
        double *ic[5] = {rho0, p0, U0, V0, W0};
        for (auto p : ic) delete[] p;
        double **st = state();
        for (int f = 0; f < 20; f++) delete[] st[f];
        delete ig;
        ig = nullptr;
    }
    double *st_[20];
    double **state() {
        double *v[20] = {rho1, rhoU1, rhoV1, rhoW1, rhoE1, rhok, rhoUk, rhoVk, rhoWk, rhoEk,
                         rho2, rhoU2, rhoV2, rhoW2, rhoE2, rhok2, rhoUk2, rhoVk2, rhoWk2, rhoEk2};
        std::memcpy(st_, v, sizeof(v));
        return st_;
    }
};

// The reference's integrators with the host-side stage combination taken
// out: the stage update runs on the GPU inside CSolver_GB300::solveEqnSet.
class RK4_GB300 : public RK4 {
  public:
    explicit RK4_GB300(AbstractCSolver *cs_) : RK4(cs_) {}
    void updateConservedData() override {}
};

class TVDRK3_GB300 : public TVDRK3 {
  public:
    explicit TVDRK3_GB300(AbstractCSolver *cs_) : TVDRK3(cs_) {}
    void updateConservedData() override {}
};

// Derivatives(dom, bcType, dir) / Filter(alphaF, dom, bcType, dir) with the
// reference's method signatures (host arrays in the direction's contiguous
// layout, synchronous) on an operator-only handle; *_dev forms take device
// arrays and queue on stream().
class Derivatives_GB300 {
  public:
    cs3d_op *op = nullptr;
    Derivatives::Direct currentDir;
    Derivatives_GB300(Domain *dom, BC::BCType bcType, Derivatives::Direct dir, double alphaF = 0.49)
        : currentDir(dir) {
        cs3d_config c;
        std::memset(&c, 0, sizeof(c));
        c.Nx = dom->Nx; c.Ny = dom->Ny; c.Nz = dom->Nz;
        c.Lx = dom->Lx; c.Ly = dom->Ly; c.Lz = dom->Lz;
        c.bc_type[(int)dir] = (int)bcType;
        c.alphaF = alphaF;
        check(cs3d_op_create(&c, (int)dir, &op), "cs3d_op_create");
    }
    Derivatives_GB300(const Derivatives_GB300 &) = delete;
    Derivatives_GB300 &operator=(const Derivatives_GB300 &) = delete;
    virtual ~Derivatives_GB300() { cs3d_op_destroy(op); }
    void calc1stDerivField(double *dataIn, double *dataOut) {
        check(cs3d_op_apply_host(op, CS3D_OP_DERIV1, dataIn, dataOut), "calc1stDerivField");
    }
    void calc2ndDerivField(double *dataIn, double *dataOut) {
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
    Filter_GB300(double alphaF, Domain *dom, BC::BCType bcType, Derivatives::Direct dir)
        : Derivatives_GB300(dom, bcType, dir, alphaF) {}
    void filterField(double *dataIn, double *dataOut) {
        check(cs3d_op_apply_host(op, CS3D_OP_FILTER, dataIn, dataOut), "filterField");
    }
    void filterField_dev(const double *in_dev, double *out_dev) {
        check(cs3d_op_apply(op, CS3D_OP_FILTER, in_dev, out_dev), "cs3d_op_apply");
    }
};

}  // namespace cs3d_ref
