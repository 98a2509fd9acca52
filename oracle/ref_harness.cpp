// ref_harness.cpp -- test harness that links the reference's own solver
// sources (Utils.cpp, Derivatives.cpp, Filter.cpp, CSolver_AWS.cpp,
// AeroOptics.cpp, compiled from the reference checkout by oracle/Makefile)
// and exposes them through a small C interface for the parity tests.
//
// TEST INFRASTRUCTURE ONLY: nothing in the product links or loads this.
//
// The stage loop below is the body of RK4::executeSolverLoop
// (RK4.hpp:120-170) / TVDRK3::executeSolverLoop (TVDRK3.hpp:98-139) without
// setInitialConditions and without the file output of preStep/postStep
// (CSolver_AWS.cpp:2897-2946): preStep is reduced to calcDtFromCFL and
// postStep to updateSponge, the two parts that change the solution.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>

#include "Macros.hpp"
#include "Utils.hpp"
#include "BC.hpp"
#include "TimeStepping.hpp"
#include "Domain.hpp"
#include "AbstractCSolver.hpp"
#include "AbstractRK.hpp"
#include "TVDRK3.hpp"
#include "RK4.hpp"
#include "CSolver_AWS.hpp"

#include "../include/cs3d.h"

struct RefHandle {
    Domain *dom;
    BC *bc;
    TimeStepping *ts;
    CSolver_AWS *cs;
    AbstractRK *rk;
    int nstages;
};

// Sponge strength ramp, the formula of SpongeBC.hpp:73 (and its five
// siblings), applied with a zero-initialised sigma: the reference reads the
// freshly allocated sigma inside fmax (SpongeBC.hpp:49,73), which the harness
// makes deterministic by rebuilding sigma here.
static void build_sigma(RefHandle *h, const cs3d_config *c) {
    CSolver_AWS *cs = h->cs;
    Domain *d = h->dom;
    int Nx = d->Nx, Ny = d->Ny, Nz = d->Nz;
    double *sigma = cs->spg->sigma;
    memset(sigma, 0, sizeof(double) * (size_t)Nx * Ny * Nz);
    const double L[3] = {d->Lx, d->Ly, d->Lz};
    const double dflt[3] = {0.25, 0.125, 0.25};
    double *coord[3] = {d->x, d->y, d->z};
    int Nd[3] = {Nx, Ny, Nz};
    for (int f = 0; f < 6; f++) {
        int dir = f / 2, hi = f % 2;
        double band;
        if (c->sponge_mode == CS3D_SPONGE_REFERENCE)
            band = (c->bc_kind[f] == CS3D_SPONGE) ? dflt[dir] * L[dir] : 0.0;
        else
            band = c->sponge_frac[f] * L[dir];
        if (band <= 0.0) continue;
        for (int a = 0; a < Nd[dir]; a++) {
            double xc = coord[dir][a], s;
            if (!hi) { if (!(xc < band)) continue; s = (band - xc) / band; }
            else { if (!(xc > L[dir] - band)) continue; s = (xc - (L[dir] - band)) / band; }
            double val = cs->spg->spongeStrength * (0.068 * pow(s, 2.0) + 0.845 * pow(s, 8.0));
            for (int k = 0; k < Nz; k++)
                for (int j = 0; j < Ny; j++)
                    for (int i = 0; i < Nx; i++) {
                        int idx[3] = {i, j, k};
                        if (idx[dir] != a) continue;
                        int ii = k * Nx * Ny + j * Nx + i;
                        sigma[ii] = fmax(val, sigma[ii]);
                    }
        }
    }
}

static bool any_sponge(const cs3d_config *c) {
    if (c->sponge_mode == CS3D_SPONGE_BANDS) {
        for (int f = 0; f < 6; f++) if (c->sponge_frac[f] > 0.0) return true;
        return false;
    }
    for (int f = 0; f < 6; f++) if (c->bc_kind[f] == CS3D_SPONGE) return true;
    return false;
}

extern "C" {

void *ref_create(const cs3d_config *c) {
    RefHandle *h = new RefHandle();
    h->dom = new Domain(c->Nx, c->Ny, c->Nz, c->Lx, c->Ly, c->Lz);
    h->ts = new TimeStepping(TimeStepping::CONST_CFL, c->CFL, 1 << 30, 1e300, c->filter_step, 1 << 30, 1 << 30);
    h->bc = new BC((BC::BCType)c->bc_type[0], (BC::BCKind)c->bc_kind[0], (BC::BCKind)c->bc_kind[1],
                   (BC::BCType)c->bc_type[1], (BC::BCKind)c->bc_kind[2], (BC::BCKind)c->bc_kind[3],
                   (BC::BCType)c->bc_type[2], (BC::BCKind)c->bc_kind[4], (BC::BCKind)c->bc_kind[5]);
    h->cs = new CSolver_AWS(h->dom, h->bc, h->ts, c->alphaF, c->mu_ref, 16, false);
    // spongeFlag is left uninitialised by the constructor when no face is a
    // sponge (CSolver_AWS.hpp:101,154-159); set it explicitly.
    if (any_sponge(c)) {
        h->cs->spongeFlag = true;
        if (!h->cs->spg) h->cs->spg = new SpongeBC(h->dom, h->cs->ig, h->bc);
        build_sigma(h, c);
    } else {
        h->cs->spongeFlag = false;
    }
    const double *wv = c->wall_vel;
    CSolver_AWS *cs = h->cs;
    cs->X0WallV = wv[0]; cs->X0WallW = wv[1]; cs->X1WallV = wv[2]; cs->X1WallW = wv[3];
    cs->Y0WallU = wv[4]; cs->Y0WallW = wv[5]; cs->Y1WallU = wv[6]; cs->Y1WallW = wv[7];
    cs->Z0WallU = wv[8]; cs->Z0WallV = wv[9]; cs->Z1WallU = wv[10]; cs->Z1WallV = wv[11];
    if (c->rk == CS3D_TVDRK3) { h->rk = new TVDRK3(cs); h->nstages = 3; }
    else { h->rk = new RK4(cs); h->nstages = 4; }
    return h;
}

void ref_set_ic(void *hp, const double *rho0, const double *p0, const double *U0,
                const double *V0, const double *W0) {
    RefHandle *h = (RefHandle *)hp;
    size_t n = (size_t)h->dom->N;
    memcpy(h->cs->rho0, rho0, n * sizeof(double));
    memcpy(h->cs->p0, p0, n * sizeof(double));
    memcpy(h->cs->U0, U0, n * sizeof(double));
    memcpy(h->cs->V0, V0, n * sizeof(double));
    memcpy(h->cs->W0, W0, n * sizeof(double));
    h->cs->setInitialConditions();
}

void ref_pre_step(void *hp) { ((RefHandle *)hp)->cs->calcDtFromCFL(); }

void ref_sub_step(void *hp, int rk_step, int rk_last) {
    RefHandle *h = (RefHandle *)hp;
    CSolver_AWS *cs = h->cs;
    cs->rkStep = rk_step;
    cs->rkLast = rk_last != 0;
    cs->preSubStep();
    cs->solveEqnSet();
    cs->postSubStep();
    h->rk->updateConservedData();
    cs->updateData();
}

void ref_post_step(void *hp) { ((RefHandle *)hp)->cs->updateSponge(); }

void ref_step(void *hp) {
    RefHandle *h = (RefHandle *)hp;
    h->cs->rkLast = false;
    ref_pre_step(hp);
    for (int s = 1; s <= h->nstages; s++) ref_sub_step(hp, s, s == h->nstages);
    ref_post_step(hp);
}

// Field access by the index constants of cs3d.h.
int ref_get_field(void *hp, int f, double *out) {
    RefHandle *h = (RefHandle *)hp;
    CSolver_AWS *cs = h->cs;
    size_t n = (size_t)h->dom->N;
    double *tab[CS3D_NUM_FIELDS] = {
        cs->rho1, cs->rhoU1, cs->rhoV1, cs->rhoW1, cs->rhoE1,
        cs->rhok, cs->rhoUk, cs->rhoVk, cs->rhoWk, cs->rhoEk,
        cs->rho2, cs->rhoU2, cs->rhoV2, cs->rhoW2, cs->rhoE2,
        cs->rhok2, cs->rhoUk2, cs->rhoVk2, cs->rhoWk2, cs->rhoEk2,
        cs->U, cs->V, cs->W, cs->p, cs->T, cs->mu, cs->sos,
        cs->spg ? cs->spg->spongeRhoAvg : 0, cs->spg ? cs->spg->spongeRhoUAvg : 0,
        cs->spg ? cs->spg->spongeRhoVAvg : 0, cs->spg ? cs->spg->spongeRhoWAvg : 0,
        cs->spg ? cs->spg->spongeRhoEAvg : 0, cs->spg ? cs->spg->sigma : 0};
    if (f < 0 || f >= CS3D_NUM_FIELDS || !tab[f]) return 1;
    memcpy(out, tab[f], n * sizeof(double));
    return 0;
}

// Derivative fields of the last stage, by name (CSolver_AWS.hpp:51-72).
int ref_get_named(void *hp, const char *name, double *out) {
    RefHandle *h = (RefHandle *)hp;
    CSolver_AWS *cs = h->cs;
    size_t n = (size_t)h->dom->N;
    struct { const char *nm; double *p; } tab[] = {
        {"Ux", cs->Ux}, {"Uy", cs->Uy}, {"Uz", cs->Uz}, {"Vx", cs->Vx}, {"Vy", cs->Vy}, {"Vz", cs->Vz},
        {"Wx", cs->Wx}, {"Wy", cs->Wy}, {"Wz", cs->Wz}, {"Uxx", cs->Uxx}, {"Uyy", cs->Uyy}, {"Uzz", cs->Uzz},
        {"Vxx", cs->Vxx}, {"Vyy", cs->Vyy}, {"Vzz", cs->Vzz}, {"Wxx", cs->Wxx}, {"Wyy", cs->Wyy},
        {"Wzz", cs->Wzz}, {"Uxy", cs->Uxy}, {"Uxz", cs->Uxz}, {"Vxy", cs->Vxy}, {"Vyz", cs->Vyz},
        {"Wxz", cs->Wxz}, {"Wyz", cs->Wyz}, {"Tx", cs->Tx}, {"Ty", cs->Ty}, {"Tz", cs->Tz},
        {"Txx", cs->Txx}, {"Tyy", cs->Tyy}, {"Tzz", cs->Tzz}, {"Amu", cs->Amu},
        {"contEulerX", cs->contEulerX}, {"contEulerY", cs->contEulerY}, {"contEulerZ", cs->contEulerZ},
        {"engyEulerX", cs->engyEulerX}, {"engyEulerY", cs->engyEulerY}, {"engyEulerZ", cs->engyEulerZ},
    };
    for (auto &e : tab)
        if (!strcmp(e.nm, name)) { memcpy(out, e.p, n * sizeof(double)); return 0; }
    return 1;
}

// The reference's own diagnostics; they write their rows to files in the
// current directory (turbdata.out, rhoprime2.out, ...).  shearLayerInfoCalc
// runs only on steps that are multiples of 25 (CSolver_AWS.cpp:2265), so the
// step counter is set to 0 around the call.
void ref_turbulence_quantities(void *hp) {
    RefHandle *h = (RefHandle *)hp;
    h->cs->calcTurbulenceQuantities();
}
void ref_shear_layer_info(void *hp) {
    RefHandle *h = (RefHandle *)hp;
    int ts = h->cs->timeStep;
    h->cs->timeStep = 0;
    h->cs->shearLayerInfoCalc();
    h->cs->timeStep = ts;
}

// dumpSolution writes only on steps that are multiples of dumpStep
// (CSolver_AWS.cpp:2497); dumpStep is set to 1 around the call.
void ref_dump_solution(void *hp) {
    RefHandle *h = (RefHandle *)hp;
    int ds = h->ts->dumpStep;
    h->ts->dumpStep = 1;
    h->cs->dumpSolution();
    h->ts->dumpStep = ds;
}

// AeroOptics::computeAO on rho2, the field the solver hands its AeroOptics
// object (CSolver_AWS.hpp:165); it also writes <angle>.OPL files to the
// current directory.
void ref_aero_optics(void *hp, int num_angles, double max_angle, double *out) {
    RefHandle *h = (RefHandle *)hp;
    AeroOptics ao(h->dom, h->cs->ig, h->cs->rho2, h->cs->p, h->cs->T, num_angles, max_angle);
    ao.computeAO();
    memcpy(out, ao.OPL, sizeof(double) * (size_t)num_angles * h->dom->Nx * h->dom->Nz);
    delete[] ao.OPL;
}

void ref_get_scalars(void *hp, double *dt, double *time, int *time_step) {
    RefHandle *h = (RefHandle *)hp;
    *dt = h->ts->dt;
    *time = h->cs->time;
    *time_step = h->cs->timeStep;
}

void ref_destroy(void *hp) {
    // The reference has no destructors and leaks its arrays
    // (CSolver_AWS.cpp:14-189); the harness frees only its own handle.
    delete (RefHandle *)hp;
}

// Single-operator entry: kind 1 = calc1stDerivField, 2 = calc2ndDerivField,
// 3 = Filter::filterField, along direction dir of an Nx x Ny x Nz domain.
void ref_line_op(int kind, int dir, int bc_type, int Nx, int Ny, int Nz, double Lx, double Ly,
                 double Lz, double alphaF, const double *in, double *out) {
    Domain dom(Nx, Ny, Nz, Lx, Ly, Lz);
    size_t n = (size_t)Nx * Ny * Nz;
    double *tin = new double[n];
    memcpy(tin, in, n * sizeof(double));
    if (kind == 3) {
        Filter f(alphaF, &dom, (BC::BCType)bc_type, (Derivatives::Direct)dir);
        f.filterField(tin, out);
    } else {
        Derivatives d(&dom, (BC::BCType)bc_type, (Derivatives::Direct)dir);
        if (kind == 1) d.calc1stDerivField(tin, out);
        else d.calc2ndDerivField(tin, out);
    }
    delete[] tin;
}

}  // extern "C"
