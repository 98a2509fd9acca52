// tgv_main.cpp -- a driver written the way the reference's case drivers are
// (3DCompact.cpp:23-259, taylorgreen_vortex/taylorgreen_run128/3DCompact.cpp),
// with CSolver_AWS replaced by CSolver_GB300.  Runs the Taylor-Green vortex
// and prints the kinetic energy after the last step.
//
//   tgv_main [N=32] [steps=5] [precision: 0 FP64, 1 FP32-mixed]
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "cs3d_solver.hpp"

using namespace cs3d_gb300;

int main(int argc, char **argv) {
    const int N = argc > 1 ? atoi(argv[1]) : 32;
    const int steps = argc > 2 ? atoi(argv[2]) : 5;
    const int precision = argc > 3 ? atoi(argv[3]) : CS3D_FP64;
    const double L = 2.0 * M_PI - (2.0 * M_PI / (double)N);
    Domain *dom = new Domain(N, N, N, L, L, L);
    TimeStepping *ts = new TimeStepping(TimeStepping::CONST_CFL, 0.5, steps, 1e300, 1, 1, 1 << 30);
    BC *bc = new BC(BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC, BC::PERIODIC_SOLVE, BC::PERIODIC,
                    BC::PERIODIC, BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC);
    const double gamma = 1.4, p0 = 1.0 / (gamma * 0.01);
    const double mu_ref = 1.0 / (1600.0 * std::pow(p0 / (1.0 / gamma), 0.76));
    CSolver_GB300 *cs;
    try {
        cs = new CSolver_GB300(dom, bc, ts, 0.49, mu_ref, 16, false, CS3D_RK4, precision);
    } catch (const Error &e) {
        fprintf(stderr, "tgv_main: %s\n", e.what());
        return 2;
    }
    AbstractRK_GB300 *rk = new RK4(cs);
    for (int k = 0; k < N; k++)
        for (int j = 0; j < N; j++)
            for (int i = 0; i < N; i++) {
                const int ii = k * N * N + j * N + i;
                const double x = dom->x[i], y = dom->y[j], z = dom->z[k];
                cs->U0[ii] = std::sin(x) * std::cos(y) * std::cos(z);
                cs->V0[ii] = -std::cos(x) * std::sin(y) * std::cos(z);
                cs->W0[ii] = 0.0;
                cs->rho0[ii] = 1.0;
                cs->p0[ii] = p0 + (1.0 / 16.0) * (std::cos(x * 2.0) + std::cos(y * 2.0)) * (std::cos(z * 2.0) + 2.0);
            }
    try {
        rk->executeSolverLoop();
        cs->syncToHost();
    } catch (const Error &e) {
        fprintf(stderr, "tgv_main: %s\n", e.what());
        return 3;
    }
    double ke = 0.0;
    for (int i = 0; i < dom->N; i++)
        ke += 0.5 * (cs->rhoU1[i] * cs->rhoU1[i] + cs->rhoV1[i] * cs->rhoV1[i] + cs->rhoW1[i] * cs->rhoW1[i]) /
              cs->rho1[i];
    printf("steps %d time %.17g dt %.17g KE %.17g\n", cs->timeStep, cs->time, ts->dt, ke);
    delete rk;
    delete cs;
    return 0;
}
