// ref_loop_main.cpp -- TEST DRIVER.  A Taylor-Green run written the way the
// reference's case drivers are (3DCompact.cpp:23-259), with CSolver_AWS
// replaced by cs3d_ref::CSolver_GB300 and RK4 / TVDRK3 by RK4_GB300 /
// TVDRK3_GB300: the reference's own, unmodified executeSolverLoop()
// (RK4.hpp:120-170, TVDRK3.hpp:98-139) drives the stage path.  Also runs
// Derivatives_GB300::calc1stDerivField once on host arrays.
//
//   ref_loop_main [N=16] [steps=3] [rk: 0 RK4, 1 TVD-RK3]
// Prints "steps <n> time <t> KE <ke> dudx <v>" and exits 0, or the error and
// exits with the C ABI status code.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "cs3d_ref_binding.hpp"

using namespace cs3d_ref;

int main(int argc, char **argv) {
    const int N = argc > 1 ? atoi(argv[1]) : 16;
    const int steps = argc > 2 ? atoi(argv[2]) : 3;
    const int rkind = argc > 3 ? atoi(argv[3]) : CS3D_RK4;
    const double L = 2.0 * M_PI - (2.0 * M_PI / (double)N);
    Domain *dom = new Domain(N, N, N, L, L, L);
    TimeStepping *ts = new TimeStepping(TimeStepping::CONST_CFL, 0.5, steps, 1e300, 1, 1, 1 << 30);
    BC *bc = new BC(BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC, BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC,
                    BC::PERIODIC_SOLVE, BC::PERIODIC, BC::PERIODIC);
    const double gamma = 1.4, p0 = 1.0 / (gamma * 0.01);
    const double mu_ref = 1.0 / (1600.0 * std::pow(p0 / (1.0 / gamma), 0.76));
    try {
        CSolver_GB300 *cs = new CSolver_GB300(dom, bc, ts, 0.49, mu_ref, 16, false, rkind);
        cs->writeDumps = false;
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
        AbstractRK *rk = rkind == CS3D_TVDRK3 ? (AbstractRK *)new TVDRK3_GB300(cs) : (AbstractRK *)new RK4_GB300(cs);
        rk->executeSolverLoop();
        double ke = 0.0;
        for (int i = 0; i < dom->N; i++)
            ke += 0.5 * (cs->rhoU1[i] * cs->rhoU1[i] + cs->rhoV1[i] * cs->rhoV1[i] + cs->rhoW1[i] * cs->rhoW1[i]) /
                  cs->rho1[i];
        // d/dx of sin x on host arrays through the operator-only handle
        Derivatives_GB300 dx(dom, BC::PERIODIC_SOLVE, Derivatives::DIRX);
        double *f = new double[dom->N], *df = new double[dom->N];
        for (int i = 0; i < dom->N; i++) f[i] = std::sin(dom->x[i % N]);
        dx.calc1stDerivField(f, df);
        printf("steps %d time %.17g KE %.17g dudx %.17g\n", cs->timeStep, cs->time, ke, df[0]);
        delete[] f;
        delete[] df;
        delete rk;
        delete cs;
    } catch (const Error &e) {
        fprintf(stderr, "ref_loop_main: %s\n", e.what());
        return e.code;
    }
    return 0;
}
