// dropin_main.cpp -- test program for the C++ drop-in (include/CLbmSolverGB300.hpp):
// the reference's own configuration, domain and solver base classes
// (src/CConfiguration.cpp, src/CDomain.cpp, src/CLbmSolver.cpp, compiled from the
// reference checkout where they lie) with CLbmSolverGB300<T> in place of
// CLbmSolverGPU<T>, driven the way CController drives a solver
// (src/CController.cpp:1278-1348): the lid plane is marked through setFlags,
// then alpha and beta alternate.  Linked against liblbm_gb300.so.
//
//   dropin CONFIG.xml STEPS OUT.bin
//
// Writes the interior populations (19 packed components, the solver's value
// type) after STEPS steps to OUT.bin.  Without a CUDA device the adapter's
// constructor reports the error and exits with LBM_ERR_NO_DEVICE (10), where
// the reference's CLbmSolverGPU exits through GPU_ERROR_CHECK.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "CConfiguration.hpp"
#include "CDomain.hpp"
#include "CLbmSolverGB300.hpp"

#ifndef DROPIN_REAL
#define DROPIN_REAL float
#endif
typedef DROPIN_REAL T;

int main(int argc, char** argv)
{
    if (argc != 4) {
        std::fprintf(stderr, "usage: dropin CONFIG.xml STEPS OUT.bin\n");
        return 2;
    }
    CConfiguration<T> configuration(argv[1]);
    const int steps = std::atoi(argv[2]);
    CDomain<T> domain(0, configuration.domainSize, CVector<3, int>(0), configuration.domainLength);
    std::vector<Flag> boundaryConditions(6, OBSTACLE);  // one subdomain: six walls (src/CManager.cpp:91-104)
    CLbmSolverGB300<T> solver(0, domain, boundaryConditions, &configuration);

    // the lid plane y = ny as CController::setDrivenCavitySzenario marks it
    CVector<3, int> size = domain.getSize();
    CVector<3, int> lidOrigin(1, size[1], 1), lidSize(size[0], 1, size[2]);
    std::vector<Flag> lid((size_t)size[0] * size[2], VELOCITY_INJECTION);
    solver.setFlags(lidOrigin, lidSize, lid.data());

    for (int i = 0; i < steps; ++i) {
        if (i & 1) solver.simulationStepBeta();
        else solver.simulationStepAlpha();
    }
    const size_t cells = (size_t)size[0] * size[1] * size[2];
    std::vector<T> dd(19 * cells);
    CVector<3, int> origin(1, 1, 1);
    solver.getDensityDistributions(origin, size, dd.data());
    cudaDeviceSynchronize();
    FILE* f = std::fopen(argv[3], "wb");
    if (!f || std::fwrite(dd.data(), sizeof(T), dd.size(), f) != dd.size()) return 3;
    std::fclose(f);
    std::printf("dropin: %d steps of a %dx%dx%d cavity written\n", steps, size[0], size[1], size[2]);
    return 0;
}
