/*
 * lbm_oracle.c -- CPU oracle for the D3Q19 A-A lid-driven cavity.
 *
 * TEST INFRASTRUCTURE ONLY: a restatement of the reference's CPU/GPU kernels
 * (saleemayman/cavityflow_cuda, src/gpukernels/lbm_{init,alpha,beta}.cu and
 * their CPU twins src/cpukernels/CLbm{Init,Alpha,Beta}CPU.cpp) used by the
 * tests, the smoke check and bench.py's CPU-baseline leg as the checker.
 * The product path (cavityflow_cuda_gb300/) never links or calls it.
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off, so the same
 * source gives the same bits on x86-64 and aarch64).
 */
#include <stdlib.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lbm_oracle.h"

#define REAL double
#define SFX(name) name##d
#include "lbm_oracle_body.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX(name) name##f
#include "lbm_oracle_body.h"
#undef REAL
#undef SFX

void orc_set_lid(int32_t* flags, int nx, int ny, int nz)
{
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    int x, z;
    for (z = 1; z <= nz; ++z)
        for (x = 1; x <= nx; ++x)
            flags[z * XY + (int64_t)ny * X + x] = ORC_VELOCITY_INJECTION;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
