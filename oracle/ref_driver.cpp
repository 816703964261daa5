/*
 * ref_driver.cpp -- a thin C harness around the reference's OWN CPU kernels
 * (saleemayman/cavityflow_cuda src/cpukernels/CLbm{Init,Alpha,Beta}CPU.cpp).
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the reference's kernel sources, where they lie in the read-only reference
 * checkout, into oracle/_ref/libref_cavity.so (git-ignored; nothing from the
 * reference is copied into this repository).  It is used to pin the C oracle
 * (oracle/lbm_oracle.c) and to generate the golden fixtures in tests/golden/.
 *
 * The harness sets flags x-fastest as the GPU init kernel does
 * (src/gpukernels/lbm_init.cu:73-93) instead of through
 * CLbmInitCPU::setFlags, which stores them x-slowest
 * (src/cpukernels/CLbmInitCPU.cpp:43-71) and so is only right for cubes.
 */
#include <cstdint>
#include <iostream>
#include <string>
#include <vector>

#include "CConfiguration.hpp"
#include "CDomain.hpp"
#include "CLbmSolver.hpp"
#include "common.h"
#include "cpukernels/CLbmAlphaCPU.hpp"
#include "cpukernels/CLbmBetaCPU.hpp"
#include "cpukernels/CLbmInitCPU.hpp"

// src/common.h:37 declares this table; src/main.cpp:34-40 defines it.  Only
// the direction-filtered copies use it, which this harness never calls.
CVector<3, int> lbm_units[19];

namespace {

template <class T>
void ref_init(T* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6])
{
    CVector<3, int> sizeWithHalo(nx + 2, ny + 2, nz + 2);
    std::vector<Flag> bcs(6);
    for (int i = 0; i < 6; ++i) bcs[i] = static_cast<Flag>(bc[i]);
    CLbmInitCPU<T> init(sizeWithHalo, bcs);
    init.initLbm(dd, reinterpret_cast<Flag*>(flags), nullptr, nullptr, false, false);

    const int X = nx + 2, Y = ny + 2, Z = nz + 2;
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x) {
                int32_t fl = FLUID;
                if (x == 0) fl = bc[0];
                if (x == X - 1 && fl != OBSTACLE) fl = bc[1];
                if (y == 0 && fl != OBSTACLE) fl = bc[2];
                if (y == Y - 1 && fl != OBSTACLE) fl = bc[3];
                if (z == 0 && fl != OBSTACLE) fl = bc[4];
                if (z == Z - 1 && fl != OBSTACLE) fl = bc[5];
                flags[(static_cast<int64_t>(z) * Y + y) * X + x] = fl;
            }
}

template <class T>
void ref_alpha(T* dd, int32_t* flags, int nx, int ny, int nz, T inv_tau,
               T gx, T gy, T gz, T lid_u, const int32_t origin[3], const int32_t size[3],
               const int32_t block[3])
{
    CVector<3, int> sizeWithHalo(nx + 2, ny + 2, nz + 2);
    CLbmAlphaCPU<T> alpha(sizeWithHalo, CVector<3, T>(gx, gy, gz));
    alpha.alphaKernelCPU(dd, reinterpret_cast<Flag*>(flags), nullptr, nullptr, inv_tau, lid_u,
                         CVector<3, int>(origin[0], origin[1], origin[2]),
                         CVector<3, int>(size[0], size[1], size[2]),
                         CVector<3, int>(block[0], block[1], block[2]), false, false);
}

template <class T>
void ref_beta(T* dd, int32_t* flags, int nx, int ny, int nz, T inv_tau, T lid_u,
              const int32_t origin[3], const int32_t size[3], const int32_t block[3])
{
    CVector<3, int> sizeWithHalo(nx + 2, ny + 2, nz + 2);
    const int cells = sizeWithHalo.elements();
    const bool pow2 = cells > 0 && (cells & (cells - 1)) == 0;
    CLbmBetaCPU<T> beta(sizeWithHalo, CVector<3, T>(0, 0, 0));
    beta.betaKernelCPU(dd, reinterpret_cast<Flag*>(flags), nullptr, nullptr, inv_tau, lid_u,
                       CVector<3, int>(origin[0], origin[1], origin[2]),
                       CVector<3, int>(size[0], size[1], size[2]),
                       CVector<3, int>(block[0], block[1], block[2]), pow2, false, false);
}

// Exposes the lattice parameters the reference's solver base class derives
// from a configuration (src/CLbmSolver.cpp:28-327).
template <class T>
class ParamProbe : public CLbmSolver<T>
{
public:
    ParamProbe(CDomain<T>& d, CConfiguration<T>* c)
        : CLbmSolver<T>(0, d, std::vector<Flag>(6, OBSTACLE), c) {}
    void dump(double out[10])
    {
        out[0] = this->timestepSize;
        out[1] = this->tau;
        out[2] = this->tauInv;
        out[3] = this->velocityDimLess[0];
        out[4] = this->velocityDimLess[1];
        out[5] = this->velocityDimLess[2];
        out[6] = this->accelerationDimLess[0];
        out[7] = this->accelerationDimLess[1];
        out[8] = this->accelerationDimLess[2];
        out[9] = this->viscosityDimLess;
    }
};

// The single-domain setup of src/CManager.cpp:27-58 with one subdomain.
template <class T>
void ref_params(const char* xml, double out[10])
{
    CConfiguration<T> cfg{std::string(xml)};
    CDomain<T> domain(0, cfg.domainSize, CVector<3, int>(0), cfg.domainLength);
    ParamProbe<T> probe(domain, &cfg);
    probe.dump(out);
}

// Every field of the reference's configuration reader
// (src/CConfiguration.hpp:57-96): 14 reals, 27 integers, 4 directories of
// 256 bytes each.
template <class T>
void ref_config(const char* xml, double* r, int32_t* n, char* dirs)
{
    CConfiguration<T> c{std::string(xml)};
    const T reals[14] = {c.velocity[0], c.velocity[1], c.velocity[2], c.acceleration[0], c.acceleration[1],
                         c.acceleration[2], c.viscosity, c.maxVelocityDimLess, c.maxAccelerationDimLess,
                         c.domainLength[0], c.domainLength[1], c.domainLength[2], c.CPUSubdomainRatio, c.timestep};
    for (int i = 0; i < 14; ++i) r[i] = (double)reals[i];
    int k = 0;
    for (int d = 0; d < 3; ++d) n[k++] = c.domainSize[d];
    for (int d = 0; d < 3; ++d) n[k++] = c.numOfSubdomains[d];
    n[k++] = c.loops;
    n[k++] = c.doBenchmark;
    n[k++] = c.doLogging;
    n[k++] = c.doValidation;
    n[k++] = c.doVisualization;
    n[k++] = c.visualizationRate;
    for (int b = 0; b < 2; ++b)
        for (int d = 0; d < 3; ++d) n[k++] = c.elementsPerBlock[b][d];
    for (int b = 0; b < 3; ++b) {
        n[k++] = (int32_t)c.threadsPerBlock[b].x;
        n[k++] = (int32_t)c.threadsPerBlock[b].y;
        n[k++] = (int32_t)c.threadsPerBlock[b].z;
    }
    const std::string* ds[4] = {&c.benchmarkOutputDir, &c.loggingOutputDir, &c.validationOutputDir,
                                &c.visualizationOutputDir};
    for (int i = 0; i < 4; ++i) {
        const size_t m = ds[i]->size() < 255 ? ds[i]->size() : 255;
        ds[i]->copy(dirs + 256 * i, m);
        dirs[256 * i + m] = 0;
    }
}

}  // namespace

extern "C" {

void ref_config_d(const char* xml, double* r, int32_t* n, char* dirs) { ref_config<double>(xml, r, n, dirs); }
void ref_config_f(const char* xml, double* r, int32_t* n, char* dirs) { ref_config<float>(xml, r, n, dirs); }

void ref_params_d(const char* xml, double out[10]) { ref_params<double>(xml, out); }
void ref_params_f(const char* xml, double out[10]) { ref_params<float>(xml, out); }

void ref_init_d(double* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6])
{ ref_init<double>(dd, flags, nx, ny, nz, bc); }
void ref_init_f(float* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6])
{ ref_init<float>(dd, flags, nx, ny, nz, bc); }

void ref_alpha_d(double* dd, int32_t* flags, int nx, int ny, int nz, double inv_tau,
                 double gx, double gy, double gz, double lid_u,
                 const int32_t origin[3], const int32_t size[3], const int32_t block[3])
{ ref_alpha<double>(dd, flags, nx, ny, nz, inv_tau, gx, gy, gz, lid_u, origin, size, block); }
void ref_alpha_f(float* dd, int32_t* flags, int nx, int ny, int nz, float inv_tau,
                 float gx, float gy, float gz, float lid_u,
                 const int32_t origin[3], const int32_t size[3], const int32_t block[3])
{ ref_alpha<float>(dd, flags, nx, ny, nz, inv_tau, gx, gy, gz, lid_u, origin, size, block); }

void ref_beta_d(double* dd, int32_t* flags, int nx, int ny, int nz, double inv_tau, double lid_u,
                const int32_t origin[3], const int32_t size[3], const int32_t block[3])
{ ref_beta<double>(dd, flags, nx, ny, nz, inv_tau, lid_u, origin, size, block); }
void ref_beta_f(float* dd, int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                const int32_t origin[3], const int32_t size[3], const int32_t block[3])
{ ref_beta<float>(dd, flags, nx, ny, nz, inv_tau, lid_u, origin, size, block); }

}  // extern "C"
