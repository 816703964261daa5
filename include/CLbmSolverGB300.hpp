/*
 * CLbmSolverGB300.hpp -- drop-in replacement for CLbmSolverGPU<T>
 * (saleemayman/cavityflow_cuda src/CLbmSolverGPU.cuh:25-95) that runs the
 * GB300 kernels through the C ABI of lbm_gb300.h.
 *
 * This header is meant to be compiled inside the reference tree: it derives
 * from the reference's own CLbmSolver<T> (src/CLbmSolver.hpp:30-89), so the
 * lattice parameters (tau, 1/tau, dimensionless lid velocity and gravity)
 * come from the reference's constructor unchanged, and it offers every
 * overload CLbmSolverGPU<T> offers, with the same argument meaning.
 * Link the program with liblbm_gb300.so.  The lid is the reference's
 * VELOCITY_INJECTION plane, marked by the caller through setFlags as
 * CController does; an optional last constructor argument
 * LBM_LID_MOVING_WALL selects the mass-conserving moving top wall instead,
 * which starts moving at construction.
 *
 * Error behaviour follows the reference: a failing CUDA call prints the error
 * and exits with its code (GPU_ERROR_CHECK, src/common.h:73-90); a cuboid
 * outside the domain fails the same way the reference's assert does.
 */
#ifndef CLBMSOLVERGB300_HPP
#define CLBMSOLVERGB300_HPP

#include <cassert>
#include <cstdlib>
#include <iostream>
#include <vector>

#include <cuda_runtime.h>

#include "CLbmSolver.hpp"
#include "lbm_gb300.h"

template <typename T>
class CLbmSolverGB300 : public CLbmSolver<T>
{
private:
    lbm_solver* solver;

    static void check(int status, const char* where)
    {
        if (status == LBM_OK) return;
        std::cerr << "----- CLbmSolverGB300<T>::" << where << " -----" << std::endl;
        std::cerr << "error:    " << lbm_status_string(status) << std::endl;
        std::cerr << "detail:   " << lbm_last_error() << std::endl;
        std::cerr << "EXECUTION WILL BE TERMINATED IMMEDIATELY" << std::endl;
        assert(status != LBM_ERR_OUT_OF_BOUNDS);
        std::exit(status == LBM_ERR_CUDA ? EXIT_FAILURE : status);
    }

    static void* st(cudaStream_t* stream) { return stream == NULL ? NULL : static_cast<void*>(*stream); }

public:
    CLbmSolverGB300(int id, CDomain<T>& domain, std::vector<Flag> boundaryConditions,
                    CConfiguration<T>* configuration, int lidMode = LBM_LID_INJECTION)
        : CLbmSolver<T>(id, domain, boundaryConditions, configuration), solver(NULL)
    {
        int numOfGPUsPerNode = 0;
        if (cudaGetDeviceCount(&numOfGPUsPerNode) != cudaSuccess || numOfGPUsPerNode == 0)
            check(LBM_ERR_NO_DEVICE, "CLbmSolverGB300()");
        lbm_params p = {};
        CVector<3, int> size = this->domain.getSize();
        for (int d = 0; d < 3; ++d) p.size[d] = size[d];
        p.storage = sizeof(T) == sizeof(double) ? LBM_STORAGE_F64 : LBM_STORAGE_F32;
        for (int f = 0; f < 6; ++f) p.boundary[f] = this->boundaryConditions[f];
        p.inv_tau = this->tauInv;
        p.lid_velocity = this->velocityDimLess[0];
        for (int d = 0; d < 3; ++d) p.gravity[d] = this->accelerationDimLess[d];
        p.device = this->id % numOfGPUsPerNode;  // src/CLbmSolverGPU.cu:42-45
        p.lid_mode = lidMode;
        check(lbm_create(&p, &solver), "CLbmSolverGB300()");
        if (lidMode == LBM_LID_MOVING_WALL) check(lbm_set_driven_cavity(solver), "CLbmSolverGB300()");
    }

    ~CLbmSolverGB300() { lbm_destroy(solver); }

    using CLbmSolver<T>::simulationStepAlpha;
    using CLbmSolver<T>::simulationStepBeta;
    using CLbmSolver<T>::getDensityDistributions;
    using CLbmSolver<T>::setDensityDistributions;

    void simulationStepAlpha(cudaStream_t* stream) { check(lbm_step_alpha(solver, st(stream)), "simulationStepAlpha()"); }
    void simulationStepAlpha() { simulationStepAlpha((cudaStream_t*)NULL); }
    void simulationStepAlpha(CVector<3, int> origin, CVector<3, int> size, cudaStream_t* stream)
    {
        check(lbm_step_alpha_cuboid(solver, origin.data, size.data, st(stream)), "simulationStepAlpha()");
    }
    void simulationStepAlpha(CVector<3, int> origin, CVector<3, int> size) { simulationStepAlpha(origin, size, NULL); }

    void simulationStepBeta(cudaStream_t* stream) { check(lbm_step_beta(solver, st(stream)), "simulationStepBeta()"); }
    void simulationStepBeta() { simulationStepBeta((cudaStream_t*)NULL); }
    void simulationStepBeta(CVector<3, int> origin, CVector<3, int> size, cudaStream_t* stream)
    {
        check(lbm_step_beta_cuboid(solver, origin.data, size.data, st(stream)), "simulationStepBeta()");
    }
    void simulationStepBeta(CVector<3, int> origin, CVector<3, int> size) { simulationStepBeta(origin, size, NULL); }

    void getDensityDistributions(CVector<3, int>& origin, CVector<3, int>& size, T* hDensityDistributions,
                                 cudaStream_t* stream)
    {
        check(lbm_get_density_distributions(solver, origin.data, size.data, hDensityDistributions, st(stream)),
              "getDensityDistributions()");
    }
    void getDensityDistributions(CVector<3, int>& origin, CVector<3, int>& size, T* hDensityDistributions)
    {
        getDensityDistributions(origin, size, hDensityDistributions, NULL);
    }
    void getDensityDistributions(T* hDensityDistributions, cudaStream_t* stream)
    {
        check(lbm_get_density_distributions(solver, NULL, NULL, hDensityDistributions, st(stream)),
              "getDensityDistributions()");
    }
    void getDensityDistributions(T* hDensityDistributions) { getDensityDistributions(hDensityDistributions, NULL); }

    void setDensityDistributions(CVector<3, int>& origin, CVector<3, int>& size, Direction direction,
                                 T* hDensityDistributions, cudaStream_t* stream)
    {
        check(lbm_set_density_distributions(solver, origin.data, size.data, (int32_t)direction, hDensityDistributions,
                                            st(stream)), "setDensityDistributions()");
    }
    void setDensityDistributions(CVector<3, int>& origin, CVector<3, int>& size, Direction direction,
                                 T* hDensityDistributions)
    {
        setDensityDistributions(origin, size, direction, hDensityDistributions, NULL);
    }
    void setDensityDistributions(CVector<3, int>& origin, CVector<3, int>& size, T* hDensityDistributions,
                                 cudaStream_t* stream)
    {
        check(lbm_set_density_distributions(solver, origin.data, size.data, LBM_DIRECTION_ALL, hDensityDistributions,
                                            st(stream)), "setDensityDistributions()");
    }
    void setDensityDistributions(CVector<3, int>& origin, CVector<3, int>& size, T* hDensityDistributions)
    {
        setDensityDistributions(origin, size, hDensityDistributions, NULL);
    }
    void setDensityDistributions(T* hDensityDistributions, cudaStream_t* stream)
    {
        check(lbm_set_density_distributions(solver, NULL, NULL, LBM_DIRECTION_ALL, hDensityDistributions, st(stream)),
              "setDensityDistributions()");
    }
    void setDensityDistributions(T* hDensityDistributions) { setDensityDistributions(hDensityDistributions, NULL); }

    void getFlags(CVector<3, int>& origin, CVector<3, int>& size, Flag* hFlags)
    {
        check(lbm_get_flags(solver, origin.data, size.data, reinterpret_cast<int32_t*>(hFlags)), "getFlags()");
    }
    void getFlags(Flag* hFlags) { check(lbm_get_flags(solver, NULL, NULL, reinterpret_cast<int32_t*>(hFlags)), "getFlags()"); }
    void setFlags(CVector<3, int>& origin, CVector<3, int>& size, Flag* hFlags)
    {
        check(lbm_set_flags(solver, origin.data, size.data, reinterpret_cast<const int32_t*>(hFlags)), "setFlags()");
    }
    void setFlags(Flag* hFlags) { check(lbm_set_flags(solver, NULL, NULL, reinterpret_cast<const int32_t*>(hFlags)), "setFlags()"); }

    void getVelocities(CVector<3, int>& origin, CVector<3, int>& size, T* hVelocities)
    {
        check(lbm_get_velocities(solver, origin.data, size.data, hVelocities), "getVelocities()");
    }
    void getVelocities(T* hVelocities) { check(lbm_get_velocities(solver, NULL, NULL, hVelocities), "getVelocities()"); }
    void setVelocities(CVector<3, int>& origin, CVector<3, int>& size, T* hVelocities)
    {
        check(lbm_set_velocities(solver, origin.data, size.data, hVelocities), "setVelocities()");
    }
    void setVelocities(T* hVelocities) { check(lbm_set_velocities(solver, NULL, NULL, hVelocities), "setVelocities()"); }

    void getDensities(CVector<3, int>& origin, CVector<3, int>& size, T* hDensities)
    {
        check(lbm_get_densities(solver, origin.data, size.data, hDensities), "getDensities()");
    }
    void getDensities(T* hDensities) { check(lbm_get_densities(solver, NULL, NULL, hDensities), "getDensities()"); }
    void setDensities(CVector<3, int>& origin, CVector<3, int>& size, T* hDensities)
    {
        check(lbm_set_densities(solver, origin.data, size.data, hDensities), "setDensities()");
    }
    void setDensities(T* hDensities) { check(lbm_set_densities(solver, NULL, NULL, hDensities), "setDensities()"); }
};

#endif
