/*
 * lbm_oracle.h -- CPU restatement of the reference D3Q19 A-A lid-driven-cavity
 * path (saleemayman/cavityflow_cuda), used ONLY as test infrastructure: the
 * parity tests, the smoke check and the CPU-baseline leg of bench.py call it as
 * the checker.  No product code path links or calls it.
 *
 * Layout is the reference's: 19 planes ("slots") of (nx+2)*(ny+2)*(nz+2) cells,
 * x fastest, one halo cell on each face (src/CLbmSolverGPU.cu:71,
 * src/gpukernels/lbm_alpha.cu:45-50).  Flags are 32-bit like the reference's
 * Flag enum (src/common.h:54-61).
 *
 * Arithmetic follows the reference kernels operation by operation (summation
 * order src/gpukernels/lbm_alpha.cu:86-186, equilibrium factorisation
 * src/common.h:132-160) and is compiled without floating-point contraction, so
 * it reproduces the reference CPU kernels built with g++ for x86-64 bit for bit.
 * That claim is pinned by tests/golden (fixtures generated by running the
 * reference's own CPU kernels, see oracle/ref_driver.cpp).
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flag values of the reference (src/common.h:54-61). */
enum { ORC_OBSTACLE = 1, ORC_FLUID = 2, ORC_VELOCITY_INJECTION = 4, ORC_GHOST_LAYER = 8 };

/* ---- double ---- */
void orc_init_d(double* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6]);
void orc_alpha_d(double* dd, const int32_t* flags, int nx, int ny, int nz,
                 double inv_tau, double gx, double gy, double gz, double lid_u,
                 const int32_t origin[3], const int32_t size[3]);
void orc_beta_d(double* dd, const int32_t* flags, int nx, int ny, int nz,
                double inv_tau, double lid_u,
                const int32_t origin[3], const int32_t size[3]);
void orc_macros_d(const double* dd, const int32_t* flags, int nx, int ny, int nz,
                  int last_was_alpha, double lid_u, double* rho, double* jx, double* jy, double* jz);
void orc_reduce_d(const double* dd, const int32_t* flags, int nx, int ny, int nz,
                  int last_was_alpha, double out[4]);

/* The same steps with the GB300 solver's opt-in moving top wall instead of an
 * injection lid (no reference counterpart): FLUID cells of row y = ny take
 * Ladd's correction -6 w_i (c_i . U) on the populations 5 and 6 the top face
 * sends back (see wall_correct in lbm_oracle_body.h). */
void orc_alpha_wall_d(double* dd, const int32_t* flags, int nx, int ny, int nz,
                      double inv_tau, double gx, double gy, double gz, double lid_u,
                      const int32_t origin[3], const int32_t size[3]);
void orc_beta_wall_d(double* dd, const int32_t* flags, int nx, int ny, int nz,
                     double inv_tau, double lid_u,
                     const int32_t origin[3], const int32_t size[3]);

/* ---- float ---- */
void orc_init_f(float* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6]);
void orc_alpha_f(float* dd, const int32_t* flags, int nx, int ny, int nz,
                 float inv_tau, float gx, float gy, float gz, float lid_u,
                 const int32_t origin[3], const int32_t size[3]);
void orc_beta_f(float* dd, const int32_t* flags, int nx, int ny, int nz,
                float inv_tau, float lid_u,
                const int32_t origin[3], const int32_t size[3]);
void orc_alpha_wall_f(float* dd, const int32_t* flags, int nx, int ny, int nz,
                      float inv_tau, float gx, float gy, float gz, float lid_u,
                      const int32_t origin[3], const int32_t size[3]);
void orc_beta_wall_f(float* dd, const int32_t* flags, int nx, int ny, int nz,
                     float inv_tau, float lid_u,
                     const int32_t origin[3], const int32_t size[3]);
void orc_macros_f(const float* dd, const int32_t* flags, int nx, int ny, int nz,
                  int last_was_alpha, float lid_u, float* rho, float* jx, float* jy, float* jz);
void orc_reduce_f(const float* dd, const int32_t* flags, int nx, int ny, int nz,
                  int last_was_alpha, double out[4]);

/* ---- shifted 16-bit storage (f - w in FP16 when kind = 0, BF16 when kind = 1,
 *      FP16 of (f - w) * 2^12 with stochastic rounding keyed by `step` when
 *      kind = 2; collision in float) -- the GB300 solver's precision extension ---- */
void orc_init_s(uint16_t* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6]);
void orc_alpha_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                 int kind, const int32_t origin[3], const int32_t size[3], uint32_t step);
void orc_beta_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                int kind, const int32_t origin[3], const int32_t size[3], uint32_t step);
void orc_alpha_wall_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                      int kind, const int32_t origin[3], const int32_t size[3], uint32_t step);
void orc_beta_wall_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                     int kind, const int32_t origin[3], const int32_t size[3], uint32_t step);
void orc_macros_s(const uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, int last_was_alpha,
                  float lid_u, int kind, float* rho, float* jx, float* jy, float* jz);
void orc_reduce_s(const uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, int last_was_alpha, int kind,
                  double out[4]);
uint16_t orc_float_to_half(float f);
uint16_t orc_float_to_half_rz(float f);
uint32_t orc_sr_hash(uint32_t cell, uint32_t step);
float orc_half_to_float(uint16_t h);
uint16_t orc_float_to_bf16(float f);

/* Marks the lid plane y = ny (interior coordinates x in [1,nx], z in [1,nz])
 * as VELOCITY_INJECTION, as src/CController.cpp:1313-1345 does. */
void orc_set_lid(int32_t* flags, int nx, int ny, int nz);

/* Number of OpenMP threads the step functions use (1 when built without OpenMP). */
int orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
