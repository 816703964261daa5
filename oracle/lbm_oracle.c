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
#include <math.h>
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

/* ------------------------------------------------------------------------
 * Shifted 16-bit storage (FP16 or BF16 holding f_i - w_i, collision in FP32).
 * Not a reference mode: this restates the GB300 solver's precision extension
 * so that its 16-bit kernels can be checked bit for bit.  The collision is
 * collide_shifted below (BGK on deviations: with the density deviation in
 * place of rho, the reference formula yields feq - w); lid cells take the
 * deviation form feq(1, U) - w = the reference formula at rho = 0.
 * Conversions are IEEE round-to-nearest-even, written out in integer
 * arithmetic so that every host gives the same bits.
 * ------------------------------------------------------------------------ */
#include <string.h>

static float bits_to_float(uint32_t x) { float f; memcpy(&f, &x, 4); return f; }
static uint32_t float_to_bits(float f) { uint32_t x; memcpy(&x, &f, 4); return x; }

static float half_to_float(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    if (e == 0) {
        int s = 0;
        if (m == 0) return bits_to_float(sign);
        while (!(m & 0x400u)) { m <<= 1; ++s; }
        return bits_to_float(sign | ((uint32_t)(113 - s) << 23) | ((m & 0x3ffu) << 13));
    }
    if (e == 31) return bits_to_float(sign | 0x7f800000u | (m << 13));
    return bits_to_float(sign | ((e + 112u) << 23) | (m << 13));
}

static uint16_t float_to_half(float f)
{
    const uint32_t x = float_to_bits(f);
    const uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);      /* rounds to >= 65520: inf */
    if (ax >= 0x38800000u) {                                        /* normal half */
        uint32_t h = ((((ax >> 23) - 112u) << 10) | ((ax & 0x7fffffu) >> 13));
        const uint32_t rem = ax & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    if (ax < 0x33000000u) return (uint16_t)sign;                     /* below half of the least subnormal */
    {
        const uint32_t mant = (ax & 0x7fffffu) | 0x800000u;
        const int shift = 126 - (int)(ax >> 23);                    /* 14..24 */
        uint32_t m = mant >> shift;
        const uint32_t rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (m & 1u))) ++m;
        return (uint16_t)(sign | m);
    }
}

static float bf16_to_float(uint16_t b) { return bits_to_float((uint32_t)b << 16); }

static uint16_t float_to_bf16(float f)
{
    uint32_t x = float_to_bits(f);
    if ((x & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((x >> 16) | 0x40u);
    x += 0x7fffu + ((x >> 16) & 1u);
    return (uint16_t)(x >> 16);
}

/* The shifted modes' collision, restating collide_shifted of
 * cavityflow_cuda_gb300/csrc/lbm_core.cuh: moments from pair sums and
 * differences, every multiply-add fused (fmaf is correctly rounded on every
 * host, and contraction is off elsewhere). */
static void relax_pair_shifted(float* sp, float* sm, float w3, float w45, float wP, float u, float omega)
{
    const float even = fmaf(w45, u * u, wP);
    const float odd = w3 * u;
    *sp = fmaf(omega, (even + odd) - *sp, *sp);
    *sm = fmaf(omega, (even - odd) - *sm, *sm);
}

/* e: the deviations are scaled by 2^e (kind 2 collides in those units); the
 * quadratic terms' constants carry 2^-e, so every result is exactly 2^e times
 * the unscaled one. */
static void collide_shifted(float* s, float omega, int e)
{
    const float inv_scale = 1.0f / (float)(1u << e);
    const float a01 = s[0] + s[1], d01 = s[0] - s[1];
    const float a23 = s[2] + s[3], d23 = s[2] - s[3];
    const float a45 = s[4] + s[5], d45 = s[4] - s[5];
    const float a67 = s[6] + s[7], d67 = s[6] - s[7];
    const float a89 = s[8] + s[9], d89 = s[8] - s[9];
    const float a1011 = s[10] + s[11], d1011 = s[10] - s[11];
    const float a1213 = s[12] + s[13], d1213 = s[12] - s[13];
    const float a1415 = s[14] + s[15], d1415 = s[14] - s[15];
    const float a1617 = s[16] + s[17], d1617 = s[16] - s[17];
    const float drho = ((a01 + a23) + (a45 + a67)) + ((a89 + a1011) + (a1213 + a1415)) + (a1617 + s[18]);
    const float jx = ((d01 + d45) + (d67 + d89)) + d1011;
    const float jy = ((d23 + d45) - d67) + (d1213 + d1415);
    const float jz = ((d89 - d1011) + (d1213 - d1415)) + d1617;
    const float vel2 = fmaf(jz, jz, fmaf(jy, jy, jx * jx));
    const float P = fmaf(-1.5f * inv_scale, vel2, drho);
    const float wa = 1.0f / 18.0f, wd = 1.0f / 36.0f;
    const float waP = wa * P, wdP = wd * P;
    const float wa3 = 3.0f * wa, wa45 = (4.5f * wa) * inv_scale, wd3 = 3.0f * wd, wd45 = (4.5f * wd) * inv_scale;
    relax_pair_shifted(&s[0], &s[1], wa3, wa45, waP, jx, omega);
    relax_pair_shifted(&s[2], &s[3], wa3, wa45, waP, jy, omega);
    relax_pair_shifted(&s[4], &s[5], wd3, wd45, wdP, jx + jy, omega);
    relax_pair_shifted(&s[6], &s[7], wd3, wd45, wdP, jx - jy, omega);
    relax_pair_shifted(&s[8], &s[9], wd3, wd45, wdP, jx + jz, omega);
    relax_pair_shifted(&s[10], &s[11], wd3, wd45, wdP, jx - jz, omega);
    relax_pair_shifted(&s[12], &s[13], wd3, wd45, wdP, jy + jz, omega);
    relax_pair_shifted(&s[14], &s[15], wd3, wd45, wdP, jy - jz, omega);
    relax_pair_shifted(&s[16], &s[17], wa3, wa45, waP, jz, omega);
    s[18] = fmaf(omega, (1.0f / 3.0f) * P - s[18], s[18]);
}

/* IEEE half, rounded toward zero (the truncation of float_to_half's normal
 * and subnormal cases; finite values beyond the range give the largest
 * finite half). */
static uint16_t float_to_half_rz(float f)
{
    const uint32_t x = float_to_bits(f);
    const uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
    if (ax > 0x7f800000u) return (uint16_t)(sign | 0x7e00u);
    if (ax == 0x7f800000u) return (uint16_t)(sign | 0x7c00u);
    if (ax >= 0x47800000u) return (uint16_t)(sign | 0x7bffu);
    if (ax >= 0x38800000u) return (uint16_t)(sign | ((((ax >> 23) - 112u) << 10) | ((ax & 0x7fffffu) >> 13)));
    {
        const int shift = 126 - (int)(ax >> 23);
        if (shift > 24) return (uint16_t)sign;
        return (uint16_t)(sign | (((ax & 0x7fffffu) | 0x800000u) >> shift));
    }
}

/* Stochastic-rounding keys of the F16SR mode (kind 2), restating sr_hash,
 * sr_cell and sr_dither of cavityflow_cuda_gb300/csrc/lbm_core.cuh: the
 * "lowbias32" integer hash (C. Wellons) of the compact index of the row's
 * first cell and the time step, a per-cell key from it and x (mixed by an
 * odd multiplier), and 13 dither bits per population: the key's top 13 bits
 * XOR a 13-bit Weyl-sequence constant of the population. */
static uint32_t sr_hash(uint32_t cell, uint32_t step)
{
    uint32_t x = cell ^ (step * 0x9E3779B9u);
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
static uint32_t sr_cell(uint32_t row_hash, int x) { return (row_hash ^ ((uint32_t)x * 0x85EBCA6Bu)) * 0x2545F491u; }
static uint32_t sr_dither(uint32_t h, int k) { return (h >> 19) ^ (((uint32_t)(k + 1) * 0x9E3779B9u) >> 19); }

/* kind 2 keeps half(s * 2^12): the scale is exact (a power of two). */
static const float kSrScale = 4096.0f, kSrUnscale = 1.0f / 4096.0f;

static float ld16(uint16_t v, int kind)
{
    if (kind == 2) return half_to_float(v) * kSrUnscale;
    return kind ? bf16_to_float(v) : half_to_float(v);
}
/* The time steps work in step units: kind 2's scaled deviations (no scaling
 * per population), the plain deviation otherwise. */
static float ld16_step(uint16_t v, int kind) { return kind == 2 ? half_to_float(v) : ld16(v, kind); }
static int step_log2(int kind) { return kind == 2 ? 12 : 0; }
/* Lid cells' equilibrium deviation in step units. */
static void lid_step(float lid_u, int kind, float* f)
{
    int k;
    equilibriumf(0.0f, lid_u, 0.0f, 0.0f, f);
    if (kind == 2)
        for (k = 0; k < 19; ++k) f[k] *= kSrScale;
}
/* Store of population k (a value in step units) of the cell with hash h:
 * kind 2 adds the dither below the 13 bits half precision drops and
 * truncates (stochastic rounding). */
static uint16_t st16k(float v, int kind, uint32_t h, int k)
{
    if (kind == 2) return float_to_half_rz(bits_to_float(float_to_bits(v) + sr_dither(h, k)));
    return kind ? float_to_bf16(v) : float_to_half(v);
}

void orc_init_s(uint16_t* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6])
{
    /* flags exactly as the float oracle sets them; the deviation at rest is 0 */
    const int64_t C = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
    float* scratch = (float*)malloc((size_t)C * 19 * sizeof(float));
    orc_init_f(scratch, flags, nx, ny, nz, bc);
    free(scratch);
    memset(dd, 0, (size_t)C * 19 * sizeof(uint16_t));
}

/* The moving top wall's correction in step units (see wall_correctf). */
static float wall_du(float lid_u, int kind)
{
    float du = lid_u * (1.0f / 6.0f);
    if (kind == 2) du *= kSrScale;
    return du;
}
static int wall_row(int wall, const int32_t origin[3], int Xi, int Yi, int Zi, int nx, int ny, int nz)
{
    return wall && origin[1] + Yi == ny && origin[0] + Xi >= 1 && origin[0] + Xi <= nx && origin[2] + Zi >= 1 &&
           origin[2] + Zi <= nz;
}

static void alpha_s_impl(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                         int kind, const int32_t origin[3], const int32_t size[3], uint32_t step, int wall)
{
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    const float du = wall_du(lid_u, kind);
    int Zi;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (Zi = 0; Zi < size[2]; ++Zi) {
        int Yi, Xi, k;
        float f[19];
        uint32_t h;
        for (Yi = 0; Yi < size[1]; ++Yi) {
            for (Xi = 0; Xi < size[0]; ++Xi) {
                const int64_t gid = (origin[2] + Zi) * XY + (origin[1] + Yi) * X + origin[0] + Xi;
                int32_t fl;
                if (gid >= C) continue;
                fl = flags[gid];
                if (fl == ORC_FLUID) {
                    for (k = 0; k < 19; ++k) f[k] = ld16_step(dd[k * C + gid], kind);
                    if (wall_row(wall, origin, Xi, Yi, Zi, nx, ny, nz)) wall_correctf(f, flags, gid, X, du);
                    collide_shifted(f, inv_tau, step_log2(kind));
                } else if (fl == ORC_VELOCITY_INJECTION) {
                    lid_step(lid_u, kind, f);
                } else {
                    continue;
                }
                h = sr_cell(sr_hash((uint32_t)(gid - (origin[0] + Xi)), step), origin[0] + Xi);
                for (k = 0; k < 18; ++k) dd[(k ^ 1) * C + gid] = st16k(f[k], kind, h, k);
                dd[18 * C + gid] = st16k(f[18], kind, h, 18);
            }
        }
    }
}

void orc_alpha_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                 int kind, const int32_t origin[3], const int32_t size[3], uint32_t step)
{
    alpha_s_impl(dd, flags, nx, ny, nz, inv_tau, lid_u, kind, origin, size, step, 0);
}

void orc_alpha_wall_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                      int kind, const int32_t origin[3], const int32_t size[3], uint32_t step)
{
    alpha_s_impl(dd, flags, nx, ny, nz, inv_tau, lid_u, kind, origin, size, step, 1);
}

static void beta_s_impl(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                        int kind, const int32_t origin[3], const int32_t size[3], uint32_t step, int wall)
{
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    const float du = wall_du(lid_u, kind);
    int64_t delta[19];
    int Zi, k0;
    for (k0 = 0; k0 < 19; ++k0) delta[k0] = beta_deltaf(k0, X, XY, C);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (Zi = 0; Zi < size[2]; ++Zi) {
        int Yi, Xi, k;
        float f[19];
        uint32_t h;
        int64_t pos[19];
        for (Yi = 0; Yi < size[1]; ++Yi) {
            for (Xi = 0; Xi < size[0]; ++Xi) {
                const int64_t gid = (origin[2] + Zi) * XY + (origin[1] + Yi) * X + origin[0] + Xi;
                int32_t fl;
                if (gid >= C) continue;
                fl = flags[gid];
                if (fl == ORC_OBSTACLE) continue;            /* swap then write back: no change */
                for (k = 0; k < 19; ++k) pos[k] = k * C + (gid + delta[k]) % C;
                if (fl == ORC_FLUID) {
                    for (k = 0; k < 18; ++k) f[k ^ 1] = ld16_step(dd[pos[k]], kind);
                    f[18] = ld16_step(dd[pos[18]], kind);
                    if (wall_row(wall, origin, Xi, Yi, Zi, nx, ny, nz)) wall_correctf(f, flags, gid, X, du);
                    collide_shifted(f, inv_tau, step_log2(kind));
                    h = sr_cell(sr_hash((uint32_t)(gid - (origin[0] + Xi)), step), origin[0] + Xi);
                    for (k = 0; k < 19; ++k) dd[pos[k]] = st16k(f[k], kind, h, k);
                } else if (fl == ORC_VELOCITY_INJECTION) {
                    lid_step(lid_u, kind, f);
                    h = sr_cell(sr_hash((uint32_t)(gid - (origin[0] + Xi)), step), origin[0] + Xi);
                    for (k = 0; k < 19; ++k) dd[pos[k]] = st16k(f[k], kind, h, k);
                } else {                                      /* streamed through unchanged */
                    uint16_t raw[19];
                    for (k = 0; k < 18; ++k) raw[k ^ 1] = dd[pos[k]];
                    raw[18] = dd[pos[18]];
                    for (k = 0; k < 19; ++k) dd[pos[k]] = raw[k];
                }
            }
        }
    }
}

void orc_beta_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                int kind, const int32_t origin[3], const int32_t size[3], uint32_t step)
{
    beta_s_impl(dd, flags, nx, ny, nz, inv_tau, lid_u, kind, origin, size, step, 0);
}

void orc_beta_wall_s(uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, float inv_tau, float lid_u,
                     int kind, const int32_t origin[3], const int32_t size[3], uint32_t step)
{
    beta_s_impl(dd, flags, nx, ny, nz, inv_tau, lid_u, kind, origin, size, step, 1);
}

void orc_macros_s(const uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, int last_was_alpha,
                  float lid_u, int kind, float* rho, float* jx, float* jy, float* jz)
{
    static const int cx[19] = {1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0};
    static const int cy[19] = {0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0};
    static const int cz[19] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0};
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    int z;
    for (z = 0; z < nz + 2; ++z) {
        int y, x, k;
        float f[19], r, vx, vy, vz;
        for (y = 0; y < ny + 2; ++y) {
            for (x = 0; x < nx + 2; ++x) {
                const int64_t gid = z * XY + y * X + x;
                const int interior = x >= 1 && x <= nx && y >= 1 && y <= ny && z >= 1 && z <= nz;
                const int32_t fl = flags[gid];
                r = vx = vy = vz = 0.0f;
                if (interior && fl == ORC_FLUID) {
                    for (k = 0; k < 19; ++k)
                        f[k] = ld16(last_was_alpha ? dd[(k == 18 ? 18 : (k ^ 1)) * C + gid]
                                                   : dd[k * C + gid + cx[k] + cy[k] * X + cz[k] * XY], kind);
                    momentsf(f, &r, &vx, &vy, &vz);
                    r = r + 1.0f;
                } else if (interior && fl == ORC_VELOCITY_INJECTION) {
                    r = 1.0f; vx = lid_u;
                }
                rho[gid] = r; jx[gid] = vx; jy[gid] = vy; jz[gid] = vz;
            }
        }
    }
}

void orc_reduce_s(const uint16_t* dd, const int32_t* flags, int nx, int ny, int nz, int last_was_alpha, int kind,
                  double out[4])
{
    /* The FP64 totals of orc_reduce_*: every live slot contributes
     * (double)(f - w) + (double)w; the momentum uses the deviations (the
     * weights' momentum is zero). */
    static const int cx[19] = {1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0};
    static const int cy[19] = {0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0};
    static const int cz[19] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0};
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    double* part = (double*)calloc((size_t)4 * (nz + 2), sizeof(double));
    int z, q;
    for (z = 1; z <= nz; ++z) {
        int y, x, k;
        double m = 0, px = 0, py = 0, pz = 0;
        for (y = 1; y <= ny; ++y) {
            for (x = 1; x <= nx; ++x) {
                const int64_t gid = z * XY + y * X + x;
                const int32_t fl = flags[gid];
                if (fl != ORC_FLUID && fl != ORC_VELOCITY_INJECTION) continue;
                for (k = 0; k < 19; ++k) {
                    const double w = (double)(k == 18 ? 1.0f / 3.0f : (k < 4 || k >= 16) ? 1.0f / 18.0f : 1.0f / 36.0f);
                    const int64_t nb = gid + cx[k] + cy[k] * X + cz[k] * XY;
                    const int32_t fn = flags[nb];
                    double f;
                    m += (double)ld16(dd[k * C + gid], kind) + w;
                    if (fn != ORC_FLUID && fn != ORC_VELOCITY_INJECTION) m += (double)ld16(dd[k * C + nb], kind) + w;
                    f = (double)ld16(last_was_alpha ? dd[(k == 18 ? 18 : (k ^ 1)) * C + gid] : dd[k * C + nb], kind);
                    px += cx[k] * f; py += cy[k] * f; pz += cz[k] * f;
                }
            }
        }
        part[4 * z + 0] = m; part[4 * z + 1] = px; part[4 * z + 2] = py; part[4 * z + 3] = pz;
    }
    for (q = 0; q < 4; ++q) out[q] = 0.0;
    for (z = 1; z <= nz; ++z)
        for (q = 0; q < 4; ++q) out[q] += part[4 * z + q];
    free(part);
}

uint16_t orc_float_to_half(float f) { return float_to_half(f); }
uint16_t orc_float_to_half_rz(float f) { return float_to_half_rz(f); }
uint32_t orc_sr_hash(uint32_t cell, uint32_t step) { return sr_hash(cell, step); }
float orc_half_to_float(uint16_t h) { return half_to_float(h); }
uint16_t orc_float_to_bf16(float f) { return float_to_bf16(f); }
