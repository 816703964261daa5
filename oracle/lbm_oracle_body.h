/*
 * Type-generic body of the CPU oracle; included by lbm_oracle.c once per
 * precision with REAL (float|double) and SFX(name) defined.  Test
 * infrastructure only (see lbm_oracle.h).
 */

/* Weights as the reference writes them: (T)1/(T)18, (T)1/(T)36, (T)1/(T)3
 * (src/common.h:132-160), folded in the working precision. */
#define W_AXIS ((REAL)1 / (REAL)18)
#define W_DIAG ((REAL)1 / (REAL)36)
#define W_REST ((REAL)1 / (REAL)3)

/* Density and momentum of 19 populations, each accumulator summed in the
 * order of src/gpukernels/lbm_alpha.cu:86-186 (the beta kernel,
 * src/gpukernels/lbm_beta.cu:98-231, uses the same per-accumulator order). */
static void SFX(moments)(const REAL* f, REAL* rho, REAL* vx, REAL* vy, REAL* vz)
{
    REAL r = f[0], x = f[0], y, z;
    r += f[1];  x -= f[1];
    r += f[2];  y = f[2];
    r += f[3];  y -= f[3];
    r += f[4];  x += f[4];  y += f[4];
    r += f[5];  x -= f[5];  y -= f[5];
    r += f[6];  x += f[6];  y -= f[6];
    r += f[7];  x -= f[7];  y += f[7];
    r += f[8];  x += f[8];  z = f[8];
    r += f[9];  x -= f[9];  z -= f[9];
    r += f[10]; x += f[10]; z -= f[10];
    r += f[11]; x -= f[11]; z += f[11];
    r += f[12]; y += f[12]; z += f[12];
    r += f[13]; y -= f[13]; z -= f[13];
    r += f[14]; y += f[14]; z -= f[14];
    r += f[15]; y -= f[15]; z += f[15];
    r += f[16]; z += f[16];
    r += f[17]; z -= f[17];
    r += f[18];
    *rho = r; *vx = x; *vy = y; *vz = z;
}

/* Incompressible BGK equilibrium of src/common.h:132-160 for the 19
 * directions: feq_k = w_k*((P + 3 s) + 4.5 s^2) with P = rho - 1.5 |j|^2 and
 * s = c_k . j, evaluated left to right exactly as the macros expand. */
static void SFX(equilibrium)(REAL rho, REAL vx, REAL vy, REAL vz, REAL* e)
{
    const REAL vel2 = vx * vx + vy * vy + vz * vz;
    const REAL P = rho - ((REAL)3 / (REAL)2) * vel2;
    REAL s, s2;

    s2 = vx * vx;
    e[0] = W_AXIS * (P + (REAL)3 * vx + ((REAL)9 / (REAL)2) * s2);
    e[1] = W_AXIS * (P + (REAL)-3 * vx + ((REAL)9 / (REAL)2) * s2);
    s2 = vy * vy;
    e[2] = W_AXIS * (P + (REAL)3 * vy + ((REAL)9 / (REAL)2) * s2);
    e[3] = W_AXIS * (P + (REAL)-3 * vy + ((REAL)9 / (REAL)2) * s2);

    s = vx + vy; s2 = s * s;
    e[4] = W_DIAG * (P + (REAL)3 * s + ((REAL)9 / (REAL)2) * s2);
    e[5] = W_DIAG * (P + (REAL)-3 * s + ((REAL)9 / (REAL)2) * s2);
    s = vx - vy; s2 = s * s;
    e[6] = W_DIAG * (P + (REAL)3 * s + ((REAL)9 / (REAL)2) * s2);
    e[7] = W_DIAG * (P + (REAL)-3 * s + ((REAL)9 / (REAL)2) * s2);

    s = vx + vz; s2 = s * s;
    e[8] = W_DIAG * (P + (REAL)3 * s + ((REAL)9 / (REAL)2) * s2);
    e[9] = W_DIAG * (P + (REAL)-3 * s + ((REAL)9 / (REAL)2) * s2);
    s = vx - vz; s2 = s * s;
    e[10] = W_DIAG * (P + (REAL)3 * s + ((REAL)9 / (REAL)2) * s2);
    e[11] = W_DIAG * (P + (REAL)-3 * s + ((REAL)9 / (REAL)2) * s2);

    s = vy + vz; s2 = s * s;
    e[12] = W_DIAG * (P + (REAL)3 * s + ((REAL)9 / (REAL)2) * s2);
    e[13] = W_DIAG * (P + (REAL)-3 * s + ((REAL)9 / (REAL)2) * s2);
    s = vy - vz; s2 = s * s;
    e[14] = W_DIAG * (P + (REAL)3 * s + ((REAL)9 / (REAL)2) * s2);
    e[15] = W_DIAG * (P + (REAL)-3 * s + ((REAL)9 / (REAL)2) * s2);

    s2 = vz * vz;
    e[16] = W_AXIS * (P + (REAL)3 * vz + ((REAL)9 / (REAL)2) * s2);
    e[17] = W_AXIS * (P + (REAL)-3 * vz + ((REAL)9 / (REAL)2) * s2);
    e[18] = W_REST * P;
}

/* The alpha kernel's gravity term (src/gpukernels/lbm_alpha.cu:213-326).  The
 * reference stores each term in `tmp`, which is `#define`d to `rho`
 * (lbm_alpha.cu:203), so every term after the first is scaled by the previous
 * term instead of by the density.  That chain is reproduced as written.  The
 * pair order (1,0),(3,2),...,(17,16) and signs follow the source. */
static void SFX(alpha_gravity)(REAL* f, REAL rho, REAL gx, REAL gy, REAL gz)
{
    REAL t = gx * W_AXIS * rho;           f[1] -= t;  f[0] += t;
    t = gy * ((REAL)-1 / (REAL)18) * t;    f[3] -= t;  f[2] += t;
    t = (gx - gy) * W_DIAG * t;            f[5] -= t;  f[4] += t;
    t = (gx + gy) * W_DIAG * t;            f[7] -= t;  f[6] += t;
    t = (gx + gz) * W_DIAG * t;            f[9] -= t;  f[8] += t;
    t = (gx - gz) * W_DIAG * t;            f[11] -= t; f[10] += t;
    t = (gz - gy) * W_DIAG * t;            f[13] -= t; f[12] += t;
    t = (gz + gy) * ((REAL)-1 / (REAL)36) * t; f[15] -= t; f[14] += t;
    t = gz * W_AXIS * t;                   f[17] -= t; f[16] += t;
}

/* FLUID collision in place: f_k += inv_tau*(feq_k - f_k)
 * (src/gpukernels/lbm_alpha.cu:209-331, src/gpukernels/lbm_beta.cu:574-636). */
static void SFX(collide_fluid)(REAL* f, REAL inv_tau, int gravity, REAL gx, REAL gy, REAL gz)
{
    REAL rho, vx, vy, vz, e[19];
    int k;
    SFX(moments)(f, &rho, &vx, &vy, &vz);
    SFX(equilibrium)(rho, vx, vy, vz, e);
    for (k = 0; k < 19; ++k)
        f[k] += inv_tau * (e[k] - f[k]);
    if (gravity)
        SFX(alpha_gravity)(f, rho, gx, gy, gz);
}

/* VELOCITY_INJECTION: populations reset to feq(rho=1, j=(U,0,0))
 * (src/gpukernels/lbm_alpha.cu:376-511, src/gpukernels/lbm_beta.cu:661-732). */
static void SFX(inject)(REAL* f, REAL lid_u, int gravity, REAL gx, REAL gy, REAL gz)
{
    SFX(equilibrium)((REAL)1, lid_u, (REAL)0, (REAL)0, f);
    if (gravity)
        SFX(alpha_gravity)(f, (REAL)1, gx, gy, gz);
}

void SFX(orc_init_)(REAL* dd, int32_t* flags, int nx, int ny, int nz, const int32_t bc[6])
{
    /* src/gpukernels/lbm_init.cu:41-208: flags from the six face conditions
     * (an OBSTACLE face wins over later faces), populations at rest. */
    const int X = nx + 2, Y = ny + 2, Z = nz + 2;
    const int64_t C = (int64_t)X * Y * Z;
    REAL e[19];
    int64_t gid;
    int k;
    SFX(equilibrium)((REAL)1, (REAL)0, (REAL)0, (REAL)0, e);
    for (gid = 0; gid < C; ++gid) {
        const int x = (int)(gid % X), y = (int)((gid / X) % Y), z = (int)(gid / ((int64_t)X * Y));
        int32_t fl = ORC_FLUID;
        if (x == 0) fl = bc[0];
        if (x == X - 1 && fl != ORC_OBSTACLE) fl = bc[1];
        if (y == 0 && fl != ORC_OBSTACLE) fl = bc[2];
        if (y == Y - 1 && fl != ORC_OBSTACLE) fl = bc[3];
        if (z == 0 && fl != ORC_OBSTACLE) fl = bc[4];
        if (z == Z - 1 && fl != ORC_OBSTACLE) fl = bc[5];
        flags[gid] = fl;
        for (k = 0; k < 19; ++k)
            dd[k * C + gid] = e[k];
    }
}

/* The GB300 solver's opt-in moving top wall (no reference counterpart): a
 * FLUID cell of row y = ny reads populations 5 (-x-y) and 6 (+x-y) that the
 * obstacle cells above it (the top face, moving at U along x) sent back as
 * bounced populations 4 (+x+y) and 7 (-x+y).  Ladd's moving-wall rule
 * f_opp(i) = f_i - 6 w_i (c_i . U) (rho_w = 1) adds -U/6 to 5 and +U/6 to 6,
 * each only where that link ends in an OBSTACLE cell. */
static void SFX(wall_correct)(REAL* f, const int32_t* flags, int64_t gid, int64_t X, REAL du)
{
    if (flags[gid + 1 + X] == ORC_OBSTACLE) f[5] -= du;
    if (flags[gid - 1 + X] == ORC_OBSTACLE) f[6] += du;
}

static void SFX(alpha_impl)(REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                            REAL inv_tau, REAL gx, REAL gy, REAL gz, REAL lid_u,
                            const int32_t origin[3], const int32_t size[3], int wall)
{
    /* src/gpukernels/lbm_alpha.cu:22-532: read the 19 slots of a cell, collide,
     * write population k into slot opp(k) of the same cell. */
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    const int gravity = (gx != (REAL)0) || (gy != (REAL)0) || (gz != (REAL)0);
    const REAL du = lid_u * ((REAL)1 / (REAL)6);
    int Zi;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (Zi = 0; Zi < size[2]; ++Zi) {
        int Yi, Xi, k;
        REAL f[19];
        for (Yi = 0; Yi < size[1]; ++Yi) {
            for (Xi = 0; Xi < size[0]; ++Xi) {
                const int64_t gid = (origin[2] + Zi) * XY + (origin[1] + Yi) * X + origin[0] + Xi;
                int32_t fl;
                if (gid >= C) continue;
                fl = flags[gid];
                if (fl != ORC_FLUID && fl != ORC_VELOCITY_INJECTION) continue;
                if (fl == ORC_FLUID) {
                    for (k = 0; k < 19; ++k) f[k] = dd[k * C + gid];
                    if (wall && origin[1] + Yi == ny && origin[0] + Xi >= 1 && origin[0] + Xi <= nx &&
                        origin[2] + Zi >= 1 && origin[2] + Zi <= nz)
                        SFX(wall_correct)(f, flags, gid, X, du);
                    SFX(collide_fluid)(f, inv_tau, gravity, gx, gy, gz);
                } else {
                    SFX(inject)(f, lid_u, gravity, gx, gy, gz);
                }
                for (k = 0; k < 18; ++k) dd[(k ^ 1) * C + gid] = f[k];
                dd[18 * C + gid] = f[18];
            }
        }
    }
}

void SFX(orc_alpha_)(REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                     REAL inv_tau, REAL gx, REAL gy, REAL gz, REAL lid_u,
                     const int32_t origin[3], const int32_t size[3])
{
    SFX(alpha_impl)(dd, flags, nx, ny, nz, inv_tau, gx, gy, gz, lid_u, origin, size, 0);
}

void SFX(orc_alpha_wall_)(REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                          REAL inv_tau, REAL gx, REAL gy, REAL gz, REAL lid_u,
                          const int32_t origin[3], const int32_t size[3])
{
    SFX(alpha_impl)(dd, flags, nx, ny, nz, inv_tau, gx, gy, gz, lid_u, origin, size, 1);
}

/* Linear-index neighbour offset of direction k, as the beta kernel forms it
 * (src/gpukernels/lbm_beta.cu:59-64, 98-231): the position of slot k that cell
 * gid reads and writes is (gid + delta_k) mod C (DOMAIN_WRAP, lbm_beta.cu:22-25). */
static int64_t SFX(beta_delta)(int k, int64_t X, int64_t XY, int64_t C)
{
    static const int cx[19] = {1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0};
    static const int cy[19] = {0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0};
    static const int cz[19] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0};
    int64_t d = 0;
    d += cx[k] > 0 ? 1 : (cx[k] < 0 ? C - 1 : 0);
    d += cy[k] > 0 ? X : (cy[k] < 0 ? C - X : 0);
    d += cz[k] > 0 ? XY : (cz[k] < 0 ? C - XY : 0);
    return d;
}

static void SFX(beta_impl)(REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                           REAL inv_tau, REAL lid_u,
                           const int32_t origin[3], const int32_t size[3], int wall)
{
    /* src/gpukernels/lbm_beta.cu:32-915 (USE_SHARED_MEMORY 0, GRAVITATION 0):
     * population opp(k) arrives from slot k at gid+delta_k; after the
     * collision, population k is written to the same address.  OBSTACLE swaps
     * each pair before the write, which restores what it read. */
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    const REAL du = lid_u * ((REAL)1 / (REAL)6);
    int64_t delta[19];
    int Zi, k0;
    for (k0 = 0; k0 < 19; ++k0) delta[k0] = SFX(beta_delta)(k0, X, XY, C);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (Zi = 0; Zi < size[2]; ++Zi) {
        int Yi, Xi, k;
        REAL f[19], t;
        int64_t pos[19];
        for (Yi = 0; Yi < size[1]; ++Yi) {
            for (Xi = 0; Xi < size[0]; ++Xi) {
                const int64_t gid = (origin[2] + Zi) * XY + (origin[1] + Yi) * X + origin[0] + Xi;
                int32_t fl;
                if (gid >= C) continue;
                fl = flags[gid];
                for (k = 0; k < 19; ++k) pos[k] = k * C + (gid + delta[k]) % C;
                /* the value in slot k at gid+delta_k is population opp(k) */
                for (k = 0; k < 18; ++k) f[k ^ 1] = dd[pos[k]];
                f[18] = dd[pos[18]];
                if (fl == ORC_FLUID) {
                    if (wall && origin[1] + Yi == ny && origin[0] + Xi >= 1 && origin[0] + Xi <= nx &&
                        origin[2] + Zi >= 1 && origin[2] + Zi <= nz)
                        SFX(wall_correct)(f, flags, gid, X, du);
                    SFX(collide_fluid)(f, inv_tau, 0, 0, 0, 0);
                } else if (fl == ORC_OBSTACLE) {
                    for (k = 0; k < 18; k += 2) { t = f[k]; f[k] = f[k + 1]; f[k + 1] = t; }
                } else if (fl == ORC_VELOCITY_INJECTION) {
                    SFX(inject)(f, lid_u, 0, 0, 0, 0);
                }
                for (k = 0; k < 19; ++k) dd[pos[k]] = f[k];
            }
        }
    }
}

void SFX(orc_beta_)(REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                    REAL inv_tau, REAL lid_u,
                    const int32_t origin[3], const int32_t size[3])
{
    SFX(beta_impl)(dd, flags, nx, ny, nz, inv_tau, lid_u, origin, size, 0);
}

void SFX(orc_beta_wall_)(REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                         REAL inv_tau, REAL lid_u,
                         const int32_t origin[3], const int32_t size[3])
{
    SFX(beta_impl)(dd, flags, nx, ny, nz, inv_tau, lid_u, origin, size, 1);
}

/* Post-collision populations of interior cell gid after the last step: after
 * alpha they sit swapped in the cell's own slots; after beta (or init) they
 * sit in slot k of the neighbour gid + c_k. */
static void SFX(post_pops)(const REAL* dd, int64_t gid, int64_t X, int64_t XY, int64_t C,
                           int last_was_alpha, REAL* f)
{
    static const int cx[19] = {1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0};
    static const int cy[19] = {0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0};
    static const int cz[19] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0};
    int k;
    if (last_was_alpha) {
        for (k = 0; k < 18; ++k) f[k] = dd[(k ^ 1) * C + gid];
        f[18] = dd[18 * C + gid];
    } else {
        for (k = 0; k < 19; ++k) f[k] = dd[k * C + gid + cx[k] + cy[k] * X + cz[k] * XY];
    }
}

void SFX(orc_macros_)(const REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                      int last_was_alpha, REAL lid_u, REAL* rho, REAL* jx, REAL* jy, REAL* jz)
{
    /* Density and momentum of the time level that was collided last, on the
     * full (nx+2)(ny+2)(nz+2) grid.  FLUID cells: moments of their
     * post-collision populations in the reference summation order.  Lid cells
     * report the imposed (1, U, 0, 0) as the reference's stores do
     * (src/gpukernels/lbm_beta.cu:661-667); walls and halo report zero
     * ("zero velocity and no fluid density", lbm_beta.cu:639-640). */
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    int z;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (z = 0; z < nz + 2; ++z) {
        int y, x;
        REAL f[19], r, vx, vy, vz;
        for (y = 0; y < ny + 2; ++y) {
            for (x = 0; x < nx + 2; ++x) {
                const int64_t gid = z * XY + y * X + x;
                const int interior = x >= 1 && x <= nx && y >= 1 && y <= ny && z >= 1 && z <= nz;
                const int32_t fl = flags[gid];
                r = vx = vy = vz = (REAL)0;
                if (interior && fl == ORC_FLUID) {
                    SFX(post_pops)(dd, gid, X, XY, C, last_was_alpha, f);
                    SFX(moments)(f, &r, &vx, &vy, &vz);
                } else if (interior && fl == ORC_VELOCITY_INJECTION) {
                    r = (REAL)1; vx = lid_u;
                }
                rho[gid] = r; jx[gid] = vx; jy[gid] = vy; jz[gid] = vz;
            }
        }
    }
}

void SFX(orc_reduce_)(const REAL* dd, const int32_t* flags, int nx, int ny, int nz,
                      int last_was_alpha, double out[4])
{
    /* FP64 totals.  out[0] is the mass held by every live slot: the 19 own
     * slots of each interior FLUID or lid cell, plus the slots of inactive
     * neighbours (walls) that the cell's pushes land in, where a population
     * waits one step before it returns.  Collision, streaming and the walls
     * conserve this sum exactly.  out[1..3] is the momentum of the cells'
     * post-collision populations.  Summed per z-plane, then the planes in
     * order, so the result does not depend on the thread count. */
    static const int cx[19] = {1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0};
    static const int cy[19] = {0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0};
    static const int cz[19] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0};
    const int64_t X = nx + 2, XY = (int64_t)(nx + 2) * (ny + 2);
    const int64_t C = XY * (nz + 2);
    double* part = (double*)calloc((size_t)4 * (nz + 2), sizeof(double));
    int z, q;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (z = 1; z <= nz; ++z) {
        int y, x, k;
        REAL f[19];
        double m = 0, px = 0, py = 0, pz = 0;
        for (y = 1; y <= ny; ++y) {
            for (x = 1; x <= nx; ++x) {
                const int64_t gid = z * XY + y * X + x;
                const int32_t fl = flags[gid];
                if (fl != ORC_FLUID && fl != ORC_VELOCITY_INJECTION) continue;
                for (k = 0; k < 19; ++k) {
                    const int64_t nb = gid + cx[k] + cy[k] * X + cz[k] * XY;
                    const int32_t fn = flags[nb];
                    m += (double)dd[k * C + gid];
                    if (fn != ORC_FLUID && fn != ORC_VELOCITY_INJECTION) m += (double)dd[k * C + nb];
                }
                SFX(post_pops)(dd, gid, X, XY, C, last_was_alpha, f);
                for (k = 0; k < 19; ++k) {
                    const double v = (double)f[k];
                    px += cx[k] * v; py += cy[k] * v; pz += cz[k] * v;
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

#undef W_AXIS
#undef W_DIAG
#undef W_REST
