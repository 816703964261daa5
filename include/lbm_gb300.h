/*
 * lbm_gb300.h -- C ABI of the GB300-native D3Q19 A-A lattice-Boltzmann
 * lid-driven-cavity solver (drop-in for the solver of
 * saleemayman/cavityflow_cuda).
 *
 * Every entry point is plain C: opaque handles, integer status codes, plain
 * pointers and sizes.  Nothing here exits the process; where the reference
 * asserts or calls exit() the call returns a status instead (see
 * lbm_status_string and lbm_last_error).
 *
 * Conventions shared with the reference solver interface
 * (src/CLbmSolver.hpp:30-89, src/CLbmSolverGPU.cuh:25-95):
 *   - A domain of nx*ny*nz interior cells carries a one-cell halo, so
 *     "halo coordinates" run 0..n+1 on each axis.  Cuboid arguments
 *     (origin, size) are in halo coordinates; passing NULL for both selects
 *     the interior, origin (1,1,1) and size (nx,ny,nz)
 *     (src/CLbmSolverGPU.cu:597-604).
 *   - Host buffers are packed [component][z][y][x], x fastest, with
 *     size[0]*size[1]*size[2] elements per component: 19 components for
 *     populations, 3 for velocities, 1 for densities and flags.
 *   - Host values have the solver's value type: double for LBM_STORAGE_F64,
 *     float for every other storage (lbm_value_size()).
 *   - Population slots are returned raw, as the reference does: after an
 *     alpha step they are in the swapped (opposite-slot) convention.
 *   - `stream` is a cudaStream_t passed as void*; NULL is the legacy default
 *     stream, as a NULL cudaStream_t* is in the reference.
 *
 * Lattice directions, flag values and directions of the direction-filtered
 * copy are the reference's (src/common.h:29-71).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_GB300_ABI_VERSION 2

/* ---- status codes -------------------------------------------------------- */
typedef enum lbm_status {
    LBM_OK = 0,
    LBM_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size, enum or flag value        */
    LBM_ERR_OUT_OF_BOUNDS = 2,    /* cuboid outside the domain (reference: assert) */
    LBM_ERR_CUDA = 3,             /* a CUDA runtime call or launch failed          */
    LBM_ERR_OUT_OF_MEMORY = 4,    /* device or pinned-host allocation failed       */
    LBM_ERR_UNSUPPORTED = 5,      /* valid request this build does not provide     */
    LBM_ERR_CONFIG = 6,           /* no stable time step (reference: exit()), or a
                                     configuration file the reader rejects        */
    LBM_ERR_IO = 7,               /* file could not be read or written             */
    LBM_ERR_BUDGET = 8,           /* request does not fit the memory budget        */
    LBM_ERR_NOT_READY = 9,        /* result requested before it exists             */
    LBM_ERR_NO_DEVICE = 10,       /* no CUDA device visible                        */
    LBM_ERR_TIMEOUT = 11          /* a kernel gave up a bounded device-side wait   */
} lbm_status;

/* Flag values, src/common.h:54-61. */
enum { LBM_OBSTACLE = 1, LBM_FLUID = 2, LBM_VELOCITY_INJECTION = 4, LBM_GHOST_LAYER = 8 };

/* Faces of the direction-filtered population copy, src/common.h:63-71.
 * LBM_DIRECTION_ALL selects the unfiltered copy. */
enum { LBM_DIRECTION_ALL = -1, LBM_LEFT = 0, LBM_RIGHT = 1, LBM_BOTTOM = 2, LBM_TOP = 3,
       LBM_BACK = 4, LBM_FRONT = 5 };

/* Storage precision of the population array.  F64 and F32 reproduce the
 * reference kernels' arithmetic exactly.  F16S, BF16S and F16SR store the
 * deviation f_i - w_i in 16 bits and collide in FP32 registers; F16S and
 * BF16S round to nearest, F16SR keeps IEEE half values of the deviation
 * times 2^12 and rounds the time steps' stores stochastically, with a dither
 * keyed by (cell, population, step), so that results are reproducible.
 * Rounding to nearest biases slowly changing populations; stochastic
 * rounding does not, and is several times more accurate against an FP64 run
 * at the same 2 bytes per value. */
typedef enum lbm_storage {
    LBM_STORAGE_F64 = 0,
    LBM_STORAGE_F32 = 1,
    LBM_STORAGE_F16S = 2,
    LBM_STORAGE_BF16S = 3,
    LBM_STORAGE_F16SR = 4
} lbm_storage;

/* How the lid drives the cavity (lbm_params.lid_mode).
 *
 * LBM_LID_INJECTION (default) is the reference's lid: lbm_set_driven_cavity
 * marks the interior plane y = ny as VELOCITY_INJECTION, and every step
 * resets those cells to feq(rho = 1, u = (U, 0, 0))
 * (src/CController.cpp:1289-1348, src/gpukernels/lbm_alpha.cu:376-511,
 * src/gpukernels/lbm_beta.cu:661-732).  The reset adds or removes mass, so
 * the total mass drifts.
 *
 * LBM_LID_MOVING_WALL has no counterpart in the reference: the top face
 * y = ny + 1 is a wall moving at U along x, and the interior plane y = ny
 * stays FLUID.  Populations the wall sends back to the fluid carry Ladd's
 * moving-wall correction -6 w_i (c_i . U) (rho_w = 1).  Both corrections of a
 * cell cancel, so the total mass of lbm_reduce is conserved to rounding
 * (FP64: 1e-10 relative and far below).  lbm_set_driven_cavity starts the wall
 * moving and touches no flags.  The top face must be OBSTACLE. */
enum { LBM_LID_INJECTION = 0, LBM_LID_MOVING_WALL = 1 };

/* ---- parameters ----------------------------------------------------------- */

/* Physical description, the fields of the reference's XML configuration
 * that its solver base class reads (src/CConfiguration.hpp:57-104). */
typedef struct lbm_physical {
    double velocity[3];         /* lid velocity (m/s); only x drives the lid  */
    double acceleration[3];     /* external acceleration (m/s^2)              */
    double viscosity;           /* m^2/s; <= 0 selects the Re=1000 default    */
    double max_velocity;        /* max dimensionless velocity                 */
    double max_acceleration;    /* max dimensionless acceleration             */
    int32_t domain_size[3];     /* cells                                      */
    double domain_length[3];    /* m                                          */
    double timestep;            /* s                                          */
} lbm_physical;

/* Lattice-unit parameters the solver runs on. */
typedef struct lbm_lattice {
    double timestep;            /* possibly rescaled time step (s)            */
    double tau;                 /* BGK relaxation time                        */
    double inv_tau;             /* 1/tau as the kernels use it                */
    double velocity[3];         /* dimensionless velocity; [0] drives the lid */
    double acceleration[3];     /* dimensionless gravity of the alpha step    */
    double viscosity;           /* dimensionless viscosity                    */
} lbm_lattice;

/* Derives lattice parameters from physical ones exactly as
 * CLbmSolver<T>::CLbmSolver does (src/CLbmSolver.cpp:28-327), in the
 * precision of `storage` (double for F64, float otherwise): default viscosity
 * from Re = 1000, time-step rescaling for velocity, acceleration and tau
 * limits [0.51, 1.9] (src/constants.h:26-30).  Where the reference exit()s
 * (no stable time step) this returns LBM_ERR_CONFIG.  Replaces the
 * constructor body of src/CLbmSolver.cpp:28-327. */
int lbm_derive_lattice(const lbm_physical* phys, int32_t storage, lbm_lattice* out);

/* The reference's XML configuration (configurations/*.xml), field for field
 * (src/CConfiguration.hpp:57-104).  As in the reference built without MPI,
 * subdomain-num is not read: subdomain_num is 1, 1, 1 and the domain is one
 * subdomain on one GPU. */
typedef struct lbm_configuration {
    double velocity[3];
    double acceleration[3];
    double viscosity;
    double max_velocity;
    double max_acceleration;
    int32_t domain_size[3];
    int32_t subdomain_num[3];
    double domain_length[3];
    double cpu_subdomain_ratio;
    double timestep;
    int32_t loops;
    int32_t do_benchmark;
    int32_t do_logging;
    int32_t do_validation;
    int32_t do_visualization;
    int32_t visualization_rate;
    int32_t cpu_alpha_block[3];
    int32_t cpu_beta_block[3];
    int32_t gpu_init_block[3];
    int32_t gpu_alpha_block[3];
    int32_t gpu_beta_block[3];
    int32_t reserved;
    char benchmark_dir[256];
    char logging_dir[256];
    char validation_dir[256];
    char visualization_dir[256];
} lbm_configuration;

/* Reads an XML configuration with the reference's schema.  Replaces
 * CConfiguration<T>::CConfiguration (src/CConfiguration.cpp:28-172); its
 * parameter checks (:174-197, asserts there) return LBM_ERR_CONFIG, a file
 * that cannot be read LBM_ERR_IO. */
int lbm_read_configuration(const char* path, lbm_configuration* out);
/* The physical description lbm_derive_lattice takes, from a configuration. */
int lbm_configuration_physical(const lbm_configuration* config, lbm_physical* out);

/* Creation parameters of one solver. */
typedef struct lbm_params {
    int32_t size[3];            /* interior cells nx, ny, nz (domain-size):
                                   each in [1, 2^20], (nx+2)(ny+2)(nz+2) at
                                   most 2^40 (batches: all domains together,
                                   servers: each request)                      */
    int32_t storage;            /* lbm_storage                                 */
    int32_t boundary[6];        /* face flags: -x, +x, -y, +y, -z, +z
                                   (src/CLbmSolver.hpp:36-45)                  */
    double inv_tau;             /* 1/tau                                       */
    double lid_velocity;        /* x velocity imposed on injection cells       */
    double gravity[3];          /* dimensionless acceleration (alpha step)     */
    int32_t device;             /* CUDA device ordinal; the reference picks
                                   id % nGPUs (src/CLbmSolverGPU.cu:42-45)     */
    int32_t fast_variant;       /* 0: library default; v + 1 selects launch
                                   variant v of the vectorised kernels,
                                   v < lbm_fast_variant_count(); see
                                   lbm_autotune                                */
    int32_t fused_multiply_add; /* F64 and F32 storage.  0 (default): the
                                   collision performs the reference CPU
                                   kernels' unfused IEEE operations (results
                                   bit-identical to them).  1: the vectorised
                                   register-variant steps fuse its
                                   multiply-adds (and FP32 flushes subnormals),
                                   as the reference's nvcc build
                                   (-use_fast_math) does: the closest match to
                                   the reference CUDA kernels, and faster on
                                   GB300's FP64 units; no longer
                                   bit-identical to the CPU kernels.
                                   Flag-array and bulk-copy steps stay
                                   unfused.                                    */
    int32_t lid_mode;           /* LBM_LID_INJECTION (0, the reference's lid)
                                   or LBM_LID_MOVING_WALL                      */
} lbm_params;

typedef struct lbm_solver lbm_solver;   /* opaque */

/* Information about a live solver. */
typedef struct lbm_info {
    int32_t size[3];            /* interior cells                              */
    int32_t storage;
    int32_t value_size;         /* bytes per host value (4 or 8)               */
    int32_t vector_cells;       /* cells per widest vector the rows are sized
                                   for: 16 bytes, 8 in batch and server rows  */
    int64_t step_counter;       /* steps taken (alpha on even, beta on odd)    */
    int32_t last_step_was_alpha;
    int32_t fast_path;          /* 1: flags match the box cavity, so the
                                   vectorised kernels run; 0: flag-array path  */
    int32_t fast_variant;       /* launch variant of the vectorised kernels    */
    int32_t cells_per_thread;   /* cells per thread of its alpha kernel        */
    int32_t block_threads;      /* threads per block of its alpha kernel       */
    int32_t beta_cells_per_thread;  /* the same for its beta kernel            */
    int32_t beta_block_threads;
    int32_t beta_block_exchange;    /* how beta gets the one-cell-shifted
                                       slots: 0 warp shuffles (beta_fast), 1
                                       across the block (beta_fast_blk), 2 no
                                       exchange (beta_fast_direct), 3 no
                                       exchange with two 16-bit cells per
                                       register (beta_fast_pk)                 */
    int32_t fused_multiply_add;     /* lbm_params.fused_multiply_add           */
    int64_t row_pitch;          /* elements per padded x row on the device     */
    int64_t slot_stride;        /* elements per population slot                */
    int64_t device_bytes;       /* bytes of device memory the solver holds     */
    int64_t x1_column;          /* column of interior cell x = 1 in a row: 32
                                   bytes in (the default), or 8 for the
                                   packed rows of batch domains               */
    int32_t lid_mode;           /* lbm_params.lid_mode                         */
    int32_t moving_wall;        /* 1 while the top wall moves (moving-wall
                                   mode after lbm_set_driven_cavity)           */
} lbm_info;

/* ---- lifecycle ------------------------------------------------------------ */

/* Allocates the population and flag arrays on `params->device` and
 * initialises them: flags from the six face conditions, populations at rest
 * (rho = 1, u = 0).  Replaces CLbmSolverGPU<T>::CLbmSolverGPU
 * (src/CLbmSolverGPU.cu:30-160) and the lbm_init kernel
 * (src/gpukernels/lbm_init.cu:41-208). */
int lbm_create(const lbm_params* params, lbm_solver** out);

/* Frees everything the solver holds.  Replaces
 * CLbmSolverGPU<T>::~CLbmSolverGPU (src/CLbmSolverGPU.cu:162-171). */
int lbm_destroy(lbm_solver* solver);

int lbm_get_info(const lbm_solver* solver, lbm_info* info);

/* Interior size, replacing CLbmSolver<T>::getDomain()->getSize()
 * (src/CLbmSolver.cpp:329-333). */
int lbm_get_domain(const lbm_solver* solver, int32_t size[3]);

/* Bytes per host value: 8 for F64 storage, 4 otherwise. */
int lbm_value_size(const lbm_solver* solver);

/* Marks the lid plane y = ny (x in [1,nx], z in [1,nz]) as
 * VELOCITY_INJECTION.  Replaces CController<T>::setDrivenCavitySzenario
 * (src/CController.cpp:1289-1348).  In LBM_LID_MOVING_WALL mode it sets the
 * top wall moving instead and changes no flag. */
int lbm_set_driven_cavity(lbm_solver* solver);

/* ---- time steps -------------------------------------------------------------
 * Kernels are queued on `stream` and the call returns without waiting, as in
 * the reference. */

/* Whole domain.  Replaces CLbmSolverGPU<T>::simulationStepAlpha(stream)
 * (src/CLbmSolverGPU.cu:173-248). */
int lbm_step_alpha(lbm_solver* solver, void* stream);
/* Cuboid in halo coordinates.  Replaces simulationStepAlpha(origin, size,
 * stream) (src/CLbmSolverGPU.cu:250-337). */
int lbm_step_alpha_cuboid(lbm_solver* solver, const int32_t origin[3], const int32_t size[3],
                          void* stream);
/* Replaces simulationStepBeta(stream) (src/CLbmSolverGPU.cu:339-419). */
int lbm_step_beta(lbm_solver* solver, void* stream);
/* Replaces simulationStepBeta(origin, size, stream)
 * (src/CLbmSolverGPU.cu:421-513). */
int lbm_step_beta_cuboid(lbm_solver* solver, const int32_t origin[3], const int32_t size[3],
                         void* stream);

/* `steps` time steps, alpha on an even counter and beta on an odd one,
 * replacing the loop of CController<T>::run / computeNextStep
 * (src/CController.cpp:1278-1287, :1407-1412).  Long runs replay a CUDA
 * graph of captured alpha/beta pairs. */
int lbm_run(lbm_solver* solver, int64_t steps, void* stream);

/* Waits for all work queued by the solver.  LBM_ERR_TIMEOUT if one of its
 * kernels gave up a bounded device-side wait (the solver stays usable). */
int lbm_synchronize(lbm_solver* solver);

/* Diagnostics of that failure path, with no GPU fault: runs on the solver's
 * device one block that waits on an mbarrier nothing arrives at, with the
 * bulk-copy kernels' bounded wait (limit_us in [1, 2000000] microseconds
 * instead of their 2 s), raising the solver's error flag when it gives up;
 * then synchronises.  Returns LBM_ERR_TIMEOUT, after which the solver's
 * state and later steps are unaffected. */
int lbm_selftest_bounded_wait(lbm_solver* solver, int32_t limit_us);

/* ---- tuning (no counterpart in the reference, whose block shape comes from
 * the XML gpu/grid-configuration, src/CConfiguration.cpp:150-160) ---------- */

/* Number of launch variants of the box-cavity kernels: 24 register-blocked
 * vector kernels (0..23: cells per thread, threads per block and blocks per
 * SM of the alpha and the beta kernel, and whether beta exchanges edge
 * elements per warp, per block or not at all; 18..23 keep 16-bit populations
 * two cells per register) and 6 row-pipelined bulk-copy kernels (24..29: rows
 * per unit, buffers, consumer warps). */
int lbm_fast_variant_count(void);
/* Number of register variants (the first variants; the batch kernel's menu). */
int lbm_register_variant_count(void);
/* Selects a variant for subsequent steps; LBM_ERR_UNSUPPORTED if it needs more
 * shared memory than this domain allows. */
int lbm_set_fast_variant(lbm_solver* solver, int32_t variant);
/* Times every variant that fits this solver's domain (`pairs` alpha/beta pairs
 * each, CUDA events; -1 for a variant that does not fit) and selects the
 * fastest.  The populations are saved to a
 * temporary device buffer first and restored afterwards, so the simulation
 * state and step counter are unchanged.  ms_per_pair (optional) receives one
 * time per variant.  Synchronous. */
int lbm_autotune(lbm_solver* solver, int32_t pairs, int32_t* best, float* ms_per_pair);

/* ---- data access ------------------------------------------------------------ */

/* Raw population slots of a cuboid to host, asynchronous on `stream` like
 * the reference's cudaMemcpy3DAsync.  Replaces getDensityDistributions
 * (src/CLbmSolverGPU.cu:515-611). */
int lbm_get_density_distributions(lbm_solver* solver, const int32_t origin[3], const int32_t size[3],
                                  void* host, void* stream);
/* Host to raw population slots of a cuboid.  `direction` LBM_DIRECTION_ALL
 * copies all 19 slots (src/CLbmSolverGPU.cu:745-819); a face value copies
 * only the slots whose lattice vector points into the domain from that face
 * (src/CLbmSolverGPU.cu:613-714).  Host layout is 19 packed components
 * either way. */
int lbm_set_density_distributions(lbm_solver* solver, const int32_t origin[3], const int32_t size[3],
                                  int32_t direction, const void* host, void* stream);

/* Flags of a cuboid (int32 per cell, the Flag enum).  Synchronous, as the
 * reference's cudaMemcpy3D.  Replaces getFlags/setFlags
 * (src/CLbmSolverGPU.cu:821-985).  setFlags accepts only the four Flag
 * values and switches the solver between the vectorised and the
 * flag-array kernels as needed. */
int lbm_get_flags(lbm_solver* solver, const int32_t origin[3], const int32_t size[3], int32_t* host);
int lbm_set_flags(lbm_solver* solver, const int32_t origin[3], const int32_t size[3], const int32_t* host);

/* Velocity (3 components, the incompressible form u = j) and density of a
 * cuboid, synchronous.  The values are those of the time level collided
 * last, computed on demand from the populations; lid cells report
 * (1, U, 0, 0) and obstacle and halo cells zero.  Values written by the
 * setters are returned by the getters until the next time step, which
 * recomputes them, as the reference's stored arrays behave.  Replace
 * get/setVelocities and get/setDensities (src/CLbmSolverGPU.cu:987-1327). */
int lbm_get_velocities(lbm_solver* solver, const int32_t origin[3], const int32_t size[3], void* host);
int lbm_set_velocities(lbm_solver* solver, const int32_t origin[3], const int32_t size[3], const void* host);
int lbm_get_densities(lbm_solver* solver, const int32_t origin[3], const int32_t size[3], void* host);
int lbm_set_densities(lbm_solver* solver, const int32_t origin[3], const int32_t size[3], const void* host);

/* FP64 totals over interior FLUID and lid cells of the post-collision
 * populations of the last step: out = {mass, momentum x, y, z}.  A
 * deterministic two-pass reduction; synchronous.  No counterpart in the
 * reference (it has no reduction); it carries the mass-conservation check. */
int lbm_reduce(lbm_solver* solver, double out[4], void* stream);

/* FP64 {mass, momentum x, y, z} of population and flag arrays the CALLER
 * owns, written to `out_device` (4 doubles in device memory the caller owns),
 * with no device or host allocation.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: programs whose device memory is all
 * handed out by their own pool or caching allocator, or that admit work
 * against a fixed HBM budget, and time loops that cannot take the implicit
 * device synchronisation of cudaMalloc/cudaFree.  Same sums as lbm_reduce.
 *
 * Inputs are in the reference's layout: `populations` holds 19 slots of
 * (nx+2)*(ny+2)*(nz+2) values (double for LBM_STORAGE_F64, float for
 * LBM_STORAGE_F32), x fastest; `flags` one int32 Flag per cell;
 * `last_step_was_alpha` selects where the post-collision populations sit.
 * Queued on `stream`; read `out_device` after that stream completes.
 *
 * Scratch is a 128 KiB static device array (per-z-plane partial sums) that
 * every GPU loading this library holds until the process exits; domains with
 * nz > 4096 are rejected with LBM_ERR_INVALID_ARGUMENT.  All calls share that
 * array, so calls that overlap on the GPU (different streams, or different
 * host threads on one device) race and must be serialised by the caller.
 * The array has its own device address in each CUDA context.  The first call
 * in a context (for most callers: the first call on each device, in its
 * primary context) looks that address up with cudaGetSymbolAddress, with the
 * device current, and caches it by the context's unique id, so a
 * cudaDeviceReset or a caller's own driver context gets a fresh lookup; make
 * that first call before any stream capture. */
int lbm_reduce_noalloc(const void* populations, const int32_t* flags, const int32_t size[3], int32_t storage,
                       int32_t last_step_was_alpha, double* out_device, void* stream);

/* ---- checkpoint and output ------------------------------------------------ */

/* Writes the solver's whole state (parameters, flags, raw populations in the
 * storage type, step counter and A-A parity) to `path` (through a temporary
 * file renamed into place).  No counterpart in the reference, which cannot
 * resume a run; a resumed run continues bit-identically. */
int lbm_save_checkpoint(lbm_solver* solver, const char* path);
/* Restores a checkpoint into a solver of the same size and storage. */
int lbm_load_checkpoint(lbm_solver* solver, const char* path);
/* Creates a solver on `device` from a checkpoint. */
int lbm_create_from_checkpoint(const char* path, int32_t device, lbm_solver** out);

/* Writes the interior as a legacy VTK structured grid: cell-corner points
 * scaled to `length` (NULL: one unit per cell), then CELL_DATA flags,
 * densities and velocities (double for F64 storage, float otherwise).  With
 * binary = 0 the file is ASCII, as CLbmVisualizationVTK<T>::render
 * (src/libvis/CLbmVisualizationVTK.cpp:69-205) writes it; binary = 1 writes
 * the same records as legacy big-endian binary. */
int lbm_write_vtk(lbm_solver* solver, const char* path, const double length[3], int32_t binary);

/* ---- batches: many box cavities advanced together --------------------------
 * No counterpart in the reference (one solver per MPI rank there).  Every
 * domain is a lid-driven box cavity (obstacle halo, lid plane y = ny) with its
 * own size, 1/tau and lid velocity; all advance the same time steps.  The
 * populations of all domains share one device pool and one persistent kernel
 * launch per step walks a packed table of the domains; long runs replay a
 * CUDA graph.  A domain's results are bit-identical to the same domain run
 * alone by an lbm_solver of the same storage. */
typedef struct lbm_batch lbm_batch;   /* opaque */

typedef struct lbm_domain_spec {
    int32_t size[3];            /* interior cells                              */
    int32_t reserved;           /* zero                                        */
    double inv_tau;             /* 1/tau                                       */
    double lid_velocity;        /* lid x velocity                              */
} lbm_domain_spec;

typedef struct lbm_batch_info {
    int32_t count;              /* domains                                     */
    int32_t storage;
    int32_t fast_variant;       /* launch variant (register variants only)     */
    int32_t cells_per_thread;   /* alpha kernel                                */
    int32_t block_threads;
    int32_t beta_cells_per_thread;  /* beta kernel                             */
    int32_t beta_block_threads;
    int32_t reserved;
    int64_t interior_cells;     /* sum over domains: lattice updates per step  */
    int64_t step_counter;
    int64_t device_bytes;
} lbm_batch_info;

int lbm_batch_create(const lbm_domain_spec* domains, int32_t count, int32_t storage, int32_t device,
                     lbm_batch** out);
/* Frees the batch and its domain views. */
int lbm_batch_destroy(lbm_batch* batch);
int lbm_batch_get_info(const lbm_batch* batch, lbm_batch_info* info);
/* The solver handle of domain `index`: every single-domain getter, setter and
 * lbm_reduce works on it.  Owned by the batch (lbm_destroy refuses it).  Do
 * not step it alone: lbm_batch_run refuses a batch whose domains have left
 * its time level. */
int lbm_batch_domain(lbm_batch* batch, int32_t index, lbm_solver** view);
/* `steps` steps of every domain (alpha on even counters, beta on odd). */
int lbm_batch_run(lbm_batch* batch, int64_t steps, void* stream);
/* Selects a launch variant (a register variant whose vectors are at most 8
 * bytes wide, since batch rows are packed for them; LBM_ERR_UNSUPPORTED
 * otherwise) for the batch kernel. */
int lbm_batch_set_fast_variant(lbm_batch* batch, int32_t variant);
/* Times each register variant on the whole batch (`pairs` alpha/beta pairs,
 * CUDA events), keeps the fastest and restores the populations.  ms_per_pair
 * (optional) receives lbm_register_variant_count() times, -1 for a variant
 * whose vectors are wider than the batch's packed rows (8 bytes).
 * Synchronous. */
int lbm_batch_autotune(lbm_batch* batch, int32_t pairs, int32_t* best, float* ms_per_pair);

/* ---- servers: cavity-solve requests with continuous batching ---------------
 * No counterpart in the reference.  Requests wait in FIFO order and are
 * admitted while their populations fit a device arena sized to 95 % of the
 * memory budget (the rest covers the packed table and block maps); a request
 * holds nothing on the device but its populations, since the walls and the
 * lid come from the geometry.  Every round advances all resident requests
 * together (the batch kernel over a packed table of them), sized to last
 * about target_round_ms; finished requests write density and velocity to
 * mapped host memory, free their memory and post a completion.  Requests that arrive while others run join the next
 * round as memory frees up.  Each request's fields are bit-identical to the
 * same cavity solved alone.  One host thread drives a server. */
typedef struct lbm_server lbm_server;   /* opaque */

typedef struct lbm_server_config {
    int32_t storage;            /* lbm_storage of every request                */
    int32_t device;
    int32_t max_round_steps;    /* upper bound on steps per round (even)       */
    int32_t target_round_ms;    /* rounds sized to about this long; 0: fixed   */
    int32_t fast_variant;       /* 0: default; v + 1: register variant v with
                                   vectors of at most 8 bytes                  */
    int32_t reserved;
    int64_t budget_bytes;       /* device memory the server may hold           */
} lbm_server_config;

typedef struct lbm_request {
    int32_t size[3];            /* interior cells of the box cavity            */
    int32_t reserved;
    double inv_tau;
    double lid_velocity;
    int64_t steps;
} lbm_request;

typedef struct lbm_completion {
    int64_t id;
    int64_t steps;
    int64_t cells;              /* interior cells                              */
    int32_t status;             /* LBM_OK or the error that ended the request  */
    int32_t reserved;
    double submit_time;         /* seconds since the server was created        */
    double admit_time;
    double finish_time;         /* result on the host                          */
} lbm_completion;

typedef struct lbm_server_stats {
    int64_t queued, active, completed;
    int64_t bytes_in_use, peak_bytes, budget_bytes;
    int64_t lattice_updates;    /* interior-cell updates done so far           */
    int64_t rounds;
    double busy_seconds;        /* time spent in rounds                        */
    double elapsed_seconds;     /* since creation                              */
} lbm_server_stats;

int lbm_server_create(const lbm_server_config* config, lbm_server** out);
int lbm_server_destroy(lbm_server* server);
/* Queues a request; LBM_ERR_BUDGET if it could never fit the budget. */
int lbm_server_submit(lbm_server* server, const lbm_request* request, int64_t* id);
/* Admits, runs one round and retires; *ran = 0 when nothing was resident.
 * A request that finishes in a round is posted (lbm_server_poll) during the
 * next round, whose GPU work hides the copy of its result, or at the end of
 * the same round when no request is left running. */
int lbm_server_round(lbm_server* server, int32_t* ran);
/* Moves up to `capacity` new completions to `out`. */
int lbm_server_poll(lbm_server* server, lbm_completion* out, int32_t capacity, int32_t* count);
/* Copies a finished request's interior density (nx*ny*nz values) and velocity
 * (3 components) to the host buffers (either may be NULL) and releases it;
 * returns the request's status. */
int lbm_server_take_result(lbm_server* server, int64_t id, void* density, void* velocity);
int lbm_server_get_stats(const lbm_server* server, lbm_server_stats* stats);

/* ---- diagnostics ---------------------------------------------------------- */
const char* lbm_status_string(int status);
/* Detail message of the last failing call on this thread ("" if none). */
const char* lbm_last_error(void);
/* Number of kernel launches this library has queued since load (all
 * solvers); the benchmark reports it as its launch count. */
int64_t lbm_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
