/*
 * ethersph_gpu.h — C ABI of the GB300 (sm_103a) weakly-compressible SPH time step.
 *
 * This library is the drop-in for the hot loop of EtherSPHCPU.jl: the body of
 * `eachStep!` (neighbour search, continuity, equation of state, momentum with
 * pressure / viscosity / compulsive-wall / thermal terms, forward-Euler update,
 * Shepard density re-initialisation and the out-of-domain check).  A Julia
 * package adds `solve!` methods that marshal the particle vectors into plain
 * arrays and `ccall` these entry points; VTP output stays on the host.
 *
 * Reference interfaces replaced (paths inside the EtherSPHCPU.jl project):
 *   solve!(fluid, walls, kernel, model, td, vtp_io; check)
 *       src/Solve/FluidWallSolve.jl:85-140
 *       src/Solve/FluidThermostaticWallSolve.jl:127-173
 *       src/Solve/FluidCompulsiveThermostaticWallSolve.jl:154-233
 *       src/Solve/FluidVelocitySolve.jl:104-168
 *   eachStep!(...)   FluidWallSolve.jl:8-83, FluidThermostaticWallSolve.jl:8-125,
 *                    FluidCompulsiveThermostaticWallSolve.jl:8-152, FluidVelocitySolve.jl:8-102
 *
 * Conventions
 *   - Every call returns an int32 status (SPH_OK = 0).  No exceptions cross the
 *     ABI and no device trap is ever raised; sph_last_error() gives the text.
 *   - Vectors are passed as packed dim x n column-major arrays (Julia
 *     Matrix{Float64}(dim, n)): x[0], y[0], (z[0]), x[1], ...
 *   - The caller owns every host array; the library copies in and out and keeps
 *     no host pointer after a call returns.  The library owns all device memory
 *     behind the opaque handle and frees it in sph_destroy().
 *   - A handle is used by one host thread at a time.  Each handle owns one CUDA
 *     stream; different handles may be driven from different threads.
 */
#ifndef ETHERSPH_GPU_H
#define ETHERSPH_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------------------- */
enum {
    SPH_OK = 0,
    SPH_ERR_ARG = 1,           /* invalid argument or parameter block              */
    SPH_ERR_CUDA = 2,          /* a CUDA runtime call failed                        */
    SPH_ERR_OOM = 3,           /* device allocation failed or budget exceeded       */
    SPH_ERR_NAN = 4,           /* non-finite density / velocity / position found    */
    SPH_ERR_GRID_OVERFLOW = 5, /* cell grid or capacity too small for the scene     */
    SPH_ERR_TIMEOUT = 6,       /* a bounded wait gave up                            */
    SPH_ERR_STATE = 7,         /* call out of order (e.g. step before upload)       */
    SPH_ERR_NO_DEVICE = 8,     /* no CUDA device / extension not usable             */
    SPH_ERR_IO = 9             /* an output file or directory could not be written  */
};

/* ---- SPHKernel: src/SPHKernel/SmoothKernel/SmoothKernel.jl:15-20 ------------------ */
enum {
    SPH_KERNEL_CUBIC_SPLINE = 0, /* CubicSpline.jl:39-73  */
    SPH_KERNEL_GAUSSIAN = 1,     /* Gaussian.jl:31-56     */
    SPH_KERNEL_WENDLAND_C2 = 2,  /* WendlandC2.jl:38-63   */
    SPH_KERNEL_WENDLAND_C4 = 3   /* WendlandC4.jl:38-54   */
};

/* ---- which eachStep! method the step reproduces ---------------------------------- */
enum {
    SPH_SOLVE_FLUID_WALL = 0,                       /* FluidWallSolve.jl:8-83                       */
    SPH_SOLVE_FLUID_THERMOSTATIC_WALL = 1,          /* FluidThermostaticWallSolve.jl:8-125          */
    SPH_SOLVE_FLUID_COMPULSIVE_THERMOSTATIC_WALL = 2, /* FluidCompulsiveThermostaticWallSolve.jl:8-152 */
    SPH_SOLVE_FLUID_VELOCITY_WALL = 3,              /* FluidVelocitySolve.jl:8-102                  */
    SPH_SOLVE_FLUID_INLET_OUTLET_WALL = 4           /* FluidInletOutletWallSolve.jl:8-262           */
};

/* ---- wall particle types: src/Particle/FixedParticle/WallParticle.jl --------------- */
enum {
    SPH_WALL_COMPULSIVE = 0,      /* CompulsiveWallParticle      WallParticle.jl:8-19  */
    SPH_WALL_STATIC_VELOCITY = 1, /* StaticVelocityWallParticle  WallParticle.jl:21-34 */
    SPH_WALL_THERMOSTATIC = 2     /* ThermostaticWallParticle    WallParticle.jl:36-51 */
};

/* ---- arithmetic form of the pair sums -------------------------------------------- */
enum {
    SPH_PRECISION_FP64 = 0,             /* plain IEEE FP64, reference expression order */
    SPH_PRECISION_FP32_COMPENSATED = 1  /* FP32 pair math on cell-relative positions,
                                           Kahan-compensated sums, FP64 integration,
                                           FP64 Shepard sums                          */
};

/*
 * Parameter block.  Field names follow the Julia structs they are copied from:
 *   SmoothKernel            SmoothKernel.jl:37-48 (h_, sigma_, kernel_0_, influence_radius_)
 *   *WeaklyCompressibleLiquidModel   LiquidModel.jl:10-66
 *   DensityReinitializedFixedTimeIntervalForwardEuler  FixedTimeIntervalDiscretization.jl:10-16
 * The `check::Function` keyword of solve! (FluidWallSolve.jl:92) cannot run on the
 * device; it becomes an axis-aligned box: a fluid particle is deleted at a check
 * step when any coordinate is > check_hi or < check_lo (NaN compares false and
 * keeps the particle, as `!check(p)` would for the dam-break check).
 */
typedef struct SphParams {
    int32_t dim;        /* 2 or 3 */
    int32_t kernel;     /* SPH_KERNEL_* */
    int32_t solve;      /* SPH_SOLVE_* */
    int32_t precision;  /* SPH_PRECISION_* */

    /* SmoothKernel */
    double influence_radius; /* r_cut */
    double h;
    double sigma;
    double kernel_0;

    /* equation model */
    double rho_0;
    double c_0;
    double p_0;
    int32_t gamma;      /* integer exponent of the Tait equation */
    int32_t thermal;    /* 1: ThermalWeaklyCompressibleLiquidModel */
    double b;           /* c_0^2 rho_0 / gamma */
    double mu_0;
    double nu_0;
    double body_force[3];
    double t_0;
    double kappa_0;
    double cp;
    double beta;

    /* time discretisation */
    double dt;
    int64_t total_step;
    int64_t output_interval;
    int64_t check_interval;
    int64_t density_reinitialized_interval;

    /* check predicate and periodicity */
    int32_t check_enabled;
    int32_t periodic_x;     /* 1: periodic in x with period domain_hi[0]-domain_lo[0] (new; not in the reference) */
    double check_lo[3];
    double check_hi[3];

    /* extent of the cell grid; particles outside are clamped into the edge cells */
    double domain_lo[3];
    double domain_hi[3];

    int32_t nan_check;      /* 1: sph_step returns SPH_ERR_NAN when a fluid state turns non-finite */
    int32_t cell_subdivision; /* cells per r_cut along each axis (1, 2 or 3; 0 = 3): finer cells
                                 visit fewer candidates; the neighbour order, and so the
                                 summation order, depends on it */
} SphParams;

typedef struct SphStats {
    int64_t n_fluid;          /* live fluid particles */
    int64_t n_wall;
    int64_t steps_done;       /* steps run on this handle */
    double total_mass;        /* FP64 sum of fluid masses */
    double kinetic_energy;    /* FP64 sum of m |v|^2 / 2 */
    double max_speed;
    int32_t status_flags;     /* bit 0: non-finite state seen, bit 1: particle outside grid (clamped) */
    int32_t reserved0;
} SphStats;

typedef struct SphHandle SphHandle;

/* ABI version (SPH_ABI_VERSION). */
int32_t sph_version(void);

/* Create a single-scene handle: allocate device state for up to fluid_capacity fluid
 * and wall_capacity wall particles.  Replaces the set-up part of solve!
 * (FluidWallSolve.jl:94-104: InPlaceNeighborList construction). */
int32_t sph_create(const SphParams* params, int64_t fluid_capacity, int64_t wall_capacity,
                   SphHandle** out);

/* Copy fluid particles in (replaces the state).  x, v: dim x n.  p and c may be NULL
 * (then computed from rho with updatePressure!, UpdatePressure.jl:8-16); t, kappa, cp
 * are read only for thermal models (ThermalLiquidParticle, LiquidParticle.jl:43-64).
 * Particle identity is the index 0..n-1 of this call. */
int32_t sph_upload_fluid(SphHandle* h, int64_t n, const double* x, const double* v,
                         const double* rho, const double* p, const double* c,
                         const double* mass, const double* gap, const double* t,
                         const double* kappa, const double* cp);

/* Append one group of static wall particles (WallParticle.jl).  normal: dim x n.
 * t, kappa: SPH_WALL_THERMOSTATIC only; v (dim x n): SPH_WALL_STATIC_VELOCITY only. */
int32_t sph_upload_walls(SphHandle* h, int32_t kind, int64_t n, const double* x,
                         const double* normal, const double* gap, const double* t,
                         const double* kappa, const double* v);

/* Run steps first_step .. first_step+nsteps-1 of eachStep!.  Step s re-initialises
 * density when s % density_reinitialized_interval == 0 and applies the check when
 * check_enabled and s % check_interval == 0 (FixedTimeIntervalDiscretization.jl:18-23,
 * TimeDiscretization.jl:19-25).  Synchronous: returns after the last step finished. */
int32_t sph_step(SphHandle* h, int64_t first_step, int64_t nsteps);

/* Enqueue the same steps on the handle's stream and return without waiting (for
 * callers that overlap host work or time the stream with CUDA events).  Status bits
 * accumulate until sph_synchronize(), which waits and reports them like sph_step. */
int32_t sph_step_async(SphHandle* h, int64_t first_step, int64_t nsteps);
int32_t sph_synchronize(SphHandle* h);

/* Copy the live fluid particles out in their original order (deleted particles
 * removed, as deleteat! leaves the Julia vector).  Any pointer may be NULL.
 * capacity: room in the caller's arrays, in particles. */
int32_t sph_download_fluid(SphHandle* h, int64_t capacity, int64_t* n_out, double* x,
                           double* v, double* rho, double* p, double* c, double* mass,
                           double* gap, double* t, double* kappa, double* cp);

/* Indices (0-based, into the arrays of the last sph_upload_fluid) of the live fluid
 * particles, ascending: the positions deleteat! would have kept.  Same order as
 * sph_download_fluid. */
int32_t sph_download_ids(SphHandle* h, int64_t capacity, int64_t* n_out, int64_t* ids);

/* FP64 reductions over the live fluid (mass, kinetic energy, max speed). */
int32_t sph_stats(SphHandle* h, SphStats* out);

/* Unique fluid-fluid pairs (i<j, CellListMap half-list convention) and fluid-wall
 * pairs within r_cut at the current positions. */
int32_t sph_count_pairs(SphHandle* h, int64_t* fluid_pairs, int64_t* wall_pairs);

/* Diagnostic: the cell of every live fluid particle at the current positions, as the
 * step's sort assigns it — the scene-local index cx + nx (cy + ny cz) in the handle's
 * grid (cells of edge r_cut (1 + 1e-9) / cell_subdivision from domain_lo, positions
 * outside the grid clamped into its edge cells, a periodic x axis cut into equal cells).
 * Rows in the order of sph_download_fluid (ascending particle id).  grid (may be NULL)
 * receives the cell counts (nx, ny, nz).  With keys == NULL only n_out and grid are
 * written.  Single-scene handles.  Replaces nothing in the
 * reference's API: it exposes the cell assignment that CellListMap.update! makes inside
 * each step (FluidWallSolve.jl:21-27) so it can be pinned particle by particle. */
int32_t sph_download_cell_keys(SphHandle* h, int64_t capacity, int64_t* n_out, int64_t* keys, int32_t* grid);

/* Diagnostic: the fluid neighbours of every live fluid particle that the handle's gathers
 * accept — every j != i with |x_i - x_j|^2 <= r_cut^2, decided in FP64 (products and sums
 * rounded one by one, minimum image along a periodic x) for the FP64 form and in FP32 on
 * cell-relative positions for the FP32-compensated form — as particle ids (those of
 * sph_download_ids), ascending within a row; rows in the order of sph_download_fluid.
 * CSR form: offsets[0..n] (capacity: room for n + 1 offsets), ids[offsets[n]].  With
 * ids == NULL only n_out, offsets and total_out are written; SPH_ERR_ARG when the total
 * exceeds ids_capacity (total_out is still set).  Single-scene handles.  Replaces nothing
 * in the reference's API: the per-particle form of the pair list that
 * CellListMap.neighborlist! + findNeighbours! build each step (FluidWallSolve.jl:28-35,
 * Neighbour.jl:88-128), for pinning the neighbour search particle by particle. */
int32_t sph_download_neighbours(SphHandle* h, int64_t capacity, int64_t ids_capacity, int64_t* n_out,
                                int64_t* total_out, int64_t* offsets, int64_t* ids);

/* The cudaStream_t the handle launches on (for CUDA-event timing by the caller). */
int32_t sph_get_stream(SphHandle* h, void** stream);

/* Diagnostic: time each stage of one step with CUDA events on the handle's stream,
 * `reps` times, without advancing the state (every stage reads one buffer and writes
 * another).  ms_out receives SPH_NUM_STAGES averages in milliseconds. */
#define SPH_NUM_STAGES 6
enum {
    SPH_STAGE_CELL_COUNT = 0, /* cell hash + per-cell count                */
    SPH_STAGE_SCAN = 1,       /* exclusive scan -> cellStart                */
    SPH_STAGE_SORT = 2,       /* stable (cell, id) placement + reorder      */
    SPH_STAGE_CONTINUITY = 3, /* continuity gather + density + EOS          */
    SPH_STAGE_MOMENTUM = 4,   /* momentum gather + integration              */
    SPH_STAGE_REINIT = 5      /* the momentum gather of a density re-initialisation step:
                                 momentum + integration with the Shepard sums fused in */
};
int32_t sph_time_stages(SphHandle* h, int32_t reps, double* ms_out);

/* ---- batched scenes and serving ---------------------------------------------------
 * A batch handle steps many independent scenes (same dim, kernel, solve variant, form
 * and thermal flag; any geometry, resolution and physical constants) in the same kernel
 * launches: particles of all scenes share the sorted arrays, every scene owns a range
 * of cells and a region of the wall arrays, and every scene advances its own step
 * counter (Shepard and check steps follow each scene's own step numbers).  Capacities
 * are fixed at creation (that is the device memory budget); scenes can be added and
 * retired between steps, so requests are served while others run.  No reference
 * counterpart: EtherSPHCPU.jl runs one solve! per process. */

/* prototype: dim, kernel, solve, precision and thermal of every scene of the batch. */
int32_t sph_batch_create(const SphParams* prototype, int64_t particle_capacity, int64_t cell_capacity,
                         int64_t wall_capacity, int32_t scene_capacity, SphHandle** out);

/* Add a scene that will run steps first_step .. first_step+nsteps-1 and then stay
 * frozen (state kept) until retired.  Fluid arrays as in sph_upload_fluid; walls as one
 * merged set with a kind per particle (wall_t/wall_kappa read for thermostatic walls,
 * wall_v for static-velocity walls; may be NULL otherwise).  SPH_ERR_OOM when a
 * capacity (particles, a contiguous run of cells or walls, scene slots) is exhausted. */
int32_t sph_batch_add_scene(SphHandle* h, const SphParams* params, int64_t first_step, int64_t nsteps, int64_t n,
                            const double* x, const double* v, const double* rho, const double* p, const double* c,
                            const double* mass, const double* gap, const double* t, const double* kappa,
                            const double* cp, int64_t n_wall, const int32_t* wall_kind, const double* wall_x,
                            const double* wall_normal, const double* wall_gap, const double* wall_t,
                            const double* wall_kappa, const double* wall_v, int32_t* scene_id);

/* Run nsteps steps of every scene (frozen scenes are carried unchanged); asynchronous,
 * sph_synchronize() waits and reports non-finite states. */
int32_t sph_batch_step(SphHandle* h, int64_t nsteps);

/* info[4] = (live particles, steps done, finished (0/1), next step number). */
int32_t sph_batch_scene_info(SphHandle* h, int32_t scene_id, int64_t* info);

/* Live particles of one scene in their original order (as sph_download_fluid). */
int32_t sph_batch_download_scene(SphHandle* h, int32_t scene_id, int64_t capacity, int64_t* n_out, double* x,
                                 double* v, double* rho, double* p, double* c, double* mass, double* gap, double* t,
                                 double* kappa, double* cp);

/* Drop a scene's particles and free its slot, cells and walls. */
int32_t sph_batch_retire(SphHandle* h, int32_t scene_id);

/* What a scene occupies in a batch: out[3] = (fluid particles, cells including the
 * scene's sentinel cell, wall particles), from the grid the library would build for
 * `params` (no device needed).  Admission control compares it with sph_batch_free. */
int32_t sph_scene_footprint(const SphParams* params, int64_t n_fluid, int64_t n_wall, int64_t* out);

/* out[4] = (free particle slots, largest free run of cells, largest free run of walls,
 * free scene slots): what admission control compares a scene's footprint with. */
int32_t sph_batch_free(SphHandle* h, int64_t* out);

/* Pair counting that allocates no device memory.  No counterpart in the reference:
 * it serves callers that cannot let a library call cudaMalloc or cudaFree (device
 * memory owned by another framework's stream-ordered pool, code that must not cause
 * the device-wide synchronisation cudaMalloc/cudaFree can trigger).
 * Counts the same pairs as sph_count_pairs for particles the caller holds in DEVICE
 * memory: x (dim x n packed), wall_x (dim x n_wall packed); writes
 * counts[0] = unique fluid pairs, counts[1] = fluid-wall pairs into the caller's device
 * array counts[2].  Work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 * stream) and the call returns without waiting.
 * The cell list lives in one static device array of the library (about 10 MB, resident
 * on every GPU that loaded the library until the process exits): at most 262,144 fluid
 * and 262,144 wall particles and 262,144 grid cells; larger inputs return SPH_ERR_ARG.
 * The first call in a CUDA context looks up that array's device address and caches it
 * with the context's id (a call from another context, e.g. after cudaDeviceReset, looks
 * it up again): make the first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race, so serialise them on one stream.  Errors:
 * sph_last_error(NULL). */
int32_t sph_count_pairs_noalloc(const SphParams* params, int64_t n, const double* x, int64_t n_wall,
                                const double* wall_x, int64_t* counts, void* stream);

/* Autotuner of the FP32-compensated form: times the continuity and momentum gathers on
 * the current state for every lanes-per-particle count {-1, 1, 2, 4, 8} and block size
 * {64, 128, 256}, and the neighbour-list pair (continuity recording the list with lanes
 * {-1, 1, 2}, momentum reading it with lanes {-1, 1, 2, 4}); keeps the faster of the
 * cell-walk and list pairs and rebuilds the step graphs.  out[4] (may be NULL) receives
 * the launch shape (see sph_set_launch_shape).  The fluid state is left unchanged.  No-op
 * for the FP64 form, which keeps one thread per particle so that its summation order is
 * fixed. */
int32_t sph_autotune(SphHandle* h, int32_t reps, int32_t* out);

/* Momentum lanes code of the neighbour list: SPH_LANES_LIST + t, t in {1, 2, 4, -1}.
 * The continuity gather (one or two lanes per particle) records, in its walk order, every
 * neighbour within r_cut of each particle (two lanes: each lane its share of the
 * candidates, lane 0 from the list's first entry up, lane 1 from its last entry down),
 * and the momentum gather of the same step reads
 * that list with t lanes per particle instead of walking the cells a second time (same
 * pairs: positions do not change between the two gathers).  The list holds about
 * 1.25 x the lattice neighbour count of the finest uploaded spacing per particle
 * (4 bytes each, grown with the live particle count); a particle with more neighbours
 * walks the cells. */
#define SPH_LANES_LIST 16

/* Set the FP32 launch shape by hand (a new handle starts at (1, 1, 1, 128)):
 * shape[4] = (continuity lanes, momentum lanes, unused, block size).  shape[2] is kept for
 * the layout and must be a lanes code: the Shepard sums of a re-initialisation step run
 * inside the momentum gather, at its lanes.  Lanes in {1, 2, 4, 8} or -1 (one lane whose candidate loop
 * is software-pipelined: loads of the next neighbour overlap the current one's
 * arithmetic; momentum lanes -1 take blocks of at most 256), block in {32, 64, ..., 1024}
 * and a multiple of 32.  Momentum lanes may instead be a neighbour-list code
 * (SPH_LANES_LIST + 1, 2, 4 or -1; continuity lanes 1, 2 or -1 then).  Results of the FP32
 * form depend on the lanes codes (the order of the compensated partial sums, and for -1
 * against 1 the compiler's contraction of a*b+c into fused multiply-adds), never on the
 * block size. */
int32_t sph_set_launch_shape(SphHandle* h, const int32_t* shape);

/* Stencil pruning of the FP32-compensated walks (the FP64 form's walks always prune, with
 * the same bitwise-neutral rule; default: on for 3D scenes, off for 2D,
 * where it does not pay on GB300): for each neighbour row
 * the walk visits only the cells whose extent comes within r_cut of the particle (with a
 * margin of 1e-5 on r_cut^2), instead of all 2m+1 cells of the (2m+1)^dim stencil.  Only
 * candidates the distance test would reject are skipped, so with one lane per particle
 * the results are bitwise the same either way.  No counterpart in the reference. */
int32_t sph_set_stencil_pruning(SphHandle* h, int32_t on);

/* ---- inlet / outlet buffers ------------------------------------------------------
 * FluidInletOutletWallSolve (src/Solve/FluidInletOutletWallSolve.jl:8-262), for a
 * single-scene handle created with solve = SPH_SOLVE_FLUID_INLET_OUTLET_WALL (fluid,
 * compulsive walls without wall pressure, no thermal model).  Inlet and outlet particles
 * are fluid particles that enter the fluid's continuity and momentum sums as neighbours
 * but are not updated by them: each step they move by x += v dt and keep rho, p, c.
 * After the step (on the device, in the same kernels stream):
 *   - an inlet particle with n_in.x > d_in is copied into the fluid (a new fluid particle
 *     with the inlet particle's state; ids continue after the uploaded fluid, ordered by
 *     step, then by inlet index, as push! orders them) and then moved by in_shift
 *     (inlet_into_calculation_domain_check / _modify);
 *   - a fluid particle with n_out.x > d_out moves to the outlet (it leaves the fluid:
 *     outlet_out_calculation_domain_check);
 *   - an outlet particle with n_drop.x > d_drop is removed (outlet_out_check).
 * The examples' check functions compare one coordinate with a bound
 * (PoiseuilleFlow2D.jl:146-151): n is then a unit axis.  user_defined_function, a host
 * callback, becomes sph_set_buffer_velocity between step calls. */
typedef struct SphBufferRules {
    double inlet_normal[3];
    double inlet_offset;
    double inlet_shift[3];
    double outlet_normal[3];
    double outlet_offset;
    double drop_normal[3];
    double drop_offset;
} SphBufferRules;

/* Set the rules and the buffer particles (replaces earlier buffers): n_inlet inlet and
 * n_outlet outlet particles (x, v: dim x n; rho, p, c, mass, gap: n), room for
 * `capacity` buffer particles in all (the outlet grows by the fluid it receives). */
int32_t sph_upload_buffers(SphHandle* h, const SphBufferRules* rules, int64_t capacity, int64_t n_inlet,
                           const double* x, const double* v, const double* rho, const double* p, const double* c,
                           const double* mass, const double* gap, int64_t n_outlet, const double* ox,
                           const double* ov, const double* orho, const double* op, const double* oc,
                           const double* omass, const double* ogap);

/* Overwrite the velocities of the inlet (which = 0) or outlet (which = 1) particles, in
 * their order (v: dim x n, n = their current count): the device counterpart of a
 * user_defined_function that prescribes the buffer velocity between steps. */
int32_t sph_set_buffer_velocity(SphHandle* h, int32_t which, int64_t n, const double* v);

/* The inlet (which = 0) or outlet (which = 1) particles in the reference's vector order
 * (inlet: upload order; outlet: uploaded ones, then arrivals by step and fluid order). */
int32_t sph_download_buffers(SphHandle* h, int32_t which, int64_t capacity, int64_t* n_out, double* x, double* v,
                             double* rho, double* p, double* c, double* mass, double* gap);

/* ---- SPH interpolation at points (probes) --------------------------------------
 * kernelValueInterpolation (src/DataIO/VTPToDataFrame.jl:93-142) on the device state:
 * for each point, f = sum W m_j/rho_j f_j / sum W m_j/rho_j over the fluid particles j
 * within r_cut (none_value where no particle is in range).  The reference evaluates it
 * on VTP files after a run; here it reads the live state of a single-scene handle.
 * points: dim x n_points (host); fields: n_fields codes (1..8) from the list below;
 * out: n_fields x n_points (host), field-major.  A periodic x axis takes the nearest
 * image.  SPH_ERR_ARG for an unknown code, VELOCITY_Z in 2D or TEMPERATURE without a
 * thermal model. */
enum {
    SPH_PROBE_DENSITY = 0,     /* rho_ */
    SPH_PROBE_PRESSURE = 1,    /* p_   */
    SPH_PROBE_SOUND_SPEED = 2, /* c_   */
    SPH_PROBE_VELOCITY_X = 3,  /* v_vec_[1] */
    SPH_PROBE_VELOCITY_Y = 4,  /* v_vec_[2] */
    SPH_PROBE_VELOCITY_Z = 5,  /* v_vec_[3] (3D) */
    SPH_PROBE_TEMPERATURE = 6, /* t_ (thermal models) */
    SPH_PROBE_MASS = 7         /* mass_ */
};
int32_t sph_probe(SphHandle* h, int64_t n_points, const double* points, int32_t n_fields, const int32_t* fields,
                  double none_value, double* out);

/* ---- VTP output without stalling the steps --------------------------------------
 * Counterpart of writeVTP(step, t, vtp_io, [fluid, walls...]) (src/DataIO/VTPIO.jl:41-98)
 * as solve! calls it at step 0 and at every output step (FluidWallSolve.jl:95,133-136).
 * sph_output_write stages the live fluid with device-to-device copies ordered after the
 * steps already enqueued, then copies it to pinned host memory on a second stream and
 * writes the file on a host thread while later steps run.  Single-scene handles only.
 *
 * sph_output_open: VTPIO's fields (VTPIO.jl:8-15): files are
 * dir_path/file_name<file_step zero-padded to step_digit><file_suffix>; dir_path is
 * created if missing (assureDirPathExist, DataIO.jl:35-40).  field_symbols name particle
 * fields ("rho_", "p_", "c_", "mass_", "gap_", "t_", "kappa_", "cp_"; a leading ':' is
 * ignored); a symbol a group's particle type lacks gives NaN for that group, as
 * getParticleFields! (VTPIO.jl:21-38); vector and accumulator fields (x_vec_, drho_, ...)
 * are SPH_ERR_ARG.  wall_time: fixed WallTime text for every file, or NULL for the
 * clock.  Groups: the fluid (Type 1), then, for the inlet/outlet solve, the inlet and
 * the outlet particles (FluidInletOutletWallSolve.jl:282), then each sph_upload_walls
 * call in call order.  Files use the VTK XML appended raw layout with UInt64 headers. */
int32_t sph_output_open(SphHandle* h, const char* dir_path, const char* file_name, const char* file_suffix,
                        int32_t step_digit, int32_t n_fields, const char* const* field_symbols,
                        const char* const* field_names, const char* wall_time);

/* Queue the file of file_step (Step field data) at time `time` (Time field data) for
 * the state after every step enqueued so far.  Returns once the staging copies are
 * enqueued; waits only when two earlier files are still being written. */
int32_t sph_output_write(SphHandle* h, int64_t file_step, double time);

/* Wait until every queued file is on disk; returns the first write error (SPH_ERR_IO). */
int32_t sph_output_flush(SphHandle* h);

/* Text of the last error on this handle (or of the last failed sph_create when h is NULL). */
const char* sph_last_error(const SphHandle* h);

/* Free all device memory of the handle. */
int32_t sph_destroy(SphHandle* h);

#ifdef __cplusplus
}
#endif

#endif /* ETHERSPH_GPU_H */
