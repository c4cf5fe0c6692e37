/*
 * cylag_gpu.h -- C ABI of libcylag_gpu.so, the GB300 (sm_103a) particle step.
 *
 * Plain C types only: sizes, host pointers for one-time uploads, device
 * pointers for the particle state (the caller allocates and owns them, e.g.
 * as torch tensors; the library never frees caller memory).  Every call
 * returns an int status: CG_OK (0) or a negative CG_E* code, with the message
 * available from cg_last_error().  No C++ exception crosses this boundary.
 * One host thread per context; work is issued on the context's own CUDA
 * stream (cg_ctx_stream) and is asynchronous unless stated otherwise.
 *
 * Each entry point names the reference interface it replaces (CyLag, paths
 * relative to the CyLag source tree).
 */
#ifndef CYLAG_GPU_H
#define CYLAG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_OK 0
#define CG_EINVAL (-1)        /* bad argument (reference: ValueError) */
#define CG_ECUDA (-2)         /* CUDA runtime error */
#define CG_ENOMEM_BUDGET (-3) /* admission refused: HBM budget exceeded */
#define CG_EDEVICE (-4)       /* device-side error flag (see cg_run_errors) */
#define CG_ESTATE (-5)        /* call out of order (mesh/fields not uploaded) */

/* device error flags, OR-ed into the run's error word */
#define CG_ERR_INTERP_OUTSIDE 1   /* interpolation below bed / above surface
                                     (eulerian_field_set.pyx:1270-1276) */
#define CG_ERR_DEGENERATE_LAYER 2 /* |dz| < EPSILON between layers (1356-1363) */
#define CG_ERR_RNG_LIMIT 4        /* a rejection loop hit its iteration cap */
#define CG_ERR_UNSUPPORTED 8      /* option combination not built */
#define CG_ERR_NONFINITE 16       /* LSM2/LSM3 coefficients or stationary
                                     fluctuations the reference rejects with
                                     ValueError (update_state_lsm2.pyx:1283,
                                     update_state_lsm3.pyx:98-104,
                                     init_lsm2_fluctuations.pyx:68-77) */
#define CG_ERR_BOUNDS 32          /* bounds-checked library build only: a gather
                                     index read from the mesh tables or the
                                     particle state was out of range (the
                                     access was redirected, not made) */

#define CG_PRECISION_FP64 0       /* plain form: FP64 end to end */
#define CG_PRECISION_MIXED 1      /* FP32 fields/updates, FP64 position + localization */

typedef struct cg_ctx cg_ctx;
typedef struct cg_run cg_run;

/* Mesh arrays exactly as cylag.TriangularMesh holds them
 * (cylag/geom/triangular_mesh.pyx:28-629), plus the point-location grid
 * that replaces its KD-tree (triangular_mesh.pyx:602-629). Host pointers. */
typedef struct {
    int32_t nv, nt, ne, nopen;
    const double *x, *y;             /* [nv] */
    const int32_t *triangles;        /* [nt][3] */
    const double *gradx, *grady, *det; /* [nt][3] */
    const int32_t *edges;            /* [ne][2] */
    const int32_t *triedge_map;      /* [nt][3] */
    const int32_t *edgetri_map;      /* [ne][2] */
    const int32_t *edges_labels;     /* [ne] */
    double grid_x0, grid_y0, grid_inv_cell;
    int32_t grid_nx, grid_ny;
    const int32_t *grid_start;       /* [grid_nx*grid_ny + 1] */
    const int32_t *grid_tris;        /* [grid_start[last]] */
} cg_mesh_desc;

/* Node fields as cylag.EulerianFieldSet holds them
 * (cylag/core/eulerian_field_set.pyx:125-256): each [ntimes][npoints*nlayers],
 * layer l at [l*npoints, (l+1)*npoints).  NULL for an absent field. Host. */
typedef struct {
    int32_t dim, nlayers, npoints, ntimes;
    const double *times;             /* [ntimes] */
    const double *elevation;         /* field id 0 */
    const double *velocity_x, *velocity_y, *velocity_z; /* ids 1-3 */
    const double *turbulent_energy;  /* 'TURBULENT ENERG.' */
    const double *dissipation;       /* 'DISSIPATION' */
    const double *bottom;            /* 'BOTTOM' (required for 3D particles on 2D fields) */
    /* friction law of the pseudo-3D log-law profile (EulerianFieldSet's
     * friction_model 0 Chezy, 1 Strickler, 2 Manning, 3 Nikuradse, and
     * friction_coefficient; eulerian_field_set.pyx:125-138, 1957-1993) */
    int32_t friction_model;
    double friction_coefficient;
} cg_fields_desc;

/* Parameters (cylag/cylag_dico.py:9-51, cylag/core/parameters.pyx:116-195)
 * and the particle-set scalars (cylag/core/lagrangian_particle_set.pyx:158-261). */
typedef struct {
    int32_t model, time_scheme, rng_method, diffusion_model;
    int32_t diffusion_lsm2_option, lsm3_edge_opt;
    int32_t boundary_conditions, boundary_conditions_type, max_wall_rebounds;
    int32_t bnd_statistics, particle_velocity_init, frozen_eulerian_fields;
    double initial_time, final_time, time_step;
    double horizontal_diffusivity, vertical_diffusivity, schmidt_number;
    double tl_horizontal, tl_vertical;
    double rebound_damping_coef, wall_roughness_angle, stranding_probability;
    double water_density;
    /* particle set */
    int32_t dim;
    double particle_density;
    int32_t drag_coefficient_model; double drag_coefficient;
    int32_t added_mass_force; double added_mass_coef;
    int32_t buoyancy_velocity_model; double buoyancy_velocity;
    /* GPU-only */
    int32_t precision;               /* CG_PRECISION_* */
    uint64_t seed;                   /* PCG32 streams: pcg32_seed(seed, tag) */
    int32_t sort_period;             /* re-sort particles by element every this many
                                        steps (0: never); 2D runs; invisible to callers */
} cg_params;

/* Particle state: device pointers in the reference layout
 * (cylag/core/lagrangian_particle_set.pxd): rows of dim doubles.
 * tri == -1 marks an inactive particle, tri == -2 one awaiting
 * initialization (lagrangian_particle_set.pyx:620-710). */
typedef struct {
    int32_t n;
    double *position, *velocity, *fluid_velocity_seen;   /* [n][dim] */
    double *last_position, *last_velocity;               /* [n][dim] */
    int32_t *tri, *last_tri, *lowerlayer, *tag;          /* [n] */
    double *diameter;                                    /* [n] */
    uint64_t *rng_state;                                 /* [n] PCG32 state */
    double *depth;   /* [n] depth below the free surface, set at initialization and
                        after every call for active particles, zeroed at deletion
                        (LagrangianParticleSet.compute_depth, solver.pyx:325-332,
                        526-538; 3D particles), or NULL */
} cg_state_desc;

/* ---- context ---------------------------------------------------------- */
/* Creates a context on `device` with its own stream; hbm_budget_bytes bounds
 * what cg_run_create may admit (0 = no bound).  No reference counterpart:
 * the reference holds everything in Python objects. */
int cg_ctx_create(int32_t device, uint64_t hbm_budget_bytes, cg_ctx **out);
int cg_ctx_destroy(cg_ctx *ctx);
/* Copies the last error message (NUL-terminated, truncated to len). */
int cg_last_error(const cg_ctx *ctx, char *buf, uint64_t len);
/* The stream the context issues work on (a cudaStream_t as an integer). */
uint64_t cg_ctx_stream(const cg_ctx *ctx);
/* Issue all further work on the caller's stream (e.g. a torch stream); the
 * caller keeps it alive until the context is destroyed or the stream is
 * reset with 0 (back to the context's own stream).  Synchronizes the
 * previous stream first.  No reference counterpart. */
int cg_ctx_set_stream(cg_ctx *ctx, uint64_t stream);
int cg_ctx_sync(cg_ctx *ctx);

/* Replaces TriangularMesh.__init__ (triangular_mesh.pyx:75-179): packs and
 * uploads the mesh once.  Synchronous. */
int cg_mesh_upload(cg_ctx *ctx, const cg_mesh_desc *mesh);

/* Replaces EulerianFieldSet.__init__ + _init_tmp
 * (eulerian_field_set.pyx:125-256, 743-776): uploads every time record.
 * Synchronous. */
int cg_fields_upload(cg_ctx *ctx, const cg_fields_desc *fields);

/* ---- runs ------------------------------------------------------------- */
/* Replaces Solver.__init__ up to the particle loop (solver.pyx:74-197):
 * checks, time state, model coefficients.  `state` points to caller-owned
 * device buffers.  Fails with CG_ENOMEM_BUDGET when the run's bytes would
 * exceed the context budget. */
int cg_run_create(cg_ctx *ctx, const cg_params *params,
                  const cg_state_desc *state, cg_run **out);
int cg_run_destroy(cg_run *run);

/* Seeds the per-particle PCG32 streams: rng_state[i] = pcg32_seed(seed, tag[i])
 * (random_utils.pyx:30-37). */
int cg_run_seed(cg_run *run);

/* Replaces Solver.initialize_particle_state for every particle with
 * tri == -2 (solver.pyx:238-379): point location, vertical clamp, velocity
 * initialization.  Asynchronous. */
int cg_run_init(cg_run *run);

/* Replaces `nsteps` calls of Solver.forward (solver.pyx:413-585): time
 * interpolation of the fields at each step-start time, the fused particle
 * step, time += dt.  bnd_stats_host (optional) receives [nsteps][nopen]
 * open-boundary exit counts (solver.pyx:567-572).  Synchronous: returns
 * after the last step, CG_EDEVICE if the device raised an error flag.
 *
 * A run with sort_period > 0 steps on working copies of the particle state
 * in element order: gathered from the caller's arrays at the first step
 * (and at the first step after a cg_run_writeback), re-sorted every
 * sort_period steps counted across calls, and kept in the run between
 * calls.  While they are, the caller's position, tri, tag and rng_state
 * (and, as the model needs them every step, velocity, fluid_velocity_seen,
 * lowerlayer and diameter) are stale: call cg_run_writeback before reading
 * or changing them.  The other arrays are current after every call. */
int cg_run_step(cg_run *run, int32_t nsteps, int32_t *bnd_stats_host);

/* Writes a sorted run's working copies back to the caller's arrays and
 * releases them: after this (stream-ordered; cg_ctx_sync to wait) the
 * caller's arrays hold the whole state, may be read or changed, and the
 * next step gathers them again.  A no-op when nothing is held.  The
 * reference keeps its particle arrays in place (no counterpart); the
 * Python layer calls it before every access to the particle arrays.
 * cg_run_seed, cg_run_init, cg_run_added, cg_run_step_host and
 * cg_run_step_noalloc write back first themselves; cg_run_resize and
 * cg_run_destroy do not (resize refuses with CG_ESTATE while copies are
 * held; destroy drops them). */
int cg_run_writeback(cg_run *run);

/* Allocation-free variant of cg_run_step, for callers that cannot call
 * cudaMalloc while they step: code running under a memory pool or arena that
 * owns all device memory (frameworks that forbid allocations outside their
 * allocator), real-time loops that must not block in the driver's allocator,
 * and hosts that cap device memory once at start-up.  No counterpart in the
 * reference.
 *
 * Same step as cg_run_step (same kernels, same results for the same run
 * state) on the caller's arrays in their own order (a sorted run's working
 * copies are written back first), except: no open-boundary statistics, no
 * element re-sort, kernel time reported as 0 (cg_run_last_kernel_ms gives
 * this call's launch count).  Runs with control sections or stranding
 * output on are refused with CG_EINVAL: their per-call buffers belong to
 * cg_run_step.  Its scratch (the queue of particles leaving their triangle)
 * is a file-scope device array of CG_NOALLOC_MAX_PARTICLES entries (8 MiB)
 * that every GPU loading the library holds until exit; runs with more
 * particles are rejected with CG_EINVAL.  It calls no cudaMalloc, cudaFree
 * or other allocating routine.  The first call on a device (and the first
 * after that device's context was reset) looks up the array's device
 * address (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  All calls share the one array: calls whose work overlaps on the
 * GPU (two runs stepped concurrently on different streams) race on it.
 * Synchronous, like cg_run_step. */
#define CG_NOALLOC_MAX_PARTICLES 262144
int cg_run_step_noalloc(cg_run *run, int32_t nsteps);

/* The device samplers the step draws from, run in stream order from
 * pcg32_seed(seed, stream) (random_utils.pyx:30-37): kind 0 random_uniform
 * (55-67), 1 the ziggurat normal (154-194), 2 the polar normal (72-108),
 * 3 generate_random_pair(method) (202-233; 2n values), 4
 * generate_random_single(method) (235-263).  FP64 (plain-form) samplers;
 * n values copied to out_host.  Synchronous. */
int cg_rng_draws(cg_ctx *ctx, uint64_t seed, uint64_t stream, int32_t kind, int32_t method,
                 int64_t n, double *out_host);

/* Current simulated time and iteration (cylag/core/simutime.pyx:77-84). */
int cg_run_time(const cg_run *run, double *time, int64_t *iteration);

/* Device error word accumulated since the last call (then cleared). */
int cg_run_errors(cg_run *run, uint32_t *flags);

/* Number of active particles and deleted-this-call counts are derived by the
 * caller from tri (tri == -1 inactive). */

/* ---- particle state in host memory ---------------------------------------- */
/* Host arrays of the whole pool (pinned: cudaHostAlloc / torch pin_memory);
 * NULL arrays are not transferred. */
typedef struct {
    double *position;             /* [n, dim] */
    double *velocity;             /* [n, dim] */
    double *fluid_velocity_seen;  /* [n, dim] */
    int32_t *tri;
    int32_t *lowerlayer;
    int32_t *tag;
    uint64_t *rng_state;
} cg_host_arrays;

/* nsteps x Solver.forward with the particle state kept in host memory, the
 * drop-in for a caller whose arrays are the reference's host arrays: every
 * step copies the `in` arrays into the run's device arrays, steps, and copies
 * the device arrays back into the `out` arrays, chunk by chunk (`chunk`
 * particles; 0 = four equal chunks on 256-particle boundaries from 2^20
 * particles up), so that the copies of one chunk overlap the step of another
 * (a host->device stream, the run's stream, a device->host stream).  Same results as copying in, cg_run_step(run, 1), copying out, per
 * step.  Refused (CG_ESTATE) while added particles await initialization. */
int cg_run_step_host(cg_run *run, int32_t nsteps, const cg_host_arrays *in,
                     const cg_host_arrays *out, int32_t chunk, int32_t *bnd_stats);

/* ---- control sections ---------------------------------------------------- */
#define CG_MAX_SECTIONS 4096
/* Solver(control_sections=[...]) (solver.pyx:97-103, 542-549): each step
 * counts, per section, the particles whose step segment (step-start
 * position -> final position, both (0, 0) after a deletion in that step)
 * meets the section (ControlSection.c_cross, control_shapes.pyx:74-101).
 * The reference's ControlSection tests its first segment only
 * (nseg = poly.shape[1] - 1 = 1): segments[4*c .. 4*c+3] = x0, y0, x1, y1
 * of section c's first segment.  ncsec = 0 removes them.  Synchronous. */
int cg_run_set_sections(cg_run *run, int32_t ncsec, const double *segments);
/* The counts of the last cg_run_step: counts[nsteps][ncsec] (caller-sized
 * from *nsteps; pass counts = NULL to ask for nsteps first).  Host copy,
 * no device work. */
int cg_run_section_stats(const cg_run *run, int32_t *counts, int32_t *nsteps);

/* ---- stranding output --------------------------------------------------- */
/* parameters['stranding_output'] (compute_bc.pyx:109-121): on, each
 * cg_run_step records the position of every particle that strands on a wall
 * (its end-of-step position; z = 0 in 2D). */
int cg_run_set_stranding_output(cg_run *run, int32_t on);
/* The last cg_run_step's stranded positions, xyz[count][3], in the order the
 * reference's particle loop appends them (by step, then particle index);
 * xyz = NULL asks for the count only.  Host copy, no device work. */
int cg_run_stranded(const cg_run *run, double *xyz, int32_t *count);

/* ---- particle snapshots (host only) ------------------------------------- */
/* parameters['output_file'] every output_printout_period iterations
 * (write_particles.pyx:52-91).  Host arrays of the whole pool (n entries;
 * an entry is written when tri != -1, i.e. active); fvs is read when
 * model >= 2, diameter (may be NULL) adds the polydisperse column, depth
 * (may be NULL) the compute_depth column (writer_txt.pyx:177-178,
 * writer_vtk.pyx:277-283).
 * cg_snapshot_txt appends one block to <path> (writer_txt.pyx:25-180);
 * cg_snapshot_vtk writes <path> (writer_vtk.pyx:25-304).  Byte-identical to
 * the reference's files; formatted on all host threads.  No device work. */
int cg_snapshot_txt(const char *path, int32_t dim, int32_t model, double time,
                    int64_t iteration, int32_t n, const int32_t *tri, const int32_t *tag,
                    const double *pos, const double *vel, const double *fvs,
                    const double *diameter, const double *depth);
int cg_snapshot_vtk(const char *path, int32_t dim, int32_t model, double time,
                    int64_t iteration, int32_t n, const int32_t *tri, const int32_t *tag,
                    const double *pos, const double *vel, const double *fvs,
                    const double *diameter, const double *depth);

/* ---- particles added during a run -------------------------------------- */
/* Points the run at a new (larger) particle state after the caller grew
 * its arrays (LagrangianParticleSet._increase_pool_size,
 * lagrangian_particle_set.pyx:522-582); scratch follows the new count.
 * Synchronous. */
int cg_run_resize(cg_run *run, const cg_state_desc *state);
/* Particles the caller set to tri == -2 (LagrangianParticleSet.add,
 * lagrangian_particle_set.pyx:620-710: released by a source) get their
 * PCG32 streams, pcg32_seed(seed, tag); those with an index below n_init are
 * initialized (Solver.initialize_particle_state, solver.pyx:238-379) with the
 * fields of the next step, which then advances them (solver.pyx:443-470).
 * The reference's step loop covers the pool size it had before the sources
 * added (solver.pyx:430, 462): particles placed in a grown pool wait one
 * step, which the caller reproduces with n_init = that size and a second
 * call before the following step.  One deleted in its initialization
 * (outside the mesh) gets tag -2 - iteration, like a particle deleted in
 * that step. */
int cg_run_added(cg_run *run, int32_t n_init);

/* ---- serving pool ----------------------------------------------------- */
/* Many dispersion runs on one context's mesh and frozen fields, stepped
 * together: one launch per step advances every admitted run (continuous
 * batching; the step is captured once in a CUDA graph).  No reference
 * counterpart: the reference runs one Solver per process
 * (cylag/core/solver.pyx:42-80, solver_parallel.pyx:113-179); each run here
 * is that Solver's 2D step sequence, with the same results.
 *
 * Creates a pool of `capacity` particles (rounded up to 32) and `max_runs`
 * run slots on fields of 2D (frozen: the first time record is used);
 * schmidt_number is the one the nodal k-epsilon diffusivity is computed with.
 * Fails with CG_ENOMEM_BUDGET beyond the context budget.  Destroy every
 * server of a context before the context. */
typedef struct cg_server cg_server;
int cg_server_create(cg_ctx *ctx, int32_t precision, int64_t capacity, int32_t max_runs,
                     double schmidt_number, cg_server **out);
int cg_server_destroy(cg_server *srv);
/* Admits a run: n particles at host positions [n][2] (the Solver's
 * particle set), parameters as for cg_run_create (params->seed seeds its
 * PCG32 streams pcg32_seed(seed, i), i = 0..n-1; precision must be the
 * pool's; frozen fields), per-particle diameters from `diameter` [n] or all
 * `particle_diameter`, `horizon` steps.  Initializes the particles
 * (Solver.initialize_particle_state, solver.pyx:238-379); the run's step 0
 * is the next cg_server_step step.  CG_ENOMEM_BUDGET when no contiguous
 * range of the pool (or no run slot) is free: retry after a release. */
int cg_server_admit(cg_server *srv, const cg_params *params, int32_t n, const double *position,
                    double particle_diameter, const double *diameter, int32_t horizon,
                    int32_t *run_id);
/* Advances every admitted, unfinished run by nsteps steps (Solver.forward,
 * solver.pyx:413-585, for each), one graph launch per step.  Asynchronous. */
int cg_server_step(cg_server *srv, int32_t nsteps);
/* Steps the run still needs (0: finished once the queued steps complete). */
int cg_server_run_status(const cg_server *srv, int32_t run_id, int32_t *steps_left);
/* Copies a finished run's state to host arrays (NULL to skip): position,
 * velocity, fluid_velocity_seen [n][2]; tri, tag [n] (tag -1: deleted at
 * initialization, -2-k: deleted at step k; retag as
 * lagrangian_particle_set.pyx:754-788 does); rng_state [n].  Waits for the
 * run's last step only.  CG_EDEVICE (with the flags) if the run raised a
 * device error flag. */
int cg_server_read(cg_server *srv, int32_t run_id, double *position, double *velocity,
                   double *fluid_velocity_seen, int32_t *tri, int32_t *tag,
                   uint64_t *rng_state, uint32_t *err_flags);
/* Frees the run's slot and range (an unfinished run is cancelled). */
int cg_server_release(cg_server *srv, int32_t run_id);
/* Pool occupancy and the mean device time per step of the last
 * cg_server_step call (waits for it). */
int cg_server_stats(cg_server *srv, int32_t *active_runs, int64_t *active_particles,
                    int64_t *largest_free_range, int64_t *steps_issued, double *last_step_ms);

/* ---- measurement ------------------------------------------------------ */
/* Mean device time (ms) per step of the step kernel (and, for 2D LSM1
 * runs, the walk kernel) over the last cg_run_step call, measured with CUDA
 * events on the context stream; launches = every kernel that call launched
 * (step, walk, field time interpolation, element sort). */
int cg_run_last_kernel_ms(const cg_run *run, double *ms, int32_t *launches);

/* The same time split: the step kernel alone and the walk kernel alone
 * (0 for runs without a walk), mean ms per step over the last cg_run_step
 * call. */
int cg_run_last_kernel_split_ms(const cg_run *run, double *step_ms, double *walk_ms);

/* ---- checkpoint / resume ------------------------------------------------ */
/* The run's clock: simulated time, the time its current field record was
 * blended at (NaN for frozen fields or before the first step) and the
 * iteration count.  A checkpoint stores them with the particle state
 * (every array of cg_state_desc, the PCG32 states included). */
int cg_run_clock(const cg_run *run, double *time, double *fields_time, int64_t *iteration);

/* Resume a checkpoint in a run over the same mesh, fields and parameters,
 * whose state arrays now hold the checkpoint's particle state (write the
 * arrays after cg_run_writeback): the clock is set and the current field
 * record re-blended at fields_time, so that the following steps are bit for
 * bit those of the uninterrupted run (the plain form; the mixed form's
 * FP32-pair working positions round-trip through the FP64 arrays exactly
 * except at rounding ties).  CG_ESTATE while added particles await
 * initialization. */
int cg_run_resume(cg_run *run, double time, double fields_time, int64_t iteration);

#ifdef __cplusplus
}
#endif
#endif
