/* bora_flip.h - C ABI of the GB300-native sparse-grid FLIP substep.
 *
 * Drop-in boundary for the one call the reference's Houdini node makes per frame:
 * Bora::FLIPMethod (base/header/FLIPMethod.h:13-126, base/source/FLIPMethod.cu), used by
 * SOP_FlipWater (houdini/source/SOP_FlipWater.cpp:122-137, 282-292, 315-323, 358, 362).
 * The reference exposes a C++ class with unified-memory arrays and no error reporting;
 * this header exposes the same operations as plain C functions over an opaque handle,
 * host pointers and sizes, each returning a status code. include/BoraFLIPMethod.hpp
 * wraps it back into a FLIPMethod-shaped C++ class.
 *
 * Coordinates: "world" space is the caller's (the SOP's), "voxel" space is the
 * reference's internal cell space (dx = 1, Grid::voxelPoint, base/header/Grid.h:446).
 * Particle arrays are interleaved x,y,z floats, like Bora::Vec3fArray.
 *
 * Threading: a handle may be used from one host thread at a time. All work runs on one
 * CUDA stream owned by the handle, on the device that was current at creation.
 */
#ifndef BORA_FLIP_H
#define BORA_FLIP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BORA_FLIP_ABI_VERSION 1

/* Status codes. 0 = success; negative = error; positive = completed with a warning. */
#define BORA_OK 0
#define BORA_ERR_INVALID_ARG -1
#define BORA_ERR_OUT_OF_MEMORY -2
#define BORA_ERR_CUDA -3
#define BORA_ERR_NO_DEVICE -4
#define BORA_ERR_INTERNAL -5
#define BORA_ERR_CAPACITY -6
#define BORA_WARN_NOT_CONVERGED 1

/* Particle coordinate space of a call. */
#define BORA_SPACE_WORLD 0
#define BORA_SPACE_VOXEL 1

/* Pressure-solver forms. */
#define BORA_SOLVER_PLAIN 0 /* FP32 PCG, block-MIC(0) preconditioner, FP64-accurate dots, double-float refinement */
#define BORA_SOLVER_MIXED 1 /* FP32 PCG, multigrid V-cycle (FP16 storage), FP64-accurate dots, double-float refinement */

/* particle advection (bora_flip_params.advection) */
#define BORA_ADVECT_EULER 0
#define BORA_ADVECT_RK2 1

/* Grid description: nx*ny*nz cells over the world box [min, max]
 * (Grid::initialize(Nx,Ny,Nz,min,max), base/header/Grid.h:124-141). The simulation grid
 * is this grid padded to a multiple of 4 cells per axis and re-centred
 * (SparseFrame::initialize, base/source/SparseFrame.cu:28-73). */
typedef struct bora_grid_desc
{
    int nx, ny, nz;
    float min[3];
    float max[3];
} bora_grid_desc;

/* Parameters: the first block mirrors Bora::FLIPMethod::Params field for field
 * (base/header/FLIPMethod.h:51-67) with the same defaults; the second block adds the
 * solver controls the reference hard-codes (LinearSystemSolver.cpp:39,46). */
typedef struct bora_flip_params
{
    float ext_force[3];      /* (0, -9.80665, 0) world units / s^2 */
    int max_substeps;        /* 1 */
    float dt;                /* 1/24 s */
    float wall_level;        /* -1e30: world height below which walls are solid */
    int enable_water_tank;   /* 0 */
    int enable_curl;         /* 0 (curl noise is not implemented; must be 0) */
    float damping_band;      /* 0 */
    float voxel_size;        /* 0.1 */
    float col_vel_scale;     /* 1 */
    int pts_per_cell;        /* 8 */
    float vort_pres_rate;    /* 0.2 (post-processing only) */
    float adjacency_under;   /* 2 (curl only) */
    int proj_iteration;      /* 200: cap on inner PCG iterations per refinement pass */
    int redist_iteration;    /* 80 (post-processing only) */
    /* additions */
    int solver;              /* BORA_SOLVER_PLAIN */
    double tolerance;        /* 1e-6: stop when ||b - A p||_2 / ||b||_2 < tolerance ... */
    double div_tolerance;    /* 1e-5: ... and max_i |b - A p|_i * dx_world < div_tolerance */
    double inner_tolerance;  /* 1e-3: relative residual reduction of each FP32 inner solve (the
                                recurrence continues across passes while the refined and FP32 residuals agree) */
    int max_refinements;     /* 8: outer refinement passes (double-float iterate and residual) */
    int check_every;         /* 1: inner iterations between convergence checks (read back one iteration late) */
    int advection;           /* BORA_ADVECT_EULER: particle positions follow the particle velocity
                                (FLIPMethod.cu:124-145); BORA_ADVECT_RK2: midpoint rule in the grid
                                velocity field, per substep */
    int post_process;        /* 1: bora_flip_frame post-processes after the step, as
                                FLIPMethod::advanceOneFrame does (FLIPMethod.cu:177-206) */
    int persistent;          /* 0: one launch per PCG phase, convergence read back by the host
                                (check_every); 1: the plain form runs each refinement pass's inner
                                PCG in one cooperative launch whose phases meet at bounded grid
                                barriers and which checks convergence itself */
    int warm_start;          /* 0: every pressure solve starts from p = 0, as the reference's does
                                (its pressure field is re-created with the frame each step,
                                FLIPMethod.cu:28-33, FluidProjection.cu:265); 1: from the last
                                step's pressure in the cells whose tiles were active then (0
                                elsewhere, and wherever that start is no closer to the solution
                                than p = 0); the stop rule is the same. Batched steps
                                (bora_flip_step_batch) take such simulations on their own */
} bora_flip_params;

typedef struct bora_flip_stats
{
    uint64_t steps;               /* steps taken */
    uint64_t num_particles;       /* live particles after the last step */
    uint64_t killed_last_step;
    int32_t active_tiles;         /* 8^3 tiles in the last rebuild */
    int32_t fluid_cells;
    int32_t solver_iterations;    /* inner PCG iterations, all refinement passes */
    int32_t refinements;
    double residual_rel;          /* ||b - A p||_2 / ||b||_2, FP64 */
    double residual_max;          /* max_i |b - A p|_i (1/s) */
    double residual_max_dx;       /* residual_max * dx_world */
    int32_t converged;
    int32_t mg_vcycle_launches;   /* kernel launches per V-cycle in the last solve (mixed form), else 0 */
    double stage_ms[8];           /* host wall time of the last step: rebuild, p2g, system, solve,
                                     velocity, particles, -, total; after a batched step
                                     (bora_flip_step_batch) the batch's: [0] the stages before
                                     the solve, [3] the solve, [5] the stages after it, [7] total */
    double gpu_ms;                /* device time of the last step (CUDA events on the handle's stream) */
    uint64_t kernel_launches;     /* kernels launched by this handle since creation */
    uint64_t device_bytes;        /* device memory the handle holds */
} bora_flip_stats;

/* Kernel classes for opt-in per-kernel device timing (bora_flip_set_profiling). */
#define BORA_KERNEL_BIN 0
#define BORA_KERNEL_TILES 1        /* activation, tile scan, tile table, neighbour table */
#define BORA_KERNEL_SORT 2         /* dual-cell histogram, scan, scatter */
#define BORA_KERNEL_P2G 3
#define BORA_KERNEL_RHS 4          /* right-hand side, stencil code, preconditioner set-up */
#define BORA_KERNEL_PCG_DIRECTION 5
#define BORA_KERNEL_PCG_UPDATE 6
#define BORA_KERNEL_REFINE 7       /* solver init, refinement, pressure write-back */
#define BORA_KERNEL_VELOCITY 8
#define BORA_KERNEL_G2P 9
#define BORA_KERNEL_MG 10          /* multigrid V-cycle (mixed solver) */
#define BORA_KERNEL_POST 11        /* post-processing: splat, tank scan, redistancing, attributes */
#define BORA_KERNEL_CLASSES 16

/* Simulation frame description (after padding). */
typedef struct bora_frame_info
{
    int nx, ny, nz;        /* simulation grid in cells */
    int tx, ty, tz;        /* 8^3 tiles per axis */
    int tile;              /* 8 */
    int active_tiles;
    float translate[3];    /* world position of voxel (0,0,0) */
    float scale[3];        /* world size of a voxel */
    float voxel_wall_level;
    float voxel_gravity[3];
} bora_frame_info;

typedef struct bora_flip_sim* bora_flip_handle;

/* Default parameters (FLIPMethod::Params defaults, FLIPMethod.h:51-67). */
int bora_flip_default_params( bora_flip_params* out );

/* FLIPMethod::initialize (FLIPMethod.cu:16-47). */
int bora_flip_create( const bora_grid_desc* grid, const bora_flip_params* params, bora_flip_handle* out );
int bora_flip_destroy( bora_flip_handle h );
int bora_flip_set_params( bora_flip_handle h, const bora_flip_params* params );

/* FLIPMethod::newParticle (FLIPMethod.h:75-99), batched: append n particles from host
 * memory (pinned memory copies fastest). Velocities may be NULL (zero). */
int bora_flip_add_particles( bora_flip_handle h, const float* pos, const float* vel, size_t n, int space );
/* Replace all particles (ids restart at 0). */
int bora_flip_set_particles( bora_flip_handle h, const float* pos, const float* vel, size_t n, int space );
int bora_flip_clear_particles( bora_flip_handle h );
/* FLIPMethod::fillWaterTank (FLIPMethod.cu:407-478): append the water tank's particles
 * below the wall level (params.wall_level) with zero velocity, in the reference's order and
 * at its positions; params.pts_per_cell extra particles per cell fill the 4-cell band under
 * the wall. *added (may be NULL) receives the count. With params.enable_water_tank the tile
 * rows below the wall stay active every step (SparseFrame.cu:119-129). */
int bora_flip_fill_water_tank( bora_flip_handle h, size_t* added );

/* CollisionSource (base/header/CollisionSource.h): up to 8 analytic boxes, 9 floats each
 * (lo xyz, hi xyz, velocity xyz) in voxel space; samples are clamped to +-band. */
int bora_flip_set_colliders( bora_flip_handle h, const float* boxes, int n, float band );
/* CollisionSource::update (CollisionSource.h:66-126) from raw buffers instead of OpenVDB
 * grids: the collider's signed distance (voxel units, negative inside) and velocity (voxel
 * units per second; NULL = at rest) at the cell centres of the frame grid (bora_frame_info
 * nx, ny, nz; x fastest), ncells = nx*ny*nz. Normals are central differences of the
 * distances, as for boxes. Replaces any boxes; phi = NULL removes the collider. */
int bora_flip_set_collider_field( bora_flip_handle h, const float* phi, const float* vel, size_t ncells );
/* CollisionSource::update (CollisionSource.h:66-126) from a level set's active voxels, the
 * form OpenVDB's active-value iterator yields: count voxels at frame cells ijk (3 int32
 * each; cells outside the frame grid are ignored) with the signed distance phi (world
 * units, negative inside) and velocity vel (3 floats, world units per second; NULL = at
 * rest) sampled at those cells' centres, and the level set's background (world units).
 * As SparseFrame::buildFromPoints does for the reference's collider frame, every 8^3 tile
 * that holds an active voxel or neighbours one becomes a collider tile; its cells store
 * phi / dx and vel / dx (voxel units), cells without a voxel the background / dx, and every
 * other cell reads the background with zero velocity and normal. Normals are normalised
 * central differences of the stored distances. Memory follows the collider's tiles, not
 * the frame. Replaces boxes or a per-cell field; count = 0 removes the collider. */
int bora_flip_set_collider_voxels( bora_flip_handle h, const int32_t* ijk, const float* phi, const float* vel,
                                   size_t count, float background );

/* FLIPMethod::advanceOneStep (FLIPMethod.cu:208-298) in voxel space. Returns
 * BORA_WARN_NOT_CONVERGED when the pressure solve stopped on its iteration caps. */
int bora_flip_step( bora_flip_handle h, float dt );
/* Several independent simulations one step each (FLIPMethod::advanceOneStep for every
 * handle), with the pressure solve - almost all of a step's kernel launches - launched once
 * per kernel for all of them: the blocks of the simulations taking part are packed back to
 * back in each launch, simulation k running exactly the blocks of its own launch with its
 * own reductions and convergence, so each handle's result is the same as from
 * bora_flip_step_batch with that handle alone, whatever else is in the batch. The other
 * stages run on each handle's own stream, every part issued for all handles before the host
 * waits on any. A batched step keeps the multigrid levels 0-3 and one dense level in every
 * hierarchy, so a scene with fewer than 512 active tiles solves on more levels than in
 * bora_flip_step (from 512 tiles up the two give the same bits). Handles of the plain solver
 * form (or whose hierarchy does not fit the batched coarse-level kernel) take a
 * bora_flip_step of their own. status[k] receives handle k's step status; the handles must
 * live on one device and be distinct. After the call, stage_ms of the batched handles holds
 * the batch's phase times. */
int bora_flip_step_batch( bora_flip_handle* hs, int n, float dt, int* status );

/* FLIPMethod::advanceOneFrame (FLIPMethod.cu:177-206): one step of params.dt, then (with
 * params.post_process) bora_flip_post_process. */
int bora_flip_frame( bora_flip_handle h );

/* FLIPMethod::postProcess (FLIPMethod.cu:300-405), the surface pipeline that follows the
 * step in a frame: rebuild the tiles from the current particles (prepareNextStep; the
 * next step reuses them), splat the surface and velocity
 * (Rasterization::ParticlesToSurfaceAndVelocity, Rasterization.cu:311-398; influence 1.5,
 * droplet 0.5), with the water tank turn enclosed air below the wall level into liquid
 * (surf = -5), params.redist_iteration redistancing steps
 * (Rasterization::ReinitializeSurface, Rasterization.cu:400-486), then update the
 * particles' vorticity (decay (1 - params.vort_pres_rate)^params.dt) and curvature.
 * Afterwards BORA_FIELD_SURF holds the signed distance (voxel units, negative in the
 * liquid), BORA_FIELD_VELO the splatted velocity, BORA_FIELD_COMP the surface normals and
 * BORA_FIELD_PRES zero. The splat's sums are added in no fixed order (as the reference's
 * atomics). The tank's scan is the 6-connected fill of air from the wall layer and the
 * far corner; the reference's host loop reads its popped cell through a reference that
 * the loop's first push overwrites (FLIPMethod.cu:335-337), which can leave air cells of
 * one-cell-wide passages unreached that are reached here. */
int bora_flip_post_process( bora_flip_handle h );

/* The parts of bora_flip_post_process, for tests and callers that interleave their own
 * work. All need the tiles of a rebuild (BORA_STAGE_REBUILD, or a post-processing);
 * BORA_POST_SPLAT also needs the particles unchanged since. */
#define BORA_POST_SPLAT 0        /* zero the fields, splat, normalise (surf, pres = weight sum, velo, comp = mean position) */
#define BORA_POST_TANK_SCAN 1    /* water tank only: enclosed air below the wall -> surf = -5 */
#define BORA_POST_REDISTANCE 2   /* params.redist_iteration steps on surf (pres is the scratch field) */
#define BORA_POST_ATTRIBUTES 3   /* curl -> vorticity, normals -> comp, curvature -> particles, pres = 0 */
int bora_flip_run_post_stage( bora_flip_handle h, int stage );

/* Particles::vorticity / ::curvature of the live particles, in bora_flip_get_particles'
 * order (ids as there; any pointer may be NULL; zero before the first post-processing). */
int bora_flip_get_particle_attributes( bora_flip_handle h, float* vorticity, float* curvature, int32_t* ids,
                                       size_t cap, size_t* n );
/* Replace them (n = live particles, in bora_flip_get_particles' order; NULL = zeros). */
int bora_flip_set_particle_attributes( bora_flip_handle h, const float* vorticity, const float* curvature, size_t n );

/* The stages of one step, for callers that interleave their own work and for tests. */
#define BORA_STAGE_REBUILD 0          /* SparseFrame::buildFromPoints */
#define BORA_STAGE_P2G 1              /* P2G + count field + cell flags */
#define BORA_STAGE_BUILD_SYSTEM 2     /* FluidProjection::buildLinearSystem */
#define BORA_STAGE_SOLVE 3            /* pressure solve */
#define BORA_STAGE_UPDATE_VELOCITY 4  /* FluidProjection::solve after the solver */
#define BORA_STAGE_UPDATE_PARTICLES 5 /* FLIPMethod::updateParticles + compaction */
int bora_flip_run_stage( bora_flip_handle h, int stage, float dt );

int bora_flip_num_particles( bora_flip_handle h, size_t* n );
/* Copy live particles to host memory (any pointer may be NULL). ids identify particles
 * across steps (the order of particles changes every step). cap = capacity in particles. */
int bora_flip_get_particles( bora_flip_handle h, float* pos, float* vel, float* adjacency, int32_t* ids, size_t cap,
                             size_t* n, int space );

/* Asynchronous export of the current particles (the SOP's per-frame attribute export,
 * SOP_FlipWater.cpp:205-248): the live particles, their adjacency-free attributes and ids are
 * gathered on the handle's stream into a device export buffer (in bora_flip_get_particles'
 * order) and copied to the given host buffers on a second stream; the call returns at once.
 * A following bora_flip_step / frame runs while the copy is in flight (pinned host buffers
 * give full overlap). The host buffers must stay valid until bora_flip_export_wait; a new
 * export first waits for the previous one. *n = live particles. Any pointer may be NULL. */
int bora_flip_export_begin( bora_flip_handle h, float* pos, float* vel, float* vorticity, float* curvature,
                            int32_t* ids, size_t cap, int space, size_t* n );
int bora_flip_export_wait( bora_flip_handle h );

int bora_flip_frame_info( bora_flip_handle h, bora_frame_info* out );
/* Active tiles as (i,j,k) tile coordinates, in storage (slot) order. */
int bora_flip_get_tiles( bora_flip_handle h, int32_t* ijk, size_t cap_tiles );

/* Grid fields in tile storage order (active tiles x 512 cells, x fastest in a tile). */
#define BORA_FIELD_MASS 0      /* float  (getDensityField) */
#define BORA_FIELD_SURF 1      /* float  particle count per cell after a step; signed distance after post-processing */
#define BORA_FIELD_PRES 2      /* float  */
#define BORA_FIELD_VELO 3      /* 3 float per cell (pre-projection grid velocity, getVelocityField; splatted velocity after post-processing) */
#define BORA_FIELD_COMP 4      /* 3 float per cell (projected grid velocity; surface normals after post-processing) */
#define BORA_FIELD_FLAG 5      /* uint8: 0 air, 1 solid, 4 fluid, 255 beyond the grid */
#define BORA_FIELD_RHS 6       /* float  right-hand side b = -div (fluid cells) */
#define BORA_FIELD_CODE 7      /* uint16 stencil code (bit 15 fluid, bits 8-11 diagonal, bits 0-5 fluid nbrs) */
int bora_flip_get_field( bora_flip_handle h, int which, void* out, size_t bytes );

/* The SOP's sparse -> VDB conversions after a frame (SOP_FlipWater.cpp:252-264):
 * FieldCast's convertSurfaceVDB (base/header/FieldCast.h:362-440) and convertVelocityVDB
 * (FieldCast.h:14-48), computed on the device and returned as OpenVDB leaf nodes: 8^3
 * voxel blocks at multiples of 8 (VDB voxel (i,j,k) = the frame's cell (i,j,k); x fastest
 * inside a leaf, bit l of the 512-bit mask = voxel l). Per leaf: origins 3 int32 (voxel
 * coordinates, may be negative), masks 8 uint64 (active voxels), values 512 floats
 * (BORA_VDB_SURFACE) or 512 x 3 floats (BORA_VDB_VELOCITY).
 *   surface:  phi * dx (world units) on the cells of active tiles inside the grid, background
 *             * dx on inactive voxels; with params.enable_water_tank, the 3-cell border band
 *             around and below the grid up to 3 cells above params.wall_level becomes active
 *             with min(cell centre y - wall_level, value). Call after post-processing (the
 *             surface is then a signed distance with background 10 voxels).
 *   velocity: the splatted velocity times dx (world units per second), active where its
 *             length is not below 1e-30, 0 elsewhere.
 * Leaves without an active voxel are omitted. transform (4 floats, may be NULL): voxel size
 * dx and the translation min + dx/2 of the VDB linear transform; background (may be NULL).
 * With origins == NULL only *nleaves is set; BORA_ERR_CAPACITY when cap_leaves is short. */
#define BORA_VDB_SURFACE 0
#define BORA_VDB_VELOCITY 1
int bora_flip_export_vdb( bora_flip_handle h, int which, int32_t* origins, uint64_t* masks, float* values,
                          size_t cap_leaves, size_t* nleaves, float* transform, float* background );
int bora_flip_set_field( bora_flip_handle h, int which, const void* in, size_t bytes );

int bora_flip_get_stats( bora_flip_handle h, bora_flip_stats* out );

/* Record CUDA events around every launch of the kernel classes in `class_mask` (bit c =
 * class c) and accumulate their device time; setting a mask resets the totals. */
int bora_flip_set_profiling( bora_flip_handle h, uint32_t class_mask );
/* Time only one in `every` brackets of each profiled class (1, the default: all). A bracket
 * records an event on the handle's stream before and after the class's kernels, which ends the
 * programmatic overlap of a kernel with its neighbours in the solver chain; sampling keeps most
 * brackets of a long step free of it. The launch counts then count the timed brackets. */
int bora_flip_set_profiling_sampling( bora_flip_handle h, uint32_t every );
/* Accumulated device milliseconds and launch counts per kernel class (n <= 16 entries). */
int bora_flip_get_kernel_times( bora_flip_handle h, double* ms, uint64_t* launches, int n );
const char* bora_flip_status_string( int status );

/* Fault injection for tests of the error paths (no counterpart in the reference).
 * BORA_FAULT_BARRIER: the next solves' grid barriers (persistent plain PCG) wait for one
 * block more than they launch, so every wait runs out after a short limit, the kernel
 * returns, and the step returns BORA_ERR_INTERNAL with the handle still usable.
 * BORA_FAULT_NONE clears it. */
#define BORA_FAULT_NONE 0
#define BORA_FAULT_BARRIER 1
int bora_flip_set_fault( bora_flip_handle h, int fault );

/* Launch-shape autotuner (process-wide; no counterpart in the reference). Kernels with
 * several launch shapes that compute the same bits (the multigrid passes of levels 0-2:
 * tiles and threads per block) are timed in every shape on their first launches per
 * device and size class (floor(log2 tiles)), single simulations and batches apart; the
 * fastest median is kept. Tuning never changes a result. mode 1 = tune (the default),
 * 0 = the default shapes everywhere. With the environment variable BORA_TUNE_FILE set,
 * the table is read from that file on first use and written back when an entry is
 * decided. */
int bora_flip_set_tuning( int mode );
/* The table as text, one line per entry: "group device size_class shape median_ms"
 * (shape -1: still measuring). *len = its length; cap = 0 asks for the length only;
 * BORA_ERR_CAPACITY when cap cannot hold the text and its terminating zero. */
int bora_flip_tune_table( char* buf, size_t cap, size_t* len );

/* ---- device building blocks ------------------------------------------------------- */

/* Exclusive prefix sum of n uint32 counts in device memory: d_out[i] = sum_{j<i} d_in[j];
 * *d_total (device pointer, may be NULL) = sum of all. d_in and d_out may alias. Runs on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) and returns without
 * waiting. This is the compaction step of the sparse-frame rebuild: the reference
 * numbers its active tiles with a serial host loop over the tile-marker table
 * (base/source/SparseFrame.cu:131-152). Block sums go to stream-ordered scratch memory. */
int bora_scan_u32( const uint32_t* d_in, uint32_t* d_out, size_t n, uint32_t* d_total, void* stream );

/* bora_scan_u32 without any device allocation (this entry point has no counterpart in
 * the reference). For callers that cannot call cudaMalloc or the stream-ordered
 * allocator: a host plugin running under a fixed device-memory budget, code recorded
 * into a CUDA graph where allocation calls are not allowed, or real-time callbacks that
 * must not block on the allocator. The per-block sums go to a static device array of
 * 512 KiB that every device using the library keeps until the process exits, so
 * n <= 2^28 (268,435,456); larger n returns BORA_ERR_CAPACITY. The first call on a
 * device looks up the array's device address (a runtime call that does not allocate);
 * make that first call before any stream capture. All calls share the one array: two
 * calls whose work overlaps on the GPU (different streams, or different host threads)
 * race and must be serialised by the caller. Same arguments and results as
 * bora_scan_u32; returns without waiting for the GPU. */
int bora_scan_u32_noalloc( const uint32_t* d_in, uint32_t* d_out, size_t n, uint32_t* d_total, void* stream );

#ifdef __cplusplus
}
#endif

#endif /* BORA_FLIP_H */
