// Internal host-side declarations of the GB300 FLIP substep library (not installed).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "flip_common.cuh"

#include <atomic>
#include <utility>
#include <vector>

// ---- per-device values computed on first use ------------------------------------------
// Launch shapes and device attributes are queried once per device ordinal. Host threads
// that drive different handles (the serving layer runs one per request) may race to fill an
// entry: each computes the same value, and the entries are atomics. Declare instances with
// static storage (zero-initialised).
class BoraPerDevice
{
public:
    template <class F>
    int get( F compute )
    {
        int dev = 0;
        if( cudaGetDevice( &dev ) != cudaSuccess || dev < 0 || dev >= kMaxDevices ) return compute();
        int v = v_[dev].load( std::memory_order_acquire );
        if( v <= 0 )
        {
            v = compute();
            v_[dev].store( v, std::memory_order_release );
        }
        return v;
    }

private:
    static constexpr int kMaxDevices = 64;
    std::atomic<int> v_[kMaxDevices];
};

// ---- programmatic dependent launch ---------------------------------------------------
// The kernels of a solver iteration form a chain in which each one reads what the one
// before wrote. They are launched with programmatic stream serialisation: a kernel may
// start while its predecessor is finishing, runs the part of its prologue that touches
// only data no kernel of the chain writes (tile tables, stencil codes, index set-up), and
// then waits for the predecessor's completion (griddepcontrol.wait) before anything else.
// Each kernel of the chain allows its successor to launch as soon as all of its own CTAs
// have started (griddepcontrol.launch_dependents), so earlier kernels are never starved.
__device__ __forceinline__ void bora_pdl_trigger() { asm volatile( "griddepcontrol.launch_dependents;" ::: "memory" ); }
__device__ __forceinline__ void bora_pdl_wait() { asm volatile( "griddepcontrol.wait;" ::: "memory" ); }

template <typename... KArgs, typename... Args>
cudaError_t bora_launch_pdl( void ( *kernel )( KArgs... ), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                             Args&&... args )
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx( &cfg, kernel, std::forward<Args>( args )... );
}

// ---- scan ---------------------------------------------------------------------------
size_t bora_scan_scratch_elems( size_t n );
void bora_device_scan( const uint32_t* in, uint32_t* out, size_t n, uint32_t* scratch, uint32_t* total, cudaStream_t st );

// ---- particle arrays (structure of arrays) -------------------------------------------
struct BoraParticlesDev
{
    float* px;
    float* py;
    float* pz;
    float* vx;
    float* vy;
    float* vz;
    int32_t* id;  // < 0: killed in the last step
    float* vort;  // Particles::vorticity / ::curvature (post-processing), or null while unused
    float* curv;
};

// ---- cell fields over active slots x 512 ----------------------------------------------
struct BoraCellsDev
{
    float* mass;
    float* surf;  // particle count touching the cell (PointsToCountField)
    float* pres;
    float* vx;    // grid velocity after P2G and collider velocity ("velo")
    float* vy;
    float* vz;
    float* cx;    // projected grid velocity ("comp")
    float* cy;
    float* cz;
    uint8_t* flag;
    uint16_t* code;
    float* b;
};

// Tile tables.
struct BoraTilesDev
{
    const int32_t* slot_of;   // [virtual tiles] -> slot or -1
    const int32_t* tile_of;   // [slots] -> virtual tile linear index
    const int32_t* nbr;       // [slots * 27] -> neighbour slot or -1
};

// Scalars that the solver kernels exchange on the device (ring of FP64 reductions).
#define BORA_RING 64
// Largest grid of a kernel that reduces through BoraReduceDev::partials (one slot pair per
// block). Every such launcher clamps its grid to this, and the handle sizes the partials
// buffer for at least this many blocks.
constexpr int kBoraMaxReduceBlocks = 152 * 16;
struct BoraReduceDev
{
    double* ring;        // [BORA_RING * 4]: slot values
    double* partials;    // [max blocks * 2]
    uint32_t* done;      // [BORA_RING] block-arrival counters
    uint32_t* err;       // set non-zero by a kernel that met an inconsistent stencil code
    double* mirror;      // [BORA_RING] host-mapped copy of the slot values, or null
};

// ---- launchers -----------------------------------------------------------------------
void bora_launch_bin( const BoraGridDev& g, BoraParticlesDev p, size_t n, uint32_t* vkey, uint8_t* tile_flag, cudaStream_t st );
void bora_launch_activate( const BoraGridDev& g, const uint8_t* tile_flag, uint32_t* act, cudaStream_t st );
// FLIPMethod::fillWaterTank: count (write = false) or write the tank's particles.
void bora_launch_tank( const BoraGridDev& g, int hh, int per_cell, float3 tr, float3 sc, uint32_t* count,
                       const uint32_t* offset, BoraParticlesDev p, size_t base, int32_t first_id, bool write,
                       cudaStream_t st );
void bora_launch_tile_assign( const BoraGridDev& g, const uint32_t* act, const uint32_t* excl, int32_t* slot_of,
                              int32_t* tile_of, cudaStream_t st );
void bora_launch_tile_nbrs( const BoraGridDev& g, int ntiles, const int32_t* slot_of, const int32_t* tile_of,
                            int32_t* nbr, cudaStream_t st );
void bora_launch_hist( size_t n, const uint32_t* vkey, const int32_t* slot_of, uint32_t outside_key, uint32_t* key,
                       uint32_t* count, uint32_t* err, cudaStream_t st );
void bora_launch_scatter( size_t n, const uint32_t* key, const uint32_t* start, uint32_t* count, uint32_t* idx,
                          cudaStream_t st );
void bora_launch_order_bins( size_t nbins, const uint32_t* start, uint32_t* idx, cudaStream_t st );
void bora_launch_p2g( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraParticlesDev p, const uint32_t* idx,
                      const uint32_t* start, BoraCellsDev c, cudaStream_t st );
void bora_launch_rhs( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, uint32_t* nfluid, cudaStream_t st );
void bora_launch_vel_update( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, cudaStream_t st );
void bora_launch_g2p( const BoraGridDev& g, int ntiles, size_t nsorted, BoraTilesDev t, const uint32_t* start, BoraCellsDev c,
                      BoraParticlesDev src, const uint32_t* idx, BoraParticlesDev dst, float* adj, float dt,
                      uint32_t* nkilled, uint32_t* vkey, uint8_t* tile_flag, cudaStream_t st );
// ---- post-processing (FLIPMethod::postProcess) ------------------------------------------
void bora_launch_splat( const BoraGridDev& g, int ntiles, BoraTilesDev t, const uint32_t* start, const uint32_t* idx,
                        BoraParticlesDev p, BoraCellsDev c, cudaStream_t st );
// labels: ntiles * 512 + tiles-table entries; returns the number of kernels launched
int bora_tank_scan_launches( const BoraGridDev& g, int ntiles, BoraTilesDev t, float* surf, uint32_t* labels,
                             uint32_t* err, cudaStream_t st );
cudaError_t bora_launch_redistance( const BoraGridDev& g, int ntiles, BoraTilesDev t, const float* in, float* out,
                                    cudaStream_t st );
// curl of velo -> (wx, wy, wz); normals of surf -> comp; curvature of the normals -> pres
void bora_launch_surface_fields( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, float* wx, float* wy,
                                 float* wz, cudaStream_t st );
void bora_launch_particle_attributes( const BoraGridDev& g, const int32_t* slot_of, size_t np, BoraParticlesDev p,
                                      const float* wx, const float* wy, const float* wz, const float* curvature,
                                      float3 scale, float dis, cudaStream_t st );

// ---- sparse -> VDB leaf export (FieldCast convertSurfaceVDB / convertVelocityVDB) ------
// leaf_ijk: 3 ints (voxel origin) per leaf; leaf_slot: its tile's slot or -1 (band leaf);
// mask: 8 x 64 bits per leaf; val: 512 (surface) or 3 x 512 (velocity) floats per leaf.
void bora_launch_vdb_surface( const BoraGridDev& g, const float* scale, const float* translate, int nleaves,
                              const int32_t* leaf_ijk, const int32_t* leaf_slot, const float* surf, float bg, int tank,
                              float level, uint64_t* mask, float* val, cudaStream_t st );
void bora_launch_vdb_velocity( const BoraGridDev& g, const float* scale, int nleaves, const int32_t* leaf_ijk,
                               const int32_t* leaf_slot, const float* vx, const float* vy, const float* vz,
                               uint64_t* mask, float* val, cudaStream_t st );
int bora_vdb_level_index( float level, float min_y, float dx );
// tile coordinates (3 ints each) of the water tank's border band (FieldCast.h:398-440)
void bora_vdb_band_tiles( const BoraGridDev& g, const float* scale, const float* translate, float level,
                          std::vector<int32_t>& tiles );

void bora_launch_to_soa( size_t n, const float* pos, const float* vel, int space, const float* translate,
                         const float* scale, BoraParticlesDev p, size_t offset, int32_t first_id, cudaStream_t st );

// ---- pressure solve -------------------------------------------------------------------
struct BoraSolverDev
{
    float2* x;      // pressure iterate of the refinement as a double-float pair (hi, lo): ~48 bits
    float* e;       // inner correction
    float* r;       // residual
    float* d[2];    // search directions (ping-pong)
    float* q;       // A d
    float* z;       // preconditioned residual
    float* minv;    // block-MIC(0) inverse pivots
};

void bora_launch_mic_factor( const BoraGridDev& g, int ntiles, const uint16_t* code, float* minv, cudaStream_t st );
// r = b, x = 0, e = 0, d = 0, q = 0; partial sums of ||b||^2 and max|b| -> ring slots
void bora_launch_solve_init( int ntiles, const float* b, const uint16_t* code, BoraSolverDev s, BoraReduceDev red,
                             int slot_norm2, int slot_max, cudaStream_t st );
// e += alpha d; r -= alpha q; z = M^-1 r; rz, rr -> ring slots (alpha = rz_in / dq_in, or 0 when slot_rz_in < 0)
void bora_launch_pcg_update( int ntiles, const uint16_t* code, BoraSolverDev s, BoraReduceDev red, int slot_rz_in,
                             int slot_dq_in, int slot_rz_out, int slot_rr_out, cudaStream_t st );
// d' = z + beta d; q = A d'; dq -> ring slot (beta = rz_new / rz_old, or 0 when slot_rz_old < 0)
// One refinement pass of the plain form's inner PCG in one cooperative launch with bounded
// grid barriers (projection.cu). Outputs: ring slots slot_a_rz / slot_a_dq (the last
// update's alpha, whose e += alpha d is pending), slot_rr (the last r.r), *iters. bar: two
// zeroed words; part: 3 * bora_pcg_persistent_grid() doubles. never_release: every barrier
// wait runs out (a test of the error path). Returns 0, or -1 when the launch is refused.
#define BORA_REDUCE_ERR_BARRIER 0x100u  // a grid barrier wait ran out
int bora_pcg_persistent_grid();
int bora_launch_pcg_persistent( int ntiles, const int32_t* nbr, const uint16_t* code, BoraSolverDev s, BoraReduceDev red,
                                int dsel, int slot_rz_prev, int max_inner, double target, int slot_a_rz, int slot_a_dq,
                                int slot_rr, uint32_t* iters, unsigned* bar, double* part, bool never_release,
                                cudaStream_t st );
void bora_launch_pcg_direction( const BoraGridDev& g, int ntiles, BoraTilesDev t, const uint16_t* code, BoraSolverDev s,
                                int dsel_in, BoraReduceDev red, int slot_rz_new, int slot_rz_old, int slot_dq_out,
                                int slot_a_rz, int slot_a_dq, cudaStream_t st );
// x += e (FP64); e = 0; d = 0; q = 0
// x = the last step's pressure on fluid cells, read through the previous tile table (the warm start)
void bora_launch_solve_warm( int ntiles, const uint16_t* code, const int32_t* tile_of, const int32_t* slot_prev,
                             const float* pres, BoraSolverDev s, cudaStream_t st );
void bora_launch_refine_accumulate( int ntiles, const uint16_t* code, BoraSolverDev s, int dsel, const double* ring,
                                    int slot_a_rz, int slot_a_dq, cudaStream_t st );
// r = b - A x in FP64 (stored FP32); ||r||^2 and max|r| -> ring slots
void bora_launch_refine_residual( const BoraGridDev& g, int ntiles, BoraTilesDev t, const float* b, const uint16_t* code,
                                  BoraSolverDev s, BoraReduceDev red, int slot_norm2, int slot_max, cudaStream_t st );
// pres = (float) x on fluid cells, 0 elsewhere
void bora_launch_write_pressure( int ntiles, const uint16_t* code, const float2* x, float* pres, cudaStream_t st );


// ---- multigrid preconditioner (mixed form) ----------------------------------------------
struct BoraLevelDev
{
    int kind;          // 0 = tiled (E cells per tile edge), 1 = dense grid
    int E;             // tiled levels: 8, 4, 2, 1
    int level;         // 0 = fine grid
    int nx, ny, nz;    // cells of this level inside the domain
    int dx, dy, dz;    // dense storage extent (dense levels)
    size_t ncells;     // stored cells
    uint8_t* type;     // BORA_FLUID / BORA_AIR / BORA_SOLID / BORA_MASKED
    uint16_t* code;    // stencil code (fine-code layout)
    __half* r;         // level residual (levels >= 1), stencil units
    __half* z0;        // correction (pre-smoothed, then final)
    __half* z1;        // correction after prolongation + one sweep
};

// The tiled levels' passes of a V-cycle (mg_passes.cu): level l (E = 8, 4 or 2) pre-smoothed
// and restricted into level l + 1's r (down), or prolonged from the coarser correction ec and
// post-smoothed (up: level 0 into the PCG's z with r.z -> slot_rz, the others into z1).
// scratch: an FP32 vector of level 0's size. Level 0's down passes first apply the PCG's
// residual update r -= alpha q, alpha = ring[slot_rz_in] / ring[slot_dq_in] (none when
// slot_rz_in < 0), and sum the updated r.r into slot_rr_out; slot_rr gives the scale.
int bora_mg_pass_grid( int E, int ntiles, int v );  // v < 0: level 0's fixed up-2 shape
void bora_mg_pass_down( const BoraLevelDev* levels, int l, const BoraTilesDev& t, int ntiles, float* r0, const float* q,
                        float* scratch, const BoraReduceDev& red, int slot_rr, int slot_rz_in, int slot_dq_in,
                        int slot_rr_out, cudaStream_t st );
void bora_mg_pass_up( const BoraLevelDev* levels, int l, const __half* ec, const BoraTilesDev& t, int ntiles,
                      const float* r0, float* scratch, const BoraReduceDev& red, int slot_rr, float* z, int slot_rz,
                      cudaStream_t st );

// ---- launch-shape autotuner (tune.cu) ------------------------------------------------------
// Kernel groups with interchangeable launch shapes (bit-identical results): the multigrid
// passes of levels 0, 1, 2, for single simulations and for batches.
enum BoraTuneGroup
{
    kBoraTuneL0 = 0, kBoraTuneL1, kBoraTuneL2, kBoraTuneL0Batch, kBoraTuneL1Batch, kBoraTuneL2Batch, kBoraTuneGroups
};
struct BoraTunePick
{
    int variant;  // the launch shape to use
    bool timed;   // still measuring: time this launch (BoraTuneTimer)
};
int bora_tune_variants( int group );
int bora_tune_default( int group );
BoraTunePick bora_tune_pick( int group, int units );  // units: the work's size (tiles)
// Brackets the launches of a pick with events on the stream while the group is measured.
struct BoraTuneTimer
{
    bool timed;
    int group, units, variant;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    BoraTuneTimer( const BoraTunePick& p, int group, int units, cudaStream_t st );
    ~BoraTuneTimer();
    BoraTuneTimer( const BoraTuneTimer& ) = delete;
    BoraTuneTimer& operator=( const BoraTuneTimer& ) = delete;
};
// Fold the timings of completed launches into the table (call after a stream synchronize).
void bora_tune_resolve();

// Cell types and stencil codes of level c from level c-1 (levels[0] = fine, given).
// mid_image: the buffer for the coarse levels' cluster image (bora_mg_mid_image_bytes), or null
void bora_mg_setup( const BoraGridDev& g, BoraLevelDev* levels, int nlevels, BoraTilesDev t, void* mid_image,
                    uint32_t* err, cudaStream_t st );
// One preconditioned PCG update: r -= alpha q (alpha = ring[slot_rz_in] / ring[slot_dq_in],
// none when slot_rz_in < 0), r.r -> slot_rr_out, then one V-cycle z = M^-1 r (FP32 in and out,
// FP16 inside, scaled by 1 / sqrt(ring[slot_scale])); r.z -> slot_rz (FP64-accurate).
// Kernel launches of one bora_mg_vcycle call for this hierarchy.
int bora_mg_vcycle_launches( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t,
                             const void* mid_image );
// Level 3 .. coarsest of a V-cycle in one thread-block cluster out of distributed shared
// memory (mg_mid.cu). bora_mg_mid_image_bytes: the device buffer its per-step static image
// needs, 0 when the hierarchy does not have the shape or size it handles;
// bora_mg_mid_setup: lay the image out (once per step, after bora_mg_setup's codes);
// bora_mg_mid_vcycle: 1 when it runs these levels (launching the kernel when `launch`), 0
// when the caller must run them itself.
size_t bora_mg_mid_image_bytes( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles );
void bora_mg_mid_setup( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles,
                        void* image, cudaStream_t st );
int bora_mg_mid_vcycle( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles,
                        const void* image, uint32_t* err, int sweeps, cudaStream_t st, bool launch );
void bora_mg_vcycle( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, const void* mid_image,
                     float* r, const float* q, float* z, float* scratch, BoraReduceDev red, int slot_rz_in,
                     int slot_dq_in, int slot_rr_out, int slot_scale, int slot_rz, int coarse_sweeps, cudaStream_t st );
// ---- batched solve: several simulations, one launch per kernel ---------------------------
// A batched launch packs the blocks of the simulations taking part back to back into one
// 1-D grid: simulation k owns blocks start[k] .. start[k+1] - 1, exactly the grid its own
// single-simulation launch of that kernel would use (grid[], fixed by its tile count alone),
// and no block when it sits the launch out. Each simulation reduces into its own ring, so
// its block indices, grid size, arithmetic and summation order are the same alone and in
// any batch, and no block of a batched launch idles. Arguments come from device arrays.
enum BoraMemberGrid
{
    kGridDir = 0, kGridUpd, kGridCells, kGridResidual,
    kGridPass0, kGridPass0R, kGridPass1, kGridPass2,  // the multigrid passes of levels 0, 1, 2 (mg_passes.cu);
                                                      // 0R: level 0's up 2, which reduces r.z
    kGridCount
};
struct BoraMemberSolve
{
    int ntiles;
    const int32_t* nbr;
    const uint16_t* code;
    const float* b;
    float* pres;
    BoraSolverDev sv;
    BoraReduceDev red;
    BoraLevelDev L[4];     // multigrid levels 0..3 (level 3: one cell per tile)
    const __half* z3;      // level 3's correction, written by the coarse cluster kernel
    int grid[kGridCount];  // this simulation's own grid per kernel
};
struct BoraMemberSlots  // ring slots of one batched launch sequence
{
    int active;                          // 0: this simulation sits the launch out
    int dsel;                            // which search-direction buffer is the current one
    int rz_new, rz_old, dq, a_rz, a_dq;  // direction (beta = rz_new / rz_old; pending alpha)
    int rz_in, dq_in, rr_out;            // update (alpha = rz_in / dq_in), r.r out
    int rr, rz;                          // V-cycle: the scale's r.r, r.z out
    int n2, mx;                          // solve init / refinement residual: ||r||^2, max|r|
};
struct BoraBatchLaunch
{
    const BoraMemberSolve* ms;
    const BoraMemberSlots* sl;
    const int* start;  // n + 1 block offsets of this launch (device memory)
    int n;
};
#ifdef __CUDACC__
// The simulation owning block b of a batched launch - the last k with start[k] <= b (the
// ones before it that own no block share its offset) - and the block's index in its grid.
__device__ __forceinline__ int bora_batch_member( const BoraBatchLaunch& L, unsigned b, unsigned* bid )
{
    int lo = 0, hi = L.n;
    while( hi - lo > 1 )
    {
        const int mid = ( lo + hi ) >> 1;
        if( (unsigned)__ldg( L.start + mid ) <= b ) lo = mid;
        else hi = mid;
    }
    *bid = b - (unsigned)__ldg( L.start + lo );
    return lo;
}
#endif

// The coarse cluster kernel of a batch: a simulation's descriptor (opaque, desc_bytes each;
// 0 when its hierarchy does not fit the kernel), and one launch of `blocks` CTAs: one
// cluster of `ctas` CTAs per simulation taking part (all of the same size; shared memory
// for the largest).
size_t bora_mg_mid_desc_bytes();
int bora_mg_mid_describe( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles,
                          const void* image, uint32_t* err, int sweeps, void* desc, size_t* smem, int* ctas );
void bora_mg_mid_launch_batch( const void* descs, const BoraBatchLaunch& L, int blocks, int ctas, size_t smem,
                               cudaStream_t st );
// Batched launches of the solver kernels (projection.cu, multigrid.cu) with `blocks` =
// start[n] blocks in all.
void bora_launch_solve_init_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st );
void bora_launch_pcg_direction_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st );
void bora_launch_refine_accumulate_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st );
void bora_launch_refine_residual_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st );
void bora_launch_write_pressure_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st );
void bora_launch_pcg_update_noprec_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st );
// pass `pass` (0, 1 down; 2, 3 up) of multigrid level l (0, 1, 2) for the batch, launch
// shape v (level 0's up 2 has a fixed shape)
void bora_launch_mg_pass_batch( int l, int pass, int v, const BoraBatchLaunch& L, int blocks, cudaStream_t st );
// this simulation's own grid per batched kernel (what its single launches use), with the
// multigrid passes of levels 0, 1, 2 in launch shapes v[0..2]
void bora_member_grids( int ntiles, int* grid, const int* v );
void bora_projection_grids( int ntiles, int* grid );  // the kGridDir, kGridCells and kGridResidual entries

// e += alpha d; r -= alpha q; r.r -> ring slot (alpha = rz / dq, or 0 when slot_rz < 0)
void bora_launch_pcg_update_noprec( int ntiles, BoraSolverDev s, BoraReduceDev red, int slot_rz, int slot_dq,
                                    int slot_rr_out, cudaStream_t st );
