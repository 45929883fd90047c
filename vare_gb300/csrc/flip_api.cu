// C ABI of the GB300 FLIP substep: the simulation handle, buffer management and the
// per-step orchestration of FLIPMethod::advanceOneStep (base/source/FLIPMethod.cu:208-298).
//
// One handle = one simulation on one device and one CUDA stream. Device buffers are
// grown geometrically and reused across steps; nothing is allocated inside a step
// unless the particle count or the active-tile count outgrows its capacity.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "bora_internal.h"
#include "../../include/bora_flip.h"

namespace {

struct DevBuf
{
    void* p = nullptr;
    size_t bytes = 0;
};

cudaError_t grow( DevBuf& b, size_t bytes, bool keep, cudaStream_t st )
{
    if( bytes <= b.bytes ) return cudaSuccess;
    size_t nb = std::max( bytes, b.bytes + b.bytes / 2 );
    nb = ( nb + 255 ) & ~(size_t)255;
    void* np = nullptr;
    cudaError_t e = cudaMalloc( &np, nb );
    if( e != cudaSuccess ) return e;
    if( keep && b.p && b.bytes ) e = cudaMemcpyAsync( np, b.p, b.bytes, cudaMemcpyDeviceToDevice, st );
    if( e == cudaSuccess && b.p ) { cudaStreamSynchronize( st ); cudaFree( b.p ); }
    b.p = np;
    b.bytes = nb;
    return e;
}

void release( DevBuf& b )
{
    if( b.p ) cudaFree( b.p );
    b.p = nullptr;
    b.bytes = 0;
}

template <class T> T* P( DevBuf& b ) { return reinterpret_cast<T*>( b.p ); }

// Compact live particles (id >= 0) into interleaved host-layout staging arrays.
__global__ void k_live_flags( size_t n, const int32_t* __restrict__ id, uint32_t* __restrict__ flag )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x )
        flag[i] = id[i] >= 0 ? 1u : 0u;
}

__global__ void k_gather_live( size_t n, BoraParticlesDev p, const float* __restrict__ adj, const uint32_t* __restrict__ excl,
                               int space, float3 tr, float3 sc, float* __restrict__ pos, float* __restrict__ vel,
                               float* __restrict__ adj_out, int32_t* __restrict__ ids )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x )
    {
        if( p.id[i] < 0 ) continue;
        const size_t o = excl[i];
        float x = p.px[i], y = p.py[i], z = p.pz[i], u = p.vx[i], v = p.vy[i], w = p.vz[i];
        if( space == BORA_SPACE_WORLD )
        {
            // Grid::worldPoint / worldVector (base/header/Grid.h:432-444)
            x = x * sc.x + tr.x; y = y * sc.y + tr.y; z = z * sc.z + tr.z;
            u = u * sc.x; v = v * sc.y; w = w * sc.z;
        }
        if( pos ) { pos[3 * o] = x; pos[3 * o + 1] = y; pos[3 * o + 2] = z; }
        if( vel ) { vel[3 * o] = u; vel[3 * o + 1] = v; vel[3 * o + 2] = w; }
        if( adj_out ) adj_out[o] = adj[i];
        if( ids ) ids[o] = p.id[i];
    }
}

// Particle vorticity / curvature of live particles, in the same order.
__global__ void k_gather_attrs( size_t n, BoraParticlesDev p, const uint32_t* __restrict__ excl, float* __restrict__ vort,
                                float* __restrict__ curv, int32_t* __restrict__ ids )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x )
    {
        if( p.id[i] < 0 ) continue;
        const size_t o = excl[i];
        vort[o] = p.vort ? p.vort[i] : 0.f;
        curv[o] = p.curv ? p.curv[i] : 0.f;
        ids[o] = p.id[i];
    }
}

__global__ void k_scatter_attrs( size_t n, BoraParticlesDev p, const uint32_t* __restrict__ excl,
                                 const float* __restrict__ vort, const float* __restrict__ curv )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x )
    {
        if( p.id[i] < 0 ) continue;
        p.vort[i] = vort[excl[i]];
        p.curv[i] = curv[excl[i]];
    }
}

__global__ void k_to_host_u32( const uint32_t* __restrict__ src, uint32_t* dst, int n )
{
    for( int i = threadIdx.x; i < n; i += blockDim.x ) ( (volatile uint32_t*)dst )[i] = src[i];
}

__global__ void k_to_host_f64( const double* __restrict__ src, double* dst, int n )
{
    for( int i = threadIdx.x; i < n; i += blockDim.x ) ( (volatile double*)dst )[i] = src[i];
}

int grid_blocks( size_t n )
{
    const size_t b = ( n + 255 ) / 256;
    return (int)std::max<size_t>( 1, std::min<size_t>( b, 152 * 16 ) );
}

}  // namespace

struct bora_flip_sim
{
    int device = 0;
    cudaStream_t st = nullptr;
    bora_grid_desc gdesc{};
    bora_flip_params prm{};
    BoraGridDev g{};
    float translate[3] = { 0, 0, 0 }, scale[3] = { 1, 1, 1 };
    size_t ntv = 0;

    // tiles
    DevBuf tile_flag, tile_act, tile_excl, slot_of, tile_of, nbr;
    DevBuf slot_prev;  // the tile table of the last solve's pressure (warm start)
    int ntiles = 0;
    size_t cap_tiles = 0;

    // cells
    DevBuf mass, surf, pres, vx, vy, vz, cx, cy, cz, flag, code, rhs;
    DevBuf sx, se, sr, sd0, sd1, sq, sz, sminv;
    DevBuf cell_count, cell_start;
    DevBuf col_phi, col_vel;  // collider signed distance / velocity per frame cell
    DevBuf col_tslot, col_tnear, col_tphi, col_tvel;  // sparse collider: tile table, samples

    // multigrid hierarchy (mixed solver): per level type, code, r, z0, z1
    static constexpr int kMaxLevels = 16;
    DevBuf mg_type[kMaxLevels], mg_code[kMaxLevels], mg_r[kMaxLevels], mg_z0[kMaxLevels], mg_z1[kMaxLevels];
    DevBuf vdb_leaf, vdb_mask, vdb_val;  // VDB leaf export: leaf origins + slots, masks, values
    DevBuf mg_mid;         // static image of the coarse levels' cluster kernel (mg_mid.cu), or empty
    bool mg_mid_on = false;
    bool batching = false; // inside bora_flip_step_batch: hierarchies keep every level shape the batch needs
    BoraLevelDev levels[kMaxLevels] = {};
    int nlevels = 0;

    // reductions
    DevBuf ring, partials, done;
    DevBuf gbar;     // the persistent solver's grid barrier: count, generation
    int fault = 0;   // BORA_FAULT_*
    int next_slot = 0;

    // particles
    DevBuf pbuf[2][7];  // px py pz vx vy vz id
    DevBuf pattr[2][2]; // vorticity, curvature (allocated by the first post-processing)
    bool attrs = false;
    DevBuf labels;      // post-processing: union-find labels of the water tank's scan
    // asynchronous export: live particles gathered into exp_buf on the handle's stream, copied
    // to the caller's host memory on a second stream while the next step runs
    DevBuf exp_buf;
    cudaStream_t st_copy = nullptr;
    cudaEvent_t ev_gathered = nullptr, ev_copied = nullptr;
    bool exporting = false;
    DevBuf adj, vkey, key, idx;
    size_t cap_p = 0;
    size_t np = 0;      // particles in the current buffer (killed ones included until the next sort)
    size_t nlive = 0;
    size_t nsorted = 0; // live particles indexed by idx after the last rebuild
    int cur = 0;
    int32_t next_id = 0;
    bool sorted = false;   // idx/cell_start describe the current buffer
    bool keys_valid = false;  // vkey and tile_flag bin the current buffer (written by the last G2P)
    bool pres_valid = false;  // pres holds the last solve's pressure over the current tiles
    bool warm_ready = false;  // slot_prev is the tile table of pres (warm start of the next solve)

    // scratch and staging
    DevBuf scan_scratch, counters, stage_in, stage_out, live_flag;
    uint32_t* h_cnt = nullptr;  // pinned, mapped: counters as the host sees them
    uint32_t* d_cnt = nullptr;  // its device address
    double* h_ring = nullptr;   // pinned, mapped
    double* d_hring = nullptr;  // its device address
    double* h_mirror = nullptr;  // pinned, mapped: reductions' slot values as the host sees them
    double* d_mirror = nullptr;  // its device address
    static constexpr int kChecks = 8;
    cudaEvent_t ev_chk[kChecks] = {};

    bora_flip_stats stats{};
    int last_status = BORA_OK;

    // device timing: per-step events (always) and opt-in per-kernel-class events
    cudaEvent_t ev_step[2] = { nullptr, nullptr };
    cudaEvent_t ev_join = nullptr;  // batched steps: joins this handle's stream with the batch's
    uint32_t prof_mask = 0;
    uint32_t prof_every = 1;                       // time one bracket in prof_every per class
    uint32_t prof_seen[BORA_KERNEL_CLASSES] = {};  // brackets of each class since the mask was set
    double kt_ms[BORA_KERNEL_CLASSES] = {};
    uint64_t kt_n[BORA_KERNEL_CLASSES] = {};
    struct Pending { int cls; cudaEvent_t a, b; };
    std::vector<cudaEvent_t> evpool;
    std::vector<Pending> pending;

    cudaEvent_t take_event()
    {
        if( !evpool.empty() ) { cudaEvent_t e = evpool.back(); evpool.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        cudaEventCreate( &e );
        return e;
    }
    // resolve recorded kernel timings; the stream must have been synchronized
    void prof_resolve()
    {
        for( const Pending& p : pending )
        {
            float ms = 0.f;
            if( cudaEventElapsedTime( &ms, p.a, p.b ) == cudaSuccess ) { kt_ms[p.cls] += ms; kt_n[p.cls] += 1; }
            evpool.push_back( p.a );
            evpool.push_back( p.b );
        }
        pending.clear();
    }

    BoraParticlesDev parts( int b )
    {
        return BoraParticlesDev{ P<float>( pbuf[b][0] ), P<float>( pbuf[b][1] ), P<float>( pbuf[b][2] ),
                                 P<float>( pbuf[b][3] ), P<float>( pbuf[b][4] ), P<float>( pbuf[b][5] ),
                                 P<int32_t>( pbuf[b][6] ), attrs ? P<float>( pattr[b][0] ) : nullptr,
                                 attrs ? P<float>( pattr[b][1] ) : nullptr };
    }
    BoraCellsDev cells()
    {
        return BoraCellsDev{ P<float>( mass ), P<float>( surf ), P<float>( pres ), P<float>( vx ), P<float>( vy ),
                             P<float>( vz ), P<float>( cx ), P<float>( cy ), P<float>( cz ), P<uint8_t>( flag ),
                             P<uint16_t>( code ), P<float>( rhs ) };
    }
    BoraTilesDev tiles() { return BoraTilesDev{ P<int32_t>( slot_of ), P<int32_t>( tile_of ), P<int32_t>( nbr ) }; }
    BoraSolverDev solver()
    {
        BoraSolverDev s;
        s.x = P<float2>( sx ); s.e = P<float>( se ); s.r = P<float>( sr );
        s.d[0] = P<float>( sd0 ); s.d[1] = P<float>( sd1 ); s.q = P<float>( sq ); s.z = P<float>( sz );
        s.minv = P<float>( sminv );
        return s;
    }
    BoraReduceDev reducer()
    {
        return BoraReduceDev{ P<double>( ring ), P<double>( partials ), P<uint32_t>( done ), P<uint32_t>( counters ) + 5,
                              d_mirror };
    }
    int slot()
    {
        const int s = next_slot;
        next_slot = ( next_slot + 1 ) % BORA_RING;
        return s;
    }
};

namespace {

int cuda_status( cudaError_t e )
{
    if( e == cudaSuccess ) return BORA_OK;
    if( e == cudaErrorMemoryAllocation ) return BORA_ERR_OUT_OF_MEMORY;
    return BORA_ERR_CUDA;
}

#define BORA_TRY( expr )                                        \
    do {                                                        \
        const cudaError_t _e = ( expr );                        \
        if( _e != cudaSuccess ) return cuda_status( _e );       \
    } while( 0 )

#define BORA_TRYS( expr )                                       \
    do {                                                        \
        const int _s = ( expr );                                \
        if( _s < 0 ) return _s;                                 \
    } while( 0 )

// Counts the kernels of one launcher call and, when its class is being profiled,
// brackets them with CUDA events on the handle's stream.
struct KTimer
{
    bora_flip_sim* s;
    int cls;
    cudaEvent_t a = nullptr;
    KTimer( bora_flip_sim* sim, int c, int nkernels ) : s( sim ), cls( c )
    {
        s->stats.kernel_launches += (uint64_t)nkernels;
        if( ( ( s->prof_mask >> cls ) & 1u ) && s->prof_seen[cls]++ % s->prof_every == 0 )
        {
            a = s->take_event();
            cudaEventRecord( a, s->st );
        }
    }
    ~KTimer()
    {
        if( a )
        {
            cudaEvent_t b = s->take_event();
            cudaEventRecord( b, s->st );
            s->pending.push_back( bora_flip_sim::Pending{ cls, a, b } );
        }
    }
};

int check_launch( bora_flip_sim* h )
{
    const cudaError_t e = cudaGetLastError();
    (void)h;
    return cuda_status( e );
}

// Frame set-up: SparseFrame::initialize (SparseFrame.cu:28-73) and FLIPMethod::initialize
// (FLIPMethod.cu:41-46) - pad each axis to a multiple of 4 cells, re-centre the box with a
// uniform spacing h = min(dx,dy,dz), convert gravity and the wall level to voxel units.
void setup_frame( bora_flip_sim* s )
{
    const bora_grid_desc& d = s->gdesc;
    const int gn[3] = { d.nx, d.ny, d.nz };
    float gT[3], gS[3], minP[3], maxP[3], cen[3], dd[3];
    for( int a = 0; a < 3; ++a )
    {
        gT[a] = d.min[a];
        gS[a] = ( d.max[a] - d.min[a] ) / (float)gn[a];
    }
    int fn[3];
    for( int a = 0; a < 3; ++a ) fn[a] = ( gn[a] / 4 + ( ( gn[a] % 4 ) ? 1 : 0 ) ) * 4;
    for( int a = 0; a < 3; ++a )
    {
        const float e = gT[a] + (float)gn[a] * gS[a];
        minP[a] = std::min( gT[a], e );
        maxP[a] = std::max( gT[a], e );
        cen[a] = ( minP[a] + maxP[a] ) * 0.5f;
        dd[a] = ( maxP[a] - minP[a] ) / (float)gn[a];
    }
    const float h = std::min( std::min( dd[0], dd[1] ), dd[2] );
    for( int a = 0; a < 3; ++a )
    {
        const float L = (float)fn[a] * h;
        const float nmin = cen[a] - L * 0.5f;
        const float nmax = nmin + L;
        s->translate[a] = nmin;
        s->scale[a] = ( nmax - nmin ) / (float)fn[a];
    }
    BoraGridDev& g = s->g;
    g.nx = fn[0]; g.ny = fn[1]; g.nz = fn[2];
    g.tx = ( g.nx + 7 ) / 8; g.ty = ( g.ny + 7 ) / 8; g.tz = ( g.nz + 7 ) / 8;
    s->ntv = (size_t)g.tx * g.ty * g.tz;
}

void apply_params( bora_flip_sim* s )
{
    BoraGridDev& g = s->g;
    const bora_flip_params& p = s->prm;
    for( int a = 0; a < 3; ++a ) g.gravity[a] = p.ext_force[a] / s->scale[a];
    g.voxel_wall = ( p.wall_level - s->translate[1] ) / s->scale[1];
    g.col_vel_scale = p.col_vel_scale;
    g.maxsubsteps = p.max_substeps;
    g.enable_tank = p.enable_water_tank;
    g.damping_band = p.damping_band / p.voxel_size;
    g.advection = p.advection;
}

int ensure_particles( bora_flip_sim* s, size_t n )
{
    if( n <= s->cap_p ) return BORA_OK;
    const size_t cap = std::max( n, s->cap_p + s->cap_p / 2 );
    for( int b = 0; b < 2; ++b )
        for( int a = 0; a < 7; ++a ) BORA_TRY( grow( s->pbuf[b][a], cap * 4, b == s->cur, s->st ) );
    if( s->attrs )
        for( int b = 0; b < 2; ++b )
            for( int a = 0; a < 2; ++a ) BORA_TRY( grow( s->pattr[b][a], cap * 4, b == s->cur, s->st ) );
    BORA_TRY( grow( s->adj, cap * 4, true, s->st ) );
    BORA_TRY( grow( s->vkey, cap * 4, false, s->st ) );
    BORA_TRY( grow( s->key, cap * 4, false, s->st ) );
    BORA_TRY( grow( s->idx, cap * 4, false, s->st ) );
    BORA_TRY( grow( s->live_flag, ( cap + 1 ) * 4, false, s->st ) );
    s->cap_p = cap;
    return BORA_OK;
}

int ensure_scan_scratch( bora_flip_sim* s, size_t n )
{
    BORA_TRY( grow( s->scan_scratch, bora_scan_scratch_elems( n ) * 4 + 16, false, s->st ) );
    return BORA_OK;
}

int ensure_cells( bora_flip_sim* s, int ntiles )
{
    if( (size_t)ntiles <= s->cap_tiles && s->cap_tiles ) return BORA_OK;
    s->warm_ready = false;  // the cell fields are re-allocated: the last pressure is gone
    const size_t cap = std::max<size_t>( (size_t)ntiles, s->cap_tiles + s->cap_tiles / 2 );
    const size_t nc = cap * BORA_TILE_CELLS;
    DevBuf* f4[] = { &s->mass, &s->surf, &s->pres, &s->vx, &s->vy, &s->vz, &s->cx, &s->cy, &s->cz, &s->rhs,
                     &s->se, &s->sr, &s->sd0, &s->sd1, &s->sq, &s->sz, &s->sminv };
    for( DevBuf* b : f4 ) BORA_TRY( grow( *b, nc * 4, false, s->st ) );
    BORA_TRY( grow( s->flag, nc, false, s->st ) );
    BORA_TRY( grow( s->code, nc * 2, false, s->st ) );
    BORA_TRY( grow( s->sx, nc * 8, false, s->st ) );
    const size_t oldc = s->cell_count.bytes;
    BORA_TRY( grow( s->cell_count, ( nc + 2 ) * 4, true, s->st ) );
    if( s->cell_count.bytes > oldc )
        BORA_TRY( cudaMemsetAsync( (char*)s->cell_count.p + oldc, 0, s->cell_count.bytes - oldc, s->st ) );
    BORA_TRY( grow( s->cell_start, ( nc + 2 ) * 4, false, s->st ) );
    BORA_TRY( grow( s->tile_of, cap * 4, false, s->st ) );
    BORA_TRY( grow( s->nbr, cap * 27 * 4, false, s->st ) );
    // two values per block for the reductions; three for the persistent solver's
    BORA_TRY( grow( s->partials, ( std::max<size_t>( cap, kBoraMaxReduceBlocks ) + 16 ) * 3 * 8, false, s->st ) );
    BORA_TRYS( ensure_scan_scratch( s, std::max( nc + 2, s->ntv ) ) );
    s->cap_tiles = cap;
    return BORA_OK;
}

// Scalars the host reads back are written into mapped host memory by a one-warp kernel
// rather than copied: a copy would queue behind a large export on the copy engines
// (bora_flip_export_begin) and stall the step it should overlap.
int issue_counters( bora_flip_sim* s, int first, int count, cudaStream_t st )
{
    s->stats.kernel_launches += 1;
    k_to_host_u32<<<1, 32, 0, st>>>( P<uint32_t>( s->counters ) + first, s->d_cnt + first, count );
    return cuda_status( cudaGetLastError() );
}

int read_counters( bora_flip_sim* s, int first, int count )
{
    BORA_TRYS( issue_counters( s, first, count, s->st ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    return BORA_OK;
}

double read_ring( bora_flip_sim* s, int slot, int* status )
{
    s->stats.kernel_launches += 1;
    k_to_host_f64<<<1, 32, 0, s->st>>>( P<double>( s->ring ) + slot, s->d_hring, 1 );
    cudaError_t e = cudaGetLastError();
    if( e == cudaSuccess ) e = cudaStreamSynchronize( s->st );
    if( e != cudaSuccess ) { *status = cuda_status( e ); return 0.0; }
    return ( (volatile double*)s->h_ring )[0];
}

// ---- stages --------------------------------------------------------------------------

// SparseFrame::buildFromPoints (SparseFrame.cu:83-155): bin, activate, number the active
// tiles, then counting-sort the particles by dual cell. Three parts around the two host
// reads (the tile count, then the sort's totals), so that a batched step can issue each part
// for all of its simulations before it waits.
int rebuild_tiles( bora_flip_sim* s )
{
    cudaStream_t st = s->st;
    BORA_TRY( cudaMemsetAsync( s->counters.p, 0, 8 * 4, st ) );
    // the warm start reads the last pressure through the tile table it was solved on
    s->warm_ready = false;
    if( s->prm.warm_start && s->pres_valid )
    {
        BORA_TRY( cudaMemcpyAsync( s->slot_prev.p, s->slot_of.p, s->ntv * 4, cudaMemcpyDeviceToDevice, st ) );
        s->warm_ready = true;
    }
    s->pres_valid = false;
    // the last G2P binned the particles it wrote, unless they have changed since
    if( !s->keys_valid )
    {
        BORA_TRY( cudaMemsetAsync( s->tile_flag.p, 0, s->ntv, st ) );
        if( s->np ) { KTimer t( s, BORA_KERNEL_BIN, 1 ); bora_launch_bin( s->g, s->parts( s->cur ), s->np, P<uint32_t>( s->vkey ), P<uint8_t>( s->tile_flag ), st ); }
    }
    s->keys_valid = false;
    {
        KTimer t( s, BORA_KERNEL_TILES, 4 );
        bora_launch_activate( s->g, P<uint8_t>( s->tile_flag ), P<uint32_t>( s->tile_act ), st );
        bora_device_scan( P<uint32_t>( s->tile_act ), P<uint32_t>( s->tile_excl ), s->ntv, P<uint32_t>( s->scan_scratch ),
                       P<uint32_t>( s->counters ) + 0, st );
    }
    BORA_TRYS( check_launch( s ) );
    return issue_counters( s, 0, 1, st );
}

// after rebuild_tiles' tile count has reached the host
int rebuild_sort( bora_flip_sim* s )
{
    cudaStream_t st = s->st;
    const int ntiles = (int)s->h_cnt[0];
    BORA_TRYS( ensure_cells( s, std::max( ntiles, 1 ) ) );
    s->ntiles = ntiles;
    const uint32_t ncell = (uint32_t)ntiles * BORA_TILE_CELLS;
    {
        KTimer t( s, BORA_KERNEL_TILES, ntiles > 0 ? 2 : 1 );
        bora_launch_tile_assign( s->g, P<uint32_t>( s->tile_act ), P<uint32_t>( s->tile_excl ), P<int32_t>( s->slot_of ),
                                 P<int32_t>( s->tile_of ), st );
        bora_launch_tile_nbrs( s->g, ntiles, P<int32_t>( s->slot_of ), P<int32_t>( s->tile_of ), P<int32_t>( s->nbr ), st );
    }
    {
        KTimer t( s, BORA_KERNEL_SORT, s->np ? 6 : 3 );
        bora_launch_hist( s->np, P<uint32_t>( s->vkey ), P<int32_t>( s->slot_of ), ncell, P<uint32_t>( s->key ),
                          P<uint32_t>( s->cell_count ), P<uint32_t>( s->counters ) + 2, st );
        bora_device_scan( P<uint32_t>( s->cell_count ), P<uint32_t>( s->cell_start ), (size_t)ncell + 1,
                       P<uint32_t>( s->scan_scratch ), P<uint32_t>( s->counters ) + 1, st );
        bora_launch_scatter( s->np, P<uint32_t>( s->key ), P<uint32_t>( s->cell_start ), P<uint32_t>( s->cell_count ),
                             P<uint32_t>( s->idx ), st );
        if( s->np ) bora_launch_order_bins( (size_t)ncell + 1, P<uint32_t>( s->cell_start ), P<uint32_t>( s->idx ), st );
    }
    BORA_TRYS( check_launch( s ) );
    return issue_counters( s, 1, 2, st );
}

// after rebuild_sort's totals have reached the host
int rebuild_finish( bora_flip_sim* s )
{
    if( s->h_cnt[2] != 0 ) return BORA_ERR_INTERNAL;
    s->nsorted = s->h_cnt[1];  // live particles, addressed through idx in dual-cell order
    s->sorted = true;
    s->stats.active_tiles = s->ntiles;
    return BORA_OK;
}

int stage_rebuild( bora_flip_sim* s )
{
    BORA_TRYS( rebuild_tiles( s ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    BORA_TRYS( rebuild_sort( s ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    return rebuild_finish( s );
}

int stage_p2g( bora_flip_sim* s )
{
    if( !s->sorted ) return BORA_ERR_INVALID_ARG;
    KTimer t( s, BORA_KERNEL_P2G, s->ntiles > 0 );
    bora_launch_p2g( s->g, s->ntiles, s->tiles(), s->parts( s->cur ), P<uint32_t>( s->idx ), P<uint32_t>( s->cell_start ),
                     s->cells(), s->st );
    return check_launch( s );
}

// Multigrid hierarchy for the current tiles: levels 0..3 tiled (8^3, 4^3, 2^3, 1 cell per
// tile), then dense grids halved per level until a level has at most 512 cells.
int build_hierarchy( bora_flip_sim* s )
{
    const BoraGridDev& g = s->g;
    const size_t nt = (size_t)s->ntiles;
    int n = 0;
    int ex = g.nx, ey = g.ny, ez = g.nz;
    auto add = [&]( int kind, int E, size_t ncells, int dx, int dy, int dz ) -> int {
        if( n >= bora_flip_sim::kMaxLevels ) return BORA_ERR_INTERNAL;
        BoraLevelDev& L = s->levels[n];
        L.kind = kind; L.E = E; L.level = n;
        L.nx = ex; L.ny = ey; L.nz = ez;
        L.dx = dx; L.dy = dy; L.dz = dz;
        L.ncells = ncells;
        if( n == 0 )
        {
            L.type = P<uint8_t>( s->flag );
            L.code = P<uint16_t>( s->code );
            L.r = nullptr;
        }
        else
        {
            BORA_TRY( grow( s->mg_type[n], ncells + 16, false, s->st ) );
            BORA_TRY( grow( s->mg_code[n], ncells * 2 + 16, false, s->st ) );
            BORA_TRY( grow( s->mg_r[n], ncells * 2 + 16, false, s->st ) );
            L.type = P<uint8_t>( s->mg_type[n] );
            L.code = P<uint16_t>( s->mg_code[n] );
            L.r = P<__half>( s->mg_r[n] );
        }
        BORA_TRY( grow( s->mg_z0[n], ncells * 2 + 16, false, s->st ) );
        BORA_TRY( grow( s->mg_z1[n], ncells * 2 + 16, false, s->st ) );
        L.z0 = P<__half>( s->mg_z0[n] );
        L.z1 = P<__half>( s->mg_z1[n] );
        ++n;
        return BORA_OK;
    };
    auto half_up = []( int v ) { return ( v + 1 ) / 2; };
    s->mg_mid_on = false;
    BORA_TRYS( add( 0, 8, nt * 512, 0, 0, 0 ) );
    for( int E = 4; E >= 1; E /= 2 )
    {
        ex = half_up( ex ); ey = half_up( ey ); ez = half_up( ez );
        BORA_TRYS( add( 0, E, nt * (size_t)E * E * E, 0, 0, 0 ) );
        // a batched step keeps the tiled levels 0-3 and at least one dense level below them
        // (the shape of its launches), whatever the size
        if( !s->batching && s->levels[n - 1].ncells <= 512 ) { s->nlevels = n; return BORA_OK; }
    }
    // level 3 has one cell per tile; its extent is the tile grid
    while( true )
    {
        ex = half_up( ex ); ey = half_up( ey ); ez = half_up( ez );
        BORA_TRYS( add( 1, 0, (size_t)ex * ey * ez, ex, ey, ez ) );
        if( s->levels[n - 1].ncells <= 512 ) break;
    }
    s->nlevels = n;
    // the coarse levels run in one cluster kernel when they fit it; its static image
    const size_t img = bora_mg_mid_image_bytes( g, s->levels, n, s->tiles(), (int)nt );
    if( img > 0 )
    {
        BORA_TRY( grow( s->mg_mid, img, false, s->st ) );
        s->mg_mid_on = true;
    }
    return BORA_OK;
}

int stage_build_system( bora_flip_sim* s )
{
    KTimer t( s, BORA_KERNEL_RHS, s->ntiles > 0 ? 1 : 0 );
    BORA_TRY( cudaMemsetAsync( P<uint32_t>( s->counters ) + 6, 0, 4, s->st ) );
    bora_launch_rhs( s->g, s->ntiles, s->tiles(), s->cells(), P<uint32_t>( s->counters ) + 6, s->st );
    if( s->ntiles <= 0 ) return check_launch( s );
    if( s->prm.solver == BORA_SOLVER_MIXED )
    {
        BORA_TRYS( build_hierarchy( s ) );
        s->stats.kernel_launches += 2 * (uint64_t)( s->nlevels - 1 ) + ( s->mg_mid_on ? 1 : 0 );
        bora_mg_setup( s->g, s->levels, s->nlevels, s->tiles(), s->mg_mid_on ? s->mg_mid.p : nullptr,
                       P<uint32_t>( s->counters ) + 5, s->st );
    }
    else
    {
        s->stats.kernel_launches += 1;
        bora_launch_mic_factor( s->g, s->ntiles, P<uint16_t>( s->code ), P<float>( s->sminv ), s->st );
    }
    return check_launch( s );
}

// Pressure solve: double-float iterative refinement around FP32 PCG passes.
int stage_solve( bora_flip_sim* s )
{
    const bora_flip_params& p = s->prm;
    BoraSolverDev sv = s->solver();
    BoraReduceDev red = s->reducer();
    const uint16_t* code = P<uint16_t>( s->code );
    const float* b = P<float>( s->rhs );
    cudaStream_t st = s->st;
    int status = BORA_OK;
    const double dx = s->scale[0];

    BORA_TRY( cudaMemsetAsync( P<uint32_t>( s->counters ) + 5, 0, 4, st ) );
    const int s_b2 = s->slot(), s_bmax = s->slot();
    { KTimer t( s, BORA_KERNEL_REFINE, 1 ); bora_launch_solve_init( s->ntiles, b, code, sv, red, s_b2, s_bmax, st ); }
    BORA_TRYS( check_launch( s ) );
    const double bnorm = std::sqrt( read_ring( s, s_b2, &status ) );
    BORA_TRYS( status );
    double rnorm = bnorm, rmax = read_ring( s, s_bmax, &status );
    BORA_TRYS( status );
    int total_it = 0, passes = 0;
    bool converged = false;
    const int max_inner = std::max( 1, p.proj_iteration );
    const int check = std::max( 1, p.check_every );
    // The Krylov recurrence continues across refinement passes (residual replacement): a
    // pass ends by replacing the recursive FP32 residual with the refined one, keeps the last
    // direction d and r.z, and the next pass carries on from them instead of restarting.
    int rz_prev = -1, dsel = 0;
    int scale_slot = s_b2;  // the latest residual norm the host has: ||b|| (r = b), then each refinement's
    if( s->warm_ready )
    {
        // warm start: x = the last step's pressure, r = b - A x; kept only if closer than x = 0
        s->warm_ready = false;
        const int w_n2 = s->slot(), w_mx = s->slot();
        {
            KTimer t( s, BORA_KERNEL_REFINE, 2 );
            bora_launch_solve_warm( s->ntiles, code, P<int32_t>( s->tile_of ), P<int32_t>( s->slot_prev ),
                                    P<float>( s->pres ), sv, st );
            bora_launch_refine_residual( s->g, s->ntiles, s->tiles(), b, code, sv, red, w_n2, w_mx, st );
        }
        BORA_TRYS( check_launch( s ) );
        const double wnorm = std::sqrt( read_ring( s, w_n2, &status ) );
        BORA_TRYS( status );
        const double wmax = read_ring( s, w_mx, &status );
        BORA_TRYS( status );
        if( wnorm < rnorm )
        {
            rnorm = wnorm;
            rmax = wmax;
            scale_slot = w_n2;
        }
        else
        {
            const int c_b2 = s->slot(), c_bmax = s->slot();  // back to x = 0, r = b
            { KTimer t( s, BORA_KERNEL_REFINE, 1 ); bora_launch_solve_init( s->ntiles, b, code, sv, red, c_b2, c_bmax, st ); }
            BORA_TRYS( check_launch( s ) );
            scale_slot = c_b2;
        }
    }
    for( ;; )
    {
        const bool norm_ok = rnorm <= p.tolerance * bnorm;
        const bool max_ok = rmax * dx <= p.div_tolerance;
        if( bnorm == 0.0 || ( norm_ok && max_ok ) ) { converged = true; break; }
        if( passes >= std::max( 1, p.max_refinements ) ) break;
        // inner FP32 PCG on A e = r
        const double target = norm_ok ? 0.1 * rnorm : std::max( p.inner_tolerance * rnorm, 0.25 * p.tolerance * bnorm );
        const bool mixed = p.solver == BORA_SOLVER_MIXED;
        const void* mid_img = s->mg_mid_on ? s->mg_mid.p : nullptr;
        const int vlaunch = mixed ? bora_mg_vcycle_launches( s->g, s->levels, s->nlevels, s->tiles(), mid_img ) : 0;
        s->stats.mg_vcycle_launches = mixed ? vlaunch : 0;
        // the mixed form's update r -= alpha q (alpha = rz_in / dq_in) and r.r run inside the
        // V-cycle's first passes, which scale the FP16 levels by the last known residual norm
        auto precondition = [&]( int rz_in, int dq_in, int rr_out, int scale, int rz_out ) {
            KTimer t( s, BORA_KERNEL_MG, vlaunch );
            bora_mg_vcycle( s->g, s->levels, s->nlevels, s->tiles(), mid_img, sv.r, sv.q, sv.z, sv.minv, red, rz_in, dq_in,
                            rr_out, scale, rz_out, 16, st );
        };
        int rz_cur = s->slot(), rr_cur = s->slot();
        int it = 0;
        int a_rz = -1, a_dq = -1;  // alpha of the last update, whose e += alpha d is still pending
        if( !mixed && p.persistent && bora_pcg_persistent_grid() > 0 )
        {
            // the whole pass in one cooperative launch (convergence checked on the device)
            const int s_a_rz = s->slot(), s_a_dq = s->slot();
            BORA_TRY( cudaMemsetAsync( P<uint32_t>( s->counters ) + 8, 0, 4, st ) );
            {
                KTimer t( s, BORA_KERNEL_PCG_UPDATE, 1 );
                if( bora_launch_pcg_persistent( s->ntiles, P<int32_t>( s->nbr ), code, sv, red, dsel, rz_prev, max_inner, target,
                                                s_a_rz, s_a_dq, rr_cur, P<uint32_t>( s->counters ) + 8,
                                                P<unsigned>( s->gbar ), P<double>( s->partials ),
                                                s->fault == BORA_FAULT_BARRIER, st ) != 0 )
                    return BORA_ERR_CUDA;
            }
            BORA_TRYS( check_launch( s ) );
            BORA_TRYS( read_counters( s, 5, 4 ) );
            if( s->h_cnt[5] & BORA_REDUCE_ERR_BARRIER ) return BORA_ERR_INTERNAL;
            it = (int)s->h_cnt[8];
            dsel ^= it & 1;
            a_rz = s_a_rz;
            a_dq = s_a_dq;
            rz_prev = s_a_rz;
        }
        else if( mixed )
        {
            precondition( -1, -1, rr_cur, scale_slot, rz_cur );
        }
        else
        {
            KTimer t( s, BORA_KERNEL_PCG_UPDATE, 1 );
            bora_launch_pcg_update( s->ntiles, code, sv, red, -1, -1, rz_cur, rr_cur, st );
        }
        // Convergence checks do not stall the device: the reductions also write their
        // results to mapped host memory, an event marks the end of iteration i, and the
        // host waits for it only once iteration i + 1 is queued (a converged solve runs one
        // extra iteration, which only lowers the residual further).
        struct Check { int it, q, slot; };
        Check pend[bora_flip_sim::kChecks];
        int npend = 0, nchk = 0;
        bool done = a_rz >= 0;  // the persistent pass has run
        while( it < max_inner && !done )
        {
            const int s_dq = s->slot();
            {
                KTimer t( s, BORA_KERNEL_PCG_DIRECTION, 1 );
                bora_launch_pcg_direction( s->g, s->ntiles, s->tiles(), code, sv, dsel, red, rz_cur, rz_prev, s_dq, a_rz, a_dq, st );
            }
            dsel ^= 1;
            const int rz_new = s->slot(), rr_new = s->slot();
            if( mixed )
            {
                precondition( rz_cur, s_dq, rr_new, rr_cur, rz_new );
            }
            else
            {
                KTimer t( s, BORA_KERNEL_PCG_UPDATE, 1 );
                bora_launch_pcg_update( s->ntiles, code, sv, red, rz_cur, s_dq, rz_new, rr_new, st );
            }
            a_rz = rz_cur;
            a_dq = s_dq;
            rz_prev = rz_cur;
            rz_cur = rz_new;
            rr_cur = rr_new;
            ++it;
            if( it % check == 0 )
            {
                BORA_TRYS( check_launch( s ) );
                const int q = nchk++ % bora_flip_sim::kChecks;
                BORA_TRY( cudaEventRecord( s->ev_chk[q], st ) );
                pend[npend++] = Check{ it, q, rr_cur };
            }
            while( npend > 0 && ( it - pend[0].it >= 1 || npend == bora_flip_sim::kChecks || it >= max_inner ) )
            {
                BORA_TRY( cudaEventSynchronize( s->ev_chk[pend[0].q] ) );
                const double rr = ( (volatile double*)s->h_mirror )[pend[0].slot];
                for( int k = 1; k < npend; ++k ) pend[k - 1] = pend[k];
                --npend;
                if( !( rr > 0.0 ) || std::sqrt( rr ) <= target ) { done = true; break; }
            }
        }
        total_it += it;
        ++passes;
        const int s_n2 = s->slot(), s_mx = s->slot();
        {
            KTimer t( s, BORA_KERNEL_REFINE, 2 );
            bora_launch_refine_accumulate( s->ntiles, code, sv, dsel, P<double>( s->ring ), a_rz, a_dq, st );
            bora_launch_refine_residual( s->g, s->ntiles, s->tiles(), b, code, sv, red, s_n2, s_mx, st );
        }
        BORA_TRYS( check_launch( s ) );
        rnorm = std::sqrt( read_ring( s, s_n2, &status ) );
        scale_slot = s_n2;
        BORA_TRYS( status );
        rmax = read_ring( s, s_mx, &status );
        BORA_TRYS( status );
        if( !std::isfinite( rnorm ) ) break;
        // Continue the recurrence only while the refined residual still agrees with the
        // recursive one (the device finished the pass, so its last r.r is in mapped memory);
        // a larger drift would break conjugacy, so the next pass restarts (beta = 0).
        const double rr_rec = ( (volatile double*)s->h_mirror )[rr_cur];
        const double rec = rr_rec > 0.0 ? std::sqrt( rr_rec ) : 0.0;
        if( !( rec > 0.0 ) || rnorm > 1.5 * rec ) rz_prev = -1;
    }
    { KTimer t( s, BORA_KERNEL_REFINE, 1 ); bora_launch_write_pressure( s->ntiles, code, sv.x, P<float>( s->pres ), st ); }
    BORA_TRYS( check_launch( s ) );
    BORA_TRYS( read_counters( s, 5, 2 ) );
    if( s->h_cnt[5] != 0 ) return BORA_ERR_INTERNAL;
    s->stats.fluid_cells = (int32_t)s->h_cnt[6];
    s->stats.solver_iterations = total_it;
    s->stats.refinements = passes;
    s->stats.residual_rel = bnorm > 0.0 ? rnorm / bnorm : 0.0;
    s->stats.residual_max = rmax;
    s->stats.residual_max_dx = rmax * dx;
    s->stats.converged = converged ? 1 : 0;
    return converged ? BORA_OK : BORA_WARN_NOT_CONVERGED;
}

int stage_update_velocity( bora_flip_sim* s )
{
    KTimer t( s, BORA_KERNEL_VELOCITY, s->ntiles > 0 );
    bora_launch_vel_update( s->g, s->ntiles, s->tiles(), s->cells(), s->st );
    const int st = check_launch( s );
    s->pres_valid = st == BORA_OK;  // the solve's pressure (and the air cells' means) over the current tiles
    return st;
}

// G2P, advection and kills (FLIPMethod.cu:54-175) into the other particle buffer; the kill
// count goes to the host. Two parts around the host read, as the rebuild.
int g2p_issue( bora_flip_sim* s, float dt )
{
    if( !s->sorted ) return BORA_ERR_INVALID_ARG;
    cudaStream_t st = s->st;
    BORA_TRY( cudaMemsetAsync( P<uint32_t>( s->counters ) + 3, 0, 4, st ) );
    BORA_TRY( cudaMemsetAsync( s->tile_flag.p, 0, s->ntv, st ) );  // G2P bins what it writes for the next rebuild
    const int nxt = s->cur ^ 1;
    {
        KTimer t( s, BORA_KERNEL_G2P, s->nsorted > 0 );
        bora_launch_g2p( s->g, s->ntiles, s->nsorted, s->tiles(), P<uint32_t>( s->cell_start ), s->cells(), s->parts( s->cur ),
                         P<uint32_t>( s->idx ), s->parts( nxt ), P<float>( s->adj ), dt, P<uint32_t>( s->counters ) + 3,
                         P<uint32_t>( s->vkey ), P<uint8_t>( s->tile_flag ), st );
    }
    BORA_TRYS( check_launch( s ) );
    return issue_counters( s, 3, 1, st );
}

int g2p_finish( bora_flip_sim* s )
{
    s->cur ^= 1;
    s->np = s->nsorted;
    s->sorted = false;
    s->keys_valid = true;
    s->stats.killed_last_step = s->h_cnt[3];
    s->nlive = s->np - s->h_cnt[3];
    s->stats.num_particles = s->nlive;
    return BORA_OK;
}

int stage_update_particles( bora_flip_sim* s, float dt )
{
    BORA_TRYS( g2p_issue( s, dt ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    return g2p_finish( s );
}

// ---- post-processing (FLIPMethod::postProcess, FLIPMethod.cu:300-405) --------------------

// Particle vorticity and curvature start at 0 for every particle (FLIPMethod.h:94-96);
// from the first post-processing on they are kept in both particle buffers.
int ensure_attrs( bora_flip_sim* s )
{
    if( s->attrs ) return BORA_OK;
    for( int b = 0; b < 2; ++b )
        for( int a = 0; a < 2; ++a ) BORA_TRY( grow( s->pattr[b][a], std::max<size_t>( s->cap_p, 1 ) * 4, false, s->st ) );
    for( int a = 0; a < 2; ++a )
        if( s->np ) BORA_TRY( cudaMemsetAsync( s->pattr[s->cur][a].p, 0, s->np * 4, s->st ) );
    s->attrs = true;
    return BORA_OK;
}

// Rasterization::ParticlesToSurfaceAndVelocity (Rasterization.cu:311-398).
int post_splat( bora_flip_sim* s )
{
    if( !s->sorted ) return BORA_ERR_INVALID_ARG;
    cudaStream_t st = s->st;
    if( s->ntiles <= 0 ) return BORA_OK;
    KTimer t( s, BORA_KERNEL_POST, 1 );
    bora_launch_splat( s->g, s->ntiles, s->tiles(), P<uint32_t>( s->cell_start ), P<uint32_t>( s->idx ), s->parts( s->cur ),
                       s->cells(), st );
    return check_launch( s );
}

// The water tank's fill of enclosed air pockets (FLIPMethod.cu:322-366).
int post_tank_scan( bora_flip_sim* s )
{
    if( !s->prm.enable_water_tank || s->ntiles <= 0 || !( s->g.voxel_wall >= 0.f ) ) return BORA_OK;
    const size_t nn = (size_t)s->ntiles * BORA_TILE_CELLS + s->ntv;
    if( nn >= ( (size_t)1 << 31 ) ) return BORA_ERR_CAPACITY;
    BORA_TRY( grow( s->labels, nn * 4, false, s->st ) );
    BORA_TRY( cudaMemsetAsync( P<uint32_t>( s->counters ) + 8, 0, 4, s->st ) );
    {
        KTimer t( s, BORA_KERNEL_POST, 6 );
        bora_tank_scan_launches( s->g, s->ntiles, s->tiles(), P<float>( s->surf ), P<uint32_t>( s->labels ),
                                 P<uint32_t>( s->counters ) + 8, s->st );
    }
    BORA_TRYS( check_launch( s ) );
    BORA_TRYS( read_counters( s, 8, 1 ) );
    return s->h_cnt[8] ? BORA_ERR_INTERNAL : BORA_OK;
}

// Rasterization::ReinitializeSurface (Rasterization.cu:400-486): surf and pres swap
// storage after every step, as the reference swaps the fields' pointers.
int post_redistance( bora_flip_sim* s )
{
    if( s->ntiles <= 0 ) return BORA_OK;
    const int iters = std::max( 0, s->prm.redist_iteration );
    KTimer t( s, BORA_KERNEL_POST, iters );
    for( int it = 0; it < iters; ++it )
    {
        BORA_TRY( bora_launch_redistance( s->g, s->ntiles, s->tiles(), P<float>( s->surf ), P<float>( s->pres ), s->st ) );
        std::swap( s->surf, s->pres );
    }
    return check_launch( s );
}

// FLIPMethod.cu:370-404: curl, normals and curvature, the particles' vorticity and
// curvature, then pres cleared.
int post_attributes( bora_flip_sim* s )
{
    BORA_TRYS( ensure_attrs( s ) );
    cudaStream_t st = s->st;
    const size_t nc = (size_t)s->ntiles * BORA_TILE_CELLS;
    float* wx = P<float>( s->sd0 );
    float* wy = P<float>( s->sd1 );
    float* wz = P<float>( s->sq );
    // FLIPMethod.cu:376, on the host as the reference computes it
    const float dis = powf( 1.f - s->prm.vort_pres_rate, s->prm.dt );
    {
        KTimer t( s, BORA_KERNEL_POST, ( s->ntiles > 0 ? 2 : 0 ) + ( s->np > 0 ? 1 : 0 ) );
        bora_launch_surface_fields( s->g, s->ntiles, s->tiles(), s->cells(), wx, wy, wz, st );
        if( s->ntiles > 0 )
            bora_launch_particle_attributes( s->g, P<int32_t>( s->slot_of ), s->np, s->parts( s->cur ), wx, wy, wz,
                                             P<float>( s->pres ), make_float3( s->scale[0], s->scale[1], s->scale[2] ),
                                             dis, st );
    }
    if( nc ) BORA_TRY( cudaMemsetAsync( s->pres.p, 0, nc * 4, st ) );
    return check_launch( s );
}

int post_process( bora_flip_sim* s )
{
    BORA_TRYS( stage_rebuild( s ) );  // FLIPMethod::prepareNextStep
    BORA_TRYS( post_splat( s ) );
    BORA_TRYS( post_tank_scan( s ) );
    BORA_TRYS( post_redistance( s ) );
    BORA_TRYS( post_attributes( s ) );
    s->warm_ready = false;  // the post-processing stages use pres as scratch and clear it
    return BORA_OK;
}

int add_particles( bora_flip_sim* s, const float* pos, const float* vel, size_t n, int space )
{
    if( n == 0 ) return BORA_OK;
    if( !pos ) return BORA_ERR_INVALID_ARG;
    if( s->np + n > (size_t)0x7FFFFFF0 ) return BORA_ERR_CAPACITY;
    BORA_TRYS( ensure_particles( s, s->np + n ) );
    BORA_TRY( grow( s->stage_in, n * 24, false, s->st ) );
    float* dpos = P<float>( s->stage_in );
    float* dvel = dpos + 3 * n;
    BORA_TRY( cudaMemcpyAsync( dpos, pos, n * 12, cudaMemcpyHostToDevice, s->st ) );
    if( vel ) BORA_TRY( cudaMemcpyAsync( dvel, vel, n * 12, cudaMemcpyHostToDevice, s->st ) );
    s->stats.kernel_launches += 1;
    bora_launch_to_soa( n, dpos, vel ? dvel : nullptr, space == BORA_SPACE_VOXEL ? 1 : 0, s->translate, s->scale,
                        s->parts( s->cur ), s->np, s->next_id, s->st );
    BORA_TRY( cudaMemsetAsync( P<float>( s->adj ) + s->np, 0, n * 4, s->st ) );
    if( s->attrs )  // FLIPMethod::newParticle appends vorticity and curvature 0 (FLIPMethod.h:94-96)
        for( int a = 0; a < 2; ++a ) BORA_TRY( cudaMemsetAsync( P<float>( s->pattr[s->cur][a] ) + s->np, 0, n * 4, s->st ) );
    BORA_TRYS( check_launch( s ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );  // the caller may free its buffers on return
    s->np += n;
    s->nlive += n;
    s->next_id += (int32_t)n;
    s->sorted = false;
    s->keys_valid = false;
    s->pres_valid = false;
    s->stats.num_particles = s->nlive;
    return BORA_OK;
}

}  // namespace

// ======================================================================================
// Every device buffer of a handle.
template <class F>
void for_each_buffer( bora_flip_sim* s, F&& f )
{
    DevBuf* all[] = { &s->tile_flag, &s->tile_act, &s->tile_excl, &s->slot_of, &s->tile_of, &s->nbr, &s->mass, &s->surf,
                      &s->pres, &s->vx, &s->vy, &s->vz, &s->cx, &s->cy, &s->cz, &s->flag, &s->code, &s->rhs, &s->sx,
                      &s->se, &s->sr, &s->sd0, &s->sd1, &s->sq, &s->sz, &s->sminv, &s->cell_count, &s->cell_start,
                      &s->ring, &s->partials, &s->done, &s->adj, &s->vkey, &s->key, &s->idx, &s->scan_scratch,
                      &s->counters, &s->stage_in, &s->stage_out, &s->live_flag, &s->col_phi, &s->col_vel,
                      &s->col_tslot, &s->col_tnear, &s->col_tphi, &s->col_tvel, &s->gbar };
    for( DevBuf* b : all ) f( *b );
    for( int q = 0; q < 2; ++q )
    {
        for( int a = 0; a < 7; ++a ) f( s->pbuf[q][a] );
        for( int a = 0; a < 2; ++a ) f( s->pattr[q][a] );
    }
    f( s->labels );
    f( s->exp_buf );
    for( int l = 0; l < bora_flip_sim::kMaxLevels; ++l )
    {
        f( s->mg_type[l] ); f( s->mg_code[l] ); f( s->mg_r[l] );
        f( s->mg_z0[l] ); f( s->mg_z1[l] );
    }
    f( s->mg_mid );
    f( s->vdb_leaf ); f( s->vdb_mask ); f( s->vdb_val );
}

extern "C" {

int bora_flip_default_params( bora_flip_params* o )
{
    if( !o ) return BORA_ERR_INVALID_ARG;
    std::memset( o, 0, sizeof( *o ) );
    o->ext_force[0] = 0.f; o->ext_force[1] = -9.80665f; o->ext_force[2] = 0.f;
    o->max_substeps = 1;
    o->dt = 1.f / 24.f;
    o->wall_level = -1e+30f;
    o->enable_water_tank = 0;
    o->enable_curl = 0;
    o->damping_band = 0.f;
    o->voxel_size = 0.1f;
    o->col_vel_scale = 1.f;
    o->pts_per_cell = 8;
    o->vort_pres_rate = 0.2f;
    o->adjacency_under = 2.f;
    o->proj_iteration = 200;
    o->redist_iteration = 80;
    o->solver = BORA_SOLVER_PLAIN;
    o->tolerance = 1e-6;
    o->div_tolerance = 1e-5;
    o->inner_tolerance = 1e-3;
    o->max_refinements = 8;
    o->check_every = 1;
    o->advection = BORA_ADVECT_EULER;
    o->post_process = 1;
    o->persistent = 0;
    o->warm_start = 0;
    return BORA_OK;
}

static int validate_params( const bora_flip_params* p )
{
    if( !p ) return BORA_ERR_INVALID_ARG;
    if( p->enable_curl ) return BORA_ERR_INVALID_ARG;  // curl noise is outside this library
    if( p->solver != BORA_SOLVER_PLAIN && p->solver != BORA_SOLVER_MIXED ) return BORA_ERR_INVALID_ARG;
    if( p->advection != BORA_ADVECT_EULER && p->advection != BORA_ADVECT_RK2 ) return BORA_ERR_INVALID_ARG;
    if( !( p->voxel_size > 0.f ) || !( p->tolerance > 0.0 ) ) return BORA_ERR_INVALID_ARG;
    if( p->persistent != 0 && p->persistent != 1 ) return BORA_ERR_INVALID_ARG;
    if( p->warm_start != 0 && p->warm_start != 1 ) return BORA_ERR_INVALID_ARG;
    return BORA_OK;
}

int bora_flip_create( const bora_grid_desc* grid, const bora_flip_params* params, bora_flip_handle* out )
{
    if( !grid || !out ) return BORA_ERR_INVALID_ARG;
    *out = nullptr;
    if( grid->nx <= 0 || grid->ny <= 0 || grid->nz <= 0 ) return BORA_ERR_INVALID_ARG;
    if( (double)grid->nx * grid->ny * grid->nz > 4.0e9 ) return BORA_ERR_CAPACITY;
    for( int a = 0; a < 3; ++a )
        if( !( grid->max[a] > grid->min[a] ) ) return BORA_ERR_INVALID_ARG;
    bora_flip_params defaults;
    bora_flip_default_params( &defaults );
    const bora_flip_params* p = params ? params : &defaults;
    BORA_TRYS( validate_params( p ) );
    int ndev = 0;
    if( cudaGetDeviceCount( &ndev ) != cudaSuccess || ndev == 0 ) return BORA_ERR_NO_DEVICE;
    bora_flip_sim* s = new( std::nothrow ) bora_flip_sim();
    if( !s ) return BORA_ERR_OUT_OF_MEMORY;
    cudaGetDevice( &s->device );
    s->gdesc = *grid;
    s->prm = *p;
    setup_frame( s );
    apply_params( s );
    int st = cuda_status( cudaStreamCreateWithFlags( &s->st, cudaStreamNonBlocking ) );
    if( st == BORA_OK ) st = cuda_status( cudaEventCreate( &s->ev_step[0] ) );
    if( st == BORA_OK ) st = cuda_status( cudaEventCreate( &s->ev_step[1] ) );
    if( st == BORA_OK ) st = cuda_status( cudaEventCreateWithFlags( &s->ev_join, cudaEventDisableTiming ) );
    if( st == BORA_OK ) st = cuda_status( cudaHostAlloc( (void**)&s->h_cnt, 64, cudaHostAllocMapped ) );
    if( st == BORA_OK ) st = cuda_status( cudaHostGetDevicePointer( (void**)&s->d_cnt, s->h_cnt, 0 ) );
    if( st == BORA_OK ) st = cuda_status( cudaHostAlloc( (void**)&s->h_ring, 64, cudaHostAllocMapped ) );
    if( st == BORA_OK ) st = cuda_status( cudaHostGetDevicePointer( (void**)&s->d_hring, s->h_ring, 0 ) );
    if( st == BORA_OK ) st = cuda_status( cudaHostAlloc( (void**)&s->h_mirror, BORA_RING * 8, cudaHostAllocMapped ) );
    if( st == BORA_OK ) st = cuda_status( cudaHostGetDevicePointer( (void**)&s->d_mirror, s->h_mirror, 0 ) );
    for( int q = 0; q < bora_flip_sim::kChecks && st == BORA_OK; ++q )
        st = cuda_status( cudaEventCreateWithFlags( &s->ev_chk[q], cudaEventDisableTiming ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->tile_flag, s->ntv, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->tile_act, s->ntv * 4, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->tile_excl, s->ntv * 4, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->slot_of, s->ntv * 4, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->slot_prev, s->ntv * 4, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->counters, 64, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->ring, BORA_RING * 8, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->done, BORA_RING * 4, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( grow( s->gbar, 16, false, s->st ) );
    if( st == BORA_OK ) st = cuda_status( cudaMemsetAsync( s->done.p, 0, BORA_RING * 4, s->st ) );
    if( st == BORA_OK ) st = cuda_status( cudaMemsetAsync( s->ring.p, 0, BORA_RING * 8, s->st ) );
    if( st == BORA_OK ) st = ensure_cells( s, 1 );
    if( st == BORA_OK ) st = ensure_scan_scratch( s, s->ntv + 2 );
    if( st == BORA_OK ) st = cuda_status( cudaStreamSynchronize( s->st ) );
    if( st != BORA_OK )
    {
        bora_flip_destroy( s );
        return st;
    }
    *out = s;
    return BORA_OK;
}

int bora_flip_destroy( bora_flip_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( s->st ) cudaStreamSynchronize( s->st );
    if( s->st_copy ) cudaStreamSynchronize( s->st_copy );
    for_each_buffer( s, []( DevBuf& b ) { release( b ); } );
    if( s->ev_gathered ) cudaEventDestroy( s->ev_gathered );
    if( s->ev_copied ) cudaEventDestroy( s->ev_copied );
    if( s->st_copy ) cudaStreamDestroy( s->st_copy );
    s->prof_resolve();
    for( cudaEvent_t e : s->evpool ) cudaEventDestroy( e );
    for( int q = 0; q < 2; ++q )
        if( s->ev_step[q] ) cudaEventDestroy( s->ev_step[q] );
    for( cudaEvent_t e : s->ev_chk )
        if( e ) cudaEventDestroy( e );
    if( s->ev_join ) cudaEventDestroy( s->ev_join );
    if( s->h_cnt ) cudaFreeHost( s->h_cnt );
    if( s->h_ring ) cudaFreeHost( s->h_ring );
    if( s->h_mirror ) cudaFreeHost( s->h_mirror );
    if( s->st ) cudaStreamDestroy( s->st );
    delete s;
    return BORA_OK;
}

int bora_flip_set_params( bora_flip_handle s, const bora_flip_params* p )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    BORA_TRYS( validate_params( p ) );
    s->prm = *p;
    apply_params( s );
    s->sorted = false;  // the water tank's rows change the activation
    s->keys_valid = false;
    s->pres_valid = false;
    return BORA_OK;
}

int bora_flip_add_particles( bora_flip_handle s, const float* pos, const float* vel, size_t n, int space )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    return add_particles( s, pos, vel, n, space );
}

int bora_flip_fill_water_tank( bora_flip_handle s, size_t* added )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( added ) *added = 0;
    const float wall = s->g.voxel_wall;
    if( wall <= 0.f ) return BORA_OK;  // FLIPMethod.cu:409
    const int hh = std::max( 0, std::min( (int)wall + 1, s->g.ny ) );
    const size_t ncell = (size_t)s->g.nx * hh * s->g.nz;
    if( ncell == 0 ) return BORA_OK;
    cudaStream_t st = s->st;
    BORA_TRY( grow( s->stage_in, ( 2 * ncell + 2 ) * 4, false, st ) );
    uint32_t* count = P<uint32_t>( s->stage_in );
    uint32_t* offset = count + ncell + 1;
    BORA_TRYS( ensure_scan_scratch( s, ncell + 1 ) );
    const float3 tr = make_float3( s->translate[0], s->translate[1], s->translate[2] );
    const float3 sc = make_float3( s->scale[0], s->scale[1], s->scale[2] );
    const int per_cell = std::max( 0, s->prm.pts_per_cell );
    s->stats.kernel_launches += 2;
    bora_launch_tank( s->g, hh, per_cell, tr, sc, count, nullptr, s->parts( s->cur ), 0, 0, false, st );
    bora_device_scan( count, offset, ncell, P<uint32_t>( s->scan_scratch ), P<uint32_t>( s->counters ) + 7, st );
    BORA_TRYS( check_launch( s ) );
    BORA_TRYS( read_counters( s, 7, 1 ) );
    const size_t n = s->h_cnt[7];
    if( n == 0 ) return BORA_OK;
    if( s->np + n > (size_t)0x7FFFFFF0 ) return BORA_ERR_CAPACITY;
    BORA_TRYS( ensure_particles( s, s->np + n ) );
    s->stats.kernel_launches += 1;
    bora_launch_tank( s->g, hh, per_cell, tr, sc, count, offset, s->parts( s->cur ), s->np, s->next_id, true, st );
    BORA_TRY( cudaMemsetAsync( P<float>( s->adj ) + s->np, 0, n * 4, st ) );
    if( s->attrs )
        for( int a = 0; a < 2; ++a ) BORA_TRY( cudaMemsetAsync( P<float>( s->pattr[s->cur][a] ) + s->np, 0, n * 4, st ) );
    BORA_TRYS( check_launch( s ) );
    BORA_TRY( cudaStreamSynchronize( st ) );
    s->np += n;
    s->nlive += n;
    s->next_id += (int32_t)n;
    s->sorted = false;
    s->keys_valid = false;
    s->pres_valid = false;
    s->stats.num_particles = s->nlive;
    if( added ) *added = n;
    return BORA_OK;
}

int bora_flip_clear_particles( bora_flip_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    s->np = 0;
    s->nlive = 0;
    s->next_id = 0;
    s->sorted = false;
    s->keys_valid = false;
    s->pres_valid = false;
    s->attrs = false;
    s->stats.num_particles = 0;
    return BORA_OK;
}

int bora_flip_set_particles( bora_flip_handle s, const float* pos, const float* vel, size_t n, int space )
{
    BORA_TRYS( bora_flip_clear_particles( s ) );
    return add_particles( s, pos, vel, n, space );
}

int bora_flip_set_colliders( bora_flip_handle s, const float* boxes, int n, float band )
{
    if( !s || n < 0 || n > BORA_MAX_COLLIDERS || ( n > 0 && !boxes ) || !( band > 0.f ) ) return BORA_ERR_INVALID_ARG;
    BoraColliderDev& c = s->g.cols;
    std::memset( &c, 0, sizeof( c ) );
    c.count = n;
    c.band = band;
    for( int q = 0; q < n; ++q )
        for( int a = 0; a < 3; ++a )
        {
            c.box[q].lo[a] = boxes[9 * q + a];
            c.box[q].hi[a] = boxes[9 * q + 3 + a];
            c.box[q].vel[a] = boxes[9 * q + 6 + a];
        }
    return BORA_OK;
}

int bora_flip_set_collider_field( bora_flip_handle s, const float* phi, const float* vel, size_t ncells )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    BoraColliderDev& c = s->g.cols;
    if( !phi )
    {
        c.fphi = nullptr;
        c.fvel = nullptr;
        return BORA_OK;
    }
    const size_t n = (size_t)s->g.nx * s->g.ny * s->g.nz;
    if( ncells != n ) return BORA_ERR_INVALID_ARG;
    // all allocations first; then the copies. A failure after the first copy leaves no
    // collider at all rather than a mix of the old and the new one.
    BORA_TRY( grow( s->col_phi, n * 4, false, s->st ) );
    if( vel ) BORA_TRY( grow( s->col_vel, n * 12, false, s->st ) );
    c.fphi = nullptr;
    c.fvel = nullptr;
    c.tslot = nullptr;
    c.count = 0;  // replaces any boxes or sparse collider
    BORA_TRY( cudaMemcpyAsync( s->col_phi.p, phi, n * 4, cudaMemcpyHostToDevice, s->st ) );
    if( vel ) BORA_TRY( cudaMemcpyAsync( s->col_vel.p, vel, n * 12, cudaMemcpyHostToDevice, s->st ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );  // the caller may free its buffers on return
    c.fphi = P<float>( s->col_phi );
    c.fvel = vel ? P<float>( s->col_vel ) : nullptr;
    return BORA_OK;
}

int bora_flip_set_collider_voxels( bora_flip_handle s, const int32_t* ijk, const float* phi, const float* vel,
                                   size_t count, float background )
{
    if( !s || ( count > 0 && ( !ijk || !phi ) ) || !std::isfinite( background ) ) return BORA_ERR_INVALID_ARG;
    BoraColliderDev& c = s->g.cols;
    if( count == 0 )
    {
        c.tslot = nullptr;
        c.tnear = nullptr;
        return BORA_OK;
    }
    const int nx = s->g.nx, ny = s->g.ny, nz = s->g.nz, tx = s->g.tx, ty = s->g.ty, tz = s->g.tz;
    const size_t ntv = (size_t)tx * ty * tz;
    auto tlin = [&]( int a, int b, int d ) { return (size_t)a + (size_t)tx * ( (size_t)b + (size_t)ty * d ); };
    // SparseFrame::buildFromPoints over the active voxels (SparseFrame.cu:83-155): a tile is
    // the collider's when an active voxel lies in it or in one of its 26 neighbours
    std::vector<uint8_t> hit( ntv, 0 ), own( ntv, 0 ), near( ntv, 0 );
    for( size_t v = 0; v < count; ++v )
    {
        const int i = ijk[3 * v], j = ijk[3 * v + 1], k = ijk[3 * v + 2];
        if( i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz ) continue;  // outside the frame: never sampled
        hit[tlin( i >> 3, j >> 3, k >> 3 )] = 1;
    }
    auto dilate = [&]( const std::vector<uint8_t>& in, std::vector<uint8_t>& out ) {
        for( int d = 0; d < tz; ++d )
            for( int b = 0; b < ty; ++b )
                for( int a = 0; a < tx; ++a )
                {
                    if( !in[tlin( a, b, d )] ) continue;
                    for( int dd = std::max( 0, d - 1 ); dd <= std::min( tz - 1, d + 1 ); ++dd )
                        for( int bb = std::max( 0, b - 1 ); bb <= std::min( ty - 1, b + 1 ); ++bb )
                            for( int aa = std::max( 0, a - 1 ); aa <= std::min( tx - 1, a + 1 ); ++aa )
                                out[tlin( aa, bb, dd )] = 1;
                }
    };
    dilate( hit, own );
    dilate( own, near );
    // slots in linear tile order; samples: phi / h and v / scale (CollisionSource.h:105-121),
    // the background / h on the other cells of the collider's tiles
    const float h = s->scale[0];
    std::vector<int32_t> slot( ntv, -1 );
    int nslots = 0;
    for( size_t t = 0; t < ntv; ++t )
        if( own[t] ) slot[t] = nslots++;
    const float bg = background / h;
    std::vector<float> tphi( (size_t)nslots * 512, bg ), tvel;
    if( vel ) tvel.assign( (size_t)nslots * 512 * 3, 0.f );
    for( size_t v = 0; v < count; ++v )
    {
        const int i = ijk[3 * v], j = ijk[3 * v + 1], k = ijk[3 * v + 2];
        if( i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz ) continue;
        const size_t q = (size_t)slot[tlin( i >> 3, j >> 3, k >> 3 )] * 512 + (size_t)bora_local( i, j, k );
        tphi[q] = phi[v] / h;
        if( vel )
            for( int a = 0; a < 3; ++a ) tvel[3 * q + a] = vel[3 * v + a] / s->scale[a];
    }
    // all allocations first; a failure after the first copy leaves no collider at all
    BORA_TRY( grow( s->col_tslot, ntv * 4, false, s->st ) );
    BORA_TRY( grow( s->col_tnear, ntv, false, s->st ) );
    BORA_TRY( grow( s->col_tphi, tphi.size() * 4 + 16, false, s->st ) );
    if( vel ) BORA_TRY( grow( s->col_tvel, tvel.size() * 4 + 16, false, s->st ) );
    std::memset( &c, 0, sizeof( c ) );  // replaces any boxes or per-cell field
    BORA_TRY( cudaMemcpyAsync( s->col_tslot.p, slot.data(), ntv * 4, cudaMemcpyHostToDevice, s->st ) );
    BORA_TRY( cudaMemcpyAsync( s->col_tnear.p, near.data(), ntv, cudaMemcpyHostToDevice, s->st ) );
    BORA_TRY( cudaMemcpyAsync( s->col_tphi.p, tphi.data(), tphi.size() * 4, cudaMemcpyHostToDevice, s->st ) );
    if( vel ) BORA_TRY( cudaMemcpyAsync( s->col_tvel.p, tvel.data(), tvel.size() * 4, cudaMemcpyHostToDevice, s->st ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );  // the host vectors go out of scope
    c.tslot = P<int32_t>( s->col_tslot );
    c.tnear = P<uint8_t>( s->col_tnear );
    c.tphi = P<float>( s->col_tphi );
    c.tvel = vel ? P<float>( s->col_tvel ) : nullptr;
    c.tbg = bg;
    c.ttx = tx;
    c.tty = ty;
    return BORA_OK;
}

int bora_flip_run_stage( bora_flip_handle s, int stage, float dt )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    switch( stage )
    {
        case BORA_STAGE_REBUILD: return stage_rebuild( s );
        case BORA_STAGE_P2G: return stage_p2g( s );
        case BORA_STAGE_BUILD_SYSTEM: return stage_build_system( s );
        case BORA_STAGE_SOLVE: return stage_solve( s );
        case BORA_STAGE_UPDATE_VELOCITY: return stage_update_velocity( s );
        case BORA_STAGE_UPDATE_PARTICLES: return stage_update_particles( s, dt );
        default: return BORA_ERR_INVALID_ARG;
    }
}

int bora_flip_step( bora_flip_handle s, float dt )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( s->np == 0 ) return BORA_OK;  // FLIPMethod.cu:179
    const auto t0 = std::chrono::steady_clock::now();
    cudaEventRecord( s->ev_step[0], s->st );
    // FLIPMethod.cu:210: the frame is rebuilt unless post-processing has just built it
    // from these particles (prepareNextStep)
    if( !s->sorted ) BORA_TRYS( stage_rebuild( s ) );
    BORA_TRYS( stage_p2g( s ) );
    BORA_TRYS( stage_build_system( s ) );
    const int solve = stage_solve( s );
    BORA_TRYS( solve );
    BORA_TRYS( stage_update_velocity( s ) );
    BORA_TRYS( stage_update_particles( s, dt ) );
    cudaEventRecord( s->ev_step[1], s->st );
    BORA_TRY( cudaEventSynchronize( s->ev_step[1] ) );
    float gms = 0.f;
    cudaEventElapsedTime( &gms, s->ev_step[0], s->ev_step[1] );
    s->stats.gpu_ms = gms;
    s->prof_resolve();
    bora_tune_resolve();
    s->stats.steps++;
    s->stats.stage_ms[7] = std::chrono::duration<double, std::milli>( std::chrono::steady_clock::now() - t0 ).count();
    return solve;
}

// ---- batched steps ---------------------------------------------------------------------
//
// bora_flip_step_batch advances several simulations one step each. Their per-simulation
// stages (tile rebuild and sort, P2G, system and multigrid set-up, velocity update, G2P)
// run on each simulation's own stream, every part issued for all of them before the host
// waits on any; the pressure solve - all but a few of a step's launches - runs every kernel
// once for all of them: simulation k of the batch is row blockIdx.y of
// each launch, on the grid of its own single launch, reducing into its own ring (the
// batched kernels in projection.cu, multigrid.cu and mg_mid.cu). Each simulation follows
// stage_solve's control flow on its own (refinement passes, convergence checks one
// iteration late, residual replacement), so its launches and arithmetic are the same
// whether it runs alone or in a batch; a launch row of a simulation that is between passes
// or finished returns at once.

namespace {

struct BatchMember
{
    bora_flip_sim* s = nullptr;
    int row = 0;    // row of the batched launches
    int index = 0;  // position in the caller's array
    enum Phase { kStart, kInner, kRefine, kDone } phase = kStart;
    double bnorm = 0, rnorm = 0, rmax = 0, dx = 1, target = 0;
    int total_it = 0, passes = 0, it = 0, max_inner = 1, check = 1;
    bool converged = false, inner_done = false;
    int rz_prev = -1, dsel = 0, rz_cur = -1, rr_cur = -1, a_rz = -1, a_dq = -1;
    int s_b2 = -1, s_bmax = -1, s_n2 = -1, s_mx = -1;
    struct Check { int it, tick, slot; };
    Check pend[bora_flip_sim::kChecks];
    int npend = 0;

    double mirror( int slot ) const { return ( (volatile double*)s->h_mirror )[slot]; }
    // the check at the top of stage_solve's pass loop
    void decide()
    {
        const bora_flip_params& p = s->prm;
        const bool norm_ok = rnorm <= p.tolerance * bnorm;
        const bool max_ok = rmax * dx <= p.div_tolerance;
        if( bnorm == 0.0 || ( norm_ok && max_ok ) ) { converged = true; phase = kDone; return; }
        if( passes >= std::max( 1, p.max_refinements ) ) { phase = kDone; return; }
        target = norm_ok ? 0.1 * rnorm : std::max( p.inner_tolerance * rnorm, 0.25 * p.tolerance * bnorm );
        phase = kStart;
    }
};

struct BatchBuffers
{
    DevBuf ms, sl, mid;
};

int batch_solve( std::vector<BatchMember>& M, cudaStream_t st, BatchBuffers& bb, bora_flip_sim* host_of_events )
{
    const int n = (int)M.size();
    // static per-simulation records: solver vectors, reductions, levels, own grids, and the
    // coarse cluster kernel's descriptors
    std::vector<BoraMemberSolve> ms( n );
    const size_t dbytes = bora_mg_mid_desc_bytes();
    std::vector<char> mid( dbytes * n );
    int ctas = 0;
    size_t smem = 0;
    // the launch shapes of the multigrid passes for this batch (the autotuner's choice for
    // the batch's total size; every shape gives the same results)
    int total_tiles = 0;
    for( int k = 0; k < n; ++k ) total_tiles += M[k].s->ntiles;
    const int tgroup[3] = { kBoraTuneL0Batch, kBoraTuneL1Batch, kBoraTuneL2Batch };
    BoraTunePick tpick[3];
    int tv[3];
    for( int l = 0; l < 3; ++l )
    {
        tpick[l] = bora_tune_pick( tgroup[l], total_tiles );
        tv[l] = tpick[l].variant;
    }
    for( int k = 0; k < n; ++k )
    {
        bora_flip_sim* s = M[k].s;
        BoraMemberSolve& m = ms[k];
        m.ntiles = s->ntiles;
        m.nbr = P<int32_t>( s->nbr );
        m.code = P<uint16_t>( s->code );
        m.b = P<float>( s->rhs );
        m.pres = P<float>( s->pres );
        m.sv = s->solver();
        m.red = s->reducer();
        for( int l = 0; l < 4; ++l ) m.L[l] = s->levels[l];
        m.z3 = s->levels[3].z0;
        bora_member_grids( s->ntiles, m.grid, tv );
        size_t sm = 0;
        int c = 0;
        if( !bora_mg_mid_describe( s->g, s->levels, s->nlevels, s->tiles(), s->ntiles, s->mg_mid.p,
                                   P<uint32_t>( s->counters ) + 5, 16, mid.data() + dbytes * k, &sm, &c ) )
            return BORA_ERR_INTERNAL;
        if( ctas && c != ctas ) return BORA_ERR_INTERNAL;
        ctas = c;
        smem = std::max( smem, sm );
    }
    // a launch group's arguments: the slots, then per kernel (and the coarse cluster kernel)
    // the n + 1 block offsets of the simulations taking part
    constexpr int kRows = kGridCount + 1;
    const size_t sl_bytes = sizeof( BoraMemberSlots ) * n;
    const size_t grp_bytes = sl_bytes + sizeof( int ) * kRows * ( n + 1 );
    BORA_TRY( grow( bb.ms, sizeof( BoraMemberSolve ) * n, false, st ) );
    BORA_TRY( grow( bb.sl, grp_bytes, false, st ) );
    BORA_TRY( grow( bb.mid, dbytes * n, false, st ) );
    BORA_TRY( cudaMemcpyAsync( bb.ms.p, ms.data(), sizeof( BoraMemberSolve ) * n, cudaMemcpyHostToDevice, st ) );
    BORA_TRY( cudaMemcpyAsync( bb.mid.p, mid.data(), dbytes * n, cudaMemcpyHostToDevice, st ) );
    const BoraMemberSolve* dms = P<BoraMemberSolve>( bb.ms );
    const BoraMemberSlots* dsl = P<BoraMemberSlots>( bb.sl );
    const int* dstart = reinterpret_cast<const int*>( static_cast<const char*>( bb.sl.p ) + sl_bytes );
    std::vector<char> grp( grp_bytes );
    BoraMemberSlots* sl = reinterpret_cast<BoraMemberSlots*>( grp.data() );
    int* start = reinterpret_cast<int*>( grp.data() + sl_bytes );
    int blocks[kRows] = {};
    uint64_t launches = 0;
    // this launch group's arguments; the copy is stream-ordered after every earlier launch
    // that read the buffer
    auto upload = [&]() -> int {
        for( int q = 0; q < kRows; ++q )
        {
            int acc = 0;
            for( int k = 0; k < n; ++k )
            {
                start[q * ( n + 1 ) + k] = acc;
                if( sl[k].active ) acc += q < kGridCount ? ms[k].grid[q] : ctas;
            }
            start[q * ( n + 1 ) + n] = acc;
            blocks[q] = acc;
        }
        BORA_TRY( cudaMemcpyAsync( bb.sl.p, grp.data(), grp_bytes, cudaMemcpyHostToDevice, st ) );
        return BORA_OK;
    };
    auto launch = [&]( int q ) { return BoraBatchLaunch{ dms, dsl, dstart + q * ( n + 1 ), n }; };
    const int lgrid[3] = { kGridPass0, kGridPass1, kGridPass2 };
    auto vcycle = [&]() {
        for( int l = 0; l < 3; ++l )
        {
            BoraTuneTimer timer( tpick[l], tgroup[l], total_tiles, st );  // times the level's two down passes
            for( int p = 0; p < 2; ++p )
            {
                // level 0's down 1 and up 2 reduce over their blocks: the fixed shape's grid
                const int q = l == 0 && p == 0 ? kGridPass0R : lgrid[l];
                bora_launch_mg_pass_batch( l, p, tv[l], launch( q ), blocks[q], st );
            }
        }
        bora_mg_mid_launch_batch( bb.mid.p, launch( kGridCount ), blocks[kGridCount], ctas, smem, st );
        for( int l = 2; l >= 0; --l )
            for( int p = 2; p < 4; ++p )
            {
                const int q = l == 0 && p == 3 ? kGridPass0R : lgrid[l];
                bora_launch_mg_pass_batch( l, p, tv[l], launch( q ), blocks[q], st );
            }
        launches += 13;
    };
    // r = b, x = e = d = q = 0; ||b||^2, max|b|
    for( int k = 0; k < n; ++k )
    {
        BatchMember& b = M[k];
        b.s_b2 = b.s->slot();
        b.s_bmax = b.s->slot();
        sl[k] = BoraMemberSlots{};
        sl[k].active = 1;
        sl[k].n2 = b.s_b2;
        sl[k].mx = b.s_bmax;
        BORA_TRY( cudaMemsetAsync( P<uint32_t>( b.s->counters ) + 5, 0, 4, st ) );
    }
    BORA_TRYS( upload() );
    bora_launch_solve_init_batch( launch( kGridCells ), blocks[kGridCells], st );
    ++launches;
    BORA_TRYS( check_launch( nullptr ) );
    BORA_TRY( cudaStreamSynchronize( st ) );
    for( BatchMember& b : M )
    {
        b.dx = b.s->scale[0];
        b.bnorm = std::sqrt( b.mirror( b.s_b2 ) );
        b.rnorm = b.bnorm;
        b.rmax = b.mirror( b.s_bmax );
        b.max_inner = std::max( 1, b.s->prm.proj_iteration );
        b.check = std::max( 1, b.s->prm.check_every );
        b.decide();
    }
    int tick = 0;
    cudaEvent_t* tev = host_of_events->ev_chk;
    constexpr int kTicks = bora_flip_sim::kChecks;
    for( ;; )
    {
        // passes that start: the first V-cycle z = M^-1 r with r.r (no residual update; scaled
        // by ||b|| on the first pass, by the refined ||r|| after)
        bool start = false;
        for( int k = 0; k < n; ++k )
        {
            BatchMember& b = M[k];
            sl[k] = BoraMemberSlots{};
            if( b.phase != BatchMember::kStart ) continue;
            b.rz_cur = b.s->slot();
            b.rr_cur = b.s->slot();
            sl[k].active = 1;
            sl[k].rz_in = -1;
            sl[k].dq_in = -1;
            sl[k].rr_out = b.rr_cur;
            sl[k].rr = b.passes == 0 ? b.s_b2 : b.s_n2;
            sl[k].rz = b.rz_cur;
            b.phase = BatchMember::kInner;
            b.it = 0;
            b.npend = 0;
            b.a_rz = b.a_dq = -1;
            b.inner_done = false;
            b.s->stats.mg_vcycle_launches = 13;
            start = true;
        }
        if( start )
        {
            BORA_TRYS( upload() );
            vcycle();
        }
        // one inner iteration for every simulation inside a pass
        bool inner = false;
        for( int k = 0; k < n; ++k )
        {
            BatchMember& b = M[k];
            sl[k] = BoraMemberSlots{};
            if( b.phase != BatchMember::kInner || b.inner_done || b.it >= b.max_inner ) continue;
            const int s_dq = b.s->slot();
            const int rz_new = b.s->slot(), rr_new = b.s->slot();
            BoraMemberSlots& q = sl[k];
            q.active = 1;
            q.dsel = b.dsel;
            q.rz_new = b.rz_cur; q.rz_old = b.rz_prev; q.dq = s_dq; q.a_rz = b.a_rz; q.a_dq = b.a_dq;
            q.rz_in = b.rz_cur; q.dq_in = s_dq; q.rr_out = rr_new;
            q.rr = b.rr_cur; q.rz = rz_new;  // the V-cycle's scale: the previous r.r
            b.dsel ^= 1;
            b.a_rz = b.rz_cur;
            b.a_dq = s_dq;
            b.rz_prev = b.rz_cur;
            b.rz_cur = rz_new;
            b.rr_cur = rr_new;
            ++b.it;
            inner = true;
        }
        if( inner )
        {
            BORA_TRYS( upload() );
            bora_launch_pcg_direction_batch( launch( kGridDir ), blocks[kGridDir], st );
            ++launches;
            vcycle();  // with the residual update
            BORA_TRYS( check_launch( nullptr ) );
            BORA_TRY( cudaEventRecord( tev[tick % kTicks], st ) );
            for( int k = 0; k < n; ++k )
            {
                if( !sl[k].active ) continue;
                BatchMember& b = M[k];
                if( b.it % b.check == 0 ) b.pend[b.npend++] = BatchMember::Check{ b.it, tick, b.rr_cur };
                // the convergence check of stage_solve: iteration i is read once i + 1 is queued
                while( b.npend > 0 && ( b.it - b.pend[0].it >= 1 || b.npend == kTicks || b.it >= b.max_inner ) )
                {
                    BORA_TRY( cudaEventSynchronize( tev[b.pend[0].tick % kTicks] ) );
                    const double rr = b.mirror( b.pend[0].slot );
                    for( int q = 1; q < b.npend; ++q ) b.pend[q - 1] = b.pend[q];
                    --b.npend;
                    if( !( rr > 0.0 ) || std::sqrt( rr ) <= b.target ) { b.inner_done = true; break; }
                }
            }
            ++tick;
        }
        // passes that end: refinement (x += e; r = b - A x in double-float arithmetic)
        bool refine = false;
        for( int k = 0; k < n; ++k )
        {
            BatchMember& b = M[k];
            sl[k] = BoraMemberSlots{};
            if( b.phase != BatchMember::kInner || !( b.inner_done || b.it >= b.max_inner ) ) continue;
            b.s_n2 = b.s->slot();
            b.s_mx = b.s->slot();
            sl[k].active = 1;
            sl[k].dsel = b.dsel;
            sl[k].a_rz = b.a_rz;
            sl[k].a_dq = b.a_dq;
            sl[k].n2 = b.s_n2;
            sl[k].mx = b.s_mx;
            b.phase = BatchMember::kRefine;
            refine = true;
        }
        if( refine )
        {
            BORA_TRYS( upload() );
            bora_launch_refine_accumulate_batch( launch( kGridCells ), blocks[kGridCells], st );
            bora_launch_refine_residual_batch( launch( kGridResidual ), blocks[kGridResidual], st );
            launches += 2;
            BORA_TRYS( check_launch( nullptr ) );
            BORA_TRY( cudaStreamSynchronize( st ) );
            for( BatchMember& b : M )
            {
                if( b.phase != BatchMember::kRefine ) continue;
                b.total_it += b.it;
                ++b.passes;
                b.rnorm = std::sqrt( b.mirror( b.s_n2 ) );
                b.rmax = b.mirror( b.s_mx );
                if( !std::isfinite( b.rnorm ) ) { b.phase = BatchMember::kDone; continue; }
                // continue the recurrence only while the refined and recursive residuals agree
                const double rr_rec = b.mirror( b.rr_cur );
                const double rec = rr_rec > 0.0 ? std::sqrt( rr_rec ) : 0.0;
                if( !( rec > 0.0 ) || b.rnorm > 1.5 * rec ) b.rz_prev = -1;
                b.decide();
            }
        }
        bool any = false;
        for( const BatchMember& b : M ) any = any || b.phase != BatchMember::kDone;
        if( !any ) break;
    }
    for( int k = 0; k < n; ++k )
    {
        sl[k] = BoraMemberSlots{};
        sl[k].active = 1;
    }
    BORA_TRYS( upload() );
    bora_launch_write_pressure_batch( launch( kGridCells ), blocks[kGridCells], st );
    ++launches;
    BORA_TRYS( check_launch( nullptr ) );
    for( BatchMember& b : M ) BORA_TRYS( issue_counters( b.s, 5, 2, st ) );
    BORA_TRY( cudaStreamSynchronize( st ) );
    int status = BORA_OK;
    for( BatchMember& b : M )
    {
        bora_flip_sim* s = b.s;
        s->stats.kernel_launches += launches;
        if( s->h_cnt[5] != 0 ) return BORA_ERR_INTERNAL;
        s->stats.fluid_cells = (int32_t)s->h_cnt[6];
        s->stats.solver_iterations = b.total_it;
        s->stats.refinements = b.passes;
        s->stats.residual_rel = b.bnorm > 0.0 ? b.rnorm / b.bnorm : 0.0;
        s->stats.residual_max = b.rmax;
        s->stats.residual_max_dx = b.rmax * b.dx;
        s->stats.converged = b.converged ? 1 : 0;
        s->last_status = b.converged ? BORA_OK : BORA_WARN_NOT_CONVERGED;
        if( !b.converged ) status = BORA_WARN_NOT_CONVERGED;
    }
    return status;
}

}  // namespace

int bora_flip_step_batch( bora_flip_handle* hs, int n, float dt, int* status )
{
    if( n < 0 || ( n > 0 && ( !hs || !status ) ) ) return BORA_ERR_INVALID_ARG;
    if( n == 0 ) return BORA_OK;
    int dev = -1;
    for( int k = 0; k < n; ++k )
    {
        if( !hs[k] ) return BORA_ERR_INVALID_ARG;
        for( int q = 0; q < k; ++q )
            if( hs[q] == hs[k] ) return BORA_ERR_INVALID_ARG;
        if( dev >= 0 && hs[k]->device != dev ) return BORA_ERR_INVALID_ARG;
        dev = hs[k]->device;
        status[k] = BORA_OK;
    }
    struct Restore
    {
        bora_flip_handle* hs;
        int n;
        ~Restore()
        {
            for( int k = 0; k < n; ++k ) hs[k]->batching = false;
        }
    } restore{ hs, n };
    // the batched solve runs on the first simulation's stream; every simulation's own stages
    // run on its own stream, so those of different simulations overlap on the device
    bora_flip_sim* h0 = hs[0];
    cudaStream_t st = h0->st;
    const auto t0 = std::chrono::steady_clock::now();
    BORA_TRY( cudaEventRecord( h0->ev_step[0], st ) );
    // simulations the batched solve cannot take (the plain form, the warm start, no tiles, a
    // hierarchy the coarse cluster kernel does not fit) step on their own afterwards
    std::vector<int> pre, solo;
    for( int k = 0; k < n; ++k )
    {
        bora_flip_sim* s = hs[k];
        if( s->np == 0 ) continue;  // FLIPMethod.cu:179
        if( s->prm.solver != BORA_SOLVER_MIXED || s->prm.warm_start ) { solo.push_back( k ); continue; }
        s->batching = true;
        pre.push_back( k );
    }
    // the stages before the solve, each part issued for every simulation before the host
    // waits for any of them: tiles (-> tile count), sort (-> totals), P2G and the system
    std::vector<char> rebuilt( n, 0 );
    for( int k : pre )
        if( !hs[k]->sorted ) { status[k] = rebuild_tiles( hs[k] ); rebuilt[k] = 1; }
    for( int k : pre )
        if( rebuilt[k] && status[k] >= 0 )
        {
            status[k] = cuda_status( cudaStreamSynchronize( hs[k]->st ) );
            if( status[k] >= 0 ) status[k] = rebuild_sort( hs[k] );
        }
    std::vector<BatchMember> M;
    for( int k : pre )
    {
        bora_flip_sim* s = hs[k];
        if( rebuilt[k] && status[k] >= 0 )
        {
            status[k] = cuda_status( cudaStreamSynchronize( s->st ) );
            if( status[k] >= 0 ) status[k] = rebuild_finish( s );
        }
        if( status[k] >= 0 ) status[k] = stage_p2g( s );
        if( status[k] >= 0 ) status[k] = stage_build_system( s );
        if( status[k] < 0 ) continue;
        if( s->ntiles <= 0 || !s->mg_mid_on ) { s->batching = false; solo.push_back( k ); continue; }
        if( s != h0 )
        {
            BORA_TRY( cudaEventRecord( s->ev_join, s->st ) );
            BORA_TRY( cudaStreamWaitEvent( st, s->ev_join, 0 ) );
        }
        BatchMember b;
        b.s = s;
        b.row = (int)M.size();
        b.index = k;
        M.push_back( b );
    }
    const auto t1 = std::chrono::steady_clock::now();
    if( !M.empty() )
    {
        static BatchBuffers bb_cache[64];  // per device: the batch's argument arrays
        static std::mutex bb_mu;
        std::lock_guard<std::mutex> lk( bb_mu );
        BatchBuffers& bb = bb_cache[dev >= 0 && dev < 64 ? dev : 0];
        const int solve = batch_solve( M, st, bb, h0 );
        if( solve < 0 ) return solve;
    }
    const auto t2 = std::chrono::steady_clock::now();
    // the stages after the solve, back on each simulation's stream
    if( !M.empty() ) BORA_TRY( cudaEventRecord( h0->ev_join, st ) );
    for( BatchMember& b : M )
    {
        bora_flip_sim* s = b.s;
        if( s != h0 ) BORA_TRY( cudaStreamWaitEvent( s->st, h0->ev_join, 0 ) );
        int stt = stage_update_velocity( s );
        if( stt >= 0 ) stt = g2p_issue( s, dt );
        status[b.index] = stt;
    }
    for( BatchMember& b : M )
    {
        bora_flip_sim* s = b.s;
        if( status[b.index] < 0 ) continue;
        int stt = cuda_status( cudaStreamSynchronize( s->st ) );
        if( stt >= 0 ) stt = g2p_finish( s );
        status[b.index] = stt < 0 ? stt : s->last_status;
    }
    BORA_TRY( cudaEventRecord( h0->ev_step[1], st ) );
    BORA_TRY( cudaEventSynchronize( h0->ev_step[1] ) );
    float gms = 0.f;
    cudaEventElapsedTime( &gms, h0->ev_step[0], h0->ev_step[1] );
    bora_tune_resolve();
    const auto t3 = std::chrono::steady_clock::now();
    auto ms = []( std::chrono::steady_clock::time_point x, std::chrono::steady_clock::time_point y ) {
        return std::chrono::duration<double, std::milli>( y - x ).count();
    };
    for( BatchMember& b : M )
    {
        bora_flip_stats& o = b.s->stats;
        o.gpu_ms = gms;
        o.steps++;
        for( double& v : o.stage_ms ) v = 0.0;
        o.stage_ms[0] = ms( t0, t1 );  // the batch's stages before the solve
        o.stage_ms[3] = ms( t1, t2 );  // the batched solve
        o.stage_ms[5] = ms( t2, t3 );  // the stages after it
        o.stage_ms[7] = ms( t0, t3 );
        b.s->batching = false;
    }
    for( int k : solo )
    {
        hs[k]->batching = false;
        status[k] = bora_flip_step( hs[k], dt );
    }
    return BORA_OK;
}

int bora_flip_frame( bora_flip_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    const int st = bora_flip_step( s, s->prm.dt );
    if( st < 0 || !s->prm.post_process ) return st;
    BORA_TRYS( bora_flip_post_process( s ) );
    return st;
}

int bora_flip_post_process( bora_flip_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( s->np == 0 ) return BORA_OK;
    BORA_TRYS( post_process( s ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    s->prof_resolve();
    return BORA_OK;
}

int bora_flip_run_post_stage( bora_flip_handle s, int stage )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    int st = BORA_ERR_INVALID_ARG;
    switch( stage )
    {
        case BORA_POST_SPLAT: st = post_splat( s ); break;
        case BORA_POST_TANK_SCAN: st = post_tank_scan( s ); break;
        case BORA_POST_REDISTANCE: st = post_redistance( s ); break;
        case BORA_POST_ATTRIBUTES: st = post_attributes( s ); break;
        default: return BORA_ERR_INVALID_ARG;
    }
    s->warm_ready = false;  // post-processing uses pres as scratch
    s->pres_valid = false;
    BORA_TRYS( st );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    s->prof_resolve();
    return BORA_OK;
}

int bora_flip_get_particle_attributes( bora_flip_handle s, float* vorticity, float* curvature, int32_t* ids, size_t cap,
                                       size_t* n )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( cap < s->nlive && ( vorticity || curvature || ids ) ) return BORA_ERR_CAPACITY;
    if( n ) *n = s->nlive;
    if( s->np == 0 ) return BORA_OK;
    cudaStream_t st = s->st;
    const size_t np = s->np, nl = s->nlive;
    BORA_TRYS( ensure_scan_scratch( s, std::max( np + 1, std::max( s->ntv, s->cap_tiles * BORA_TILE_CELLS + 2 ) ) ) );
    BORA_TRY( grow( s->stage_out, nl * 12 + 64, false, st ) );
    float* ov = P<float>( s->stage_out );
    float* oc = ov + nl;
    int32_t* oid = reinterpret_cast<int32_t*>( oc + nl );
    BoraParticlesDev p = s->parts( s->cur );
    s->stats.kernel_launches += 4;
    k_live_flags<<<grid_blocks( np ), 256, 0, st>>>( np, p.id, P<uint32_t>( s->live_flag ) );
    bora_device_scan( P<uint32_t>( s->live_flag ), P<uint32_t>( s->live_flag ), np, P<uint32_t>( s->scan_scratch ),
                   P<uint32_t>( s->counters ) + 4, st );
    k_gather_attrs<<<grid_blocks( np ), 256, 0, st>>>( np, p, P<uint32_t>( s->live_flag ), ov, oc, oid );
    BORA_TRYS( check_launch( s ) );
    if( vorticity ) BORA_TRY( cudaMemcpyAsync( vorticity, ov, nl * 4, cudaMemcpyDeviceToHost, st ) );
    if( curvature ) BORA_TRY( cudaMemcpyAsync( curvature, oc, nl * 4, cudaMemcpyDeviceToHost, st ) );
    if( ids ) BORA_TRY( cudaMemcpyAsync( ids, oid, nl * 4, cudaMemcpyDeviceToHost, st ) );
    BORA_TRY( cudaStreamSynchronize( st ) );
    return BORA_OK;
}

int bora_flip_set_particle_attributes( bora_flip_handle s, const float* vorticity, const float* curvature, size_t n )
{
    if( !s || n != s->nlive ) return BORA_ERR_INVALID_ARG;
    BORA_TRYS( ensure_attrs( s ) );
    if( s->np == 0 ) return BORA_OK;
    cudaStream_t st = s->st;
    const size_t np = s->np;
    BORA_TRYS( ensure_scan_scratch( s, std::max( np + 1, std::max( s->ntv, s->cap_tiles * BORA_TILE_CELLS + 2 ) ) ) );
    BORA_TRY( grow( s->stage_in, n * 8 + 64, false, st ) );
    float* iv = P<float>( s->stage_in );
    float* ic = iv + n;
    if( vorticity ) BORA_TRY( cudaMemcpyAsync( iv, vorticity, n * 4, cudaMemcpyHostToDevice, st ) );
    else BORA_TRY( cudaMemsetAsync( iv, 0, n * 4, st ) );
    if( curvature ) BORA_TRY( cudaMemcpyAsync( ic, curvature, n * 4, cudaMemcpyHostToDevice, st ) );
    else BORA_TRY( cudaMemsetAsync( ic, 0, n * 4, st ) );
    BoraParticlesDev p = s->parts( s->cur );
    s->stats.kernel_launches += 4;
    k_live_flags<<<grid_blocks( np ), 256, 0, st>>>( np, p.id, P<uint32_t>( s->live_flag ) );
    bora_device_scan( P<uint32_t>( s->live_flag ), P<uint32_t>( s->live_flag ), np, P<uint32_t>( s->scan_scratch ),
                   P<uint32_t>( s->counters ) + 4, st );
    k_scatter_attrs<<<grid_blocks( np ), 256, 0, st>>>( np, p, P<uint32_t>( s->live_flag ), iv, ic );
    BORA_TRYS( check_launch( s ) );
    BORA_TRY( cudaStreamSynchronize( st ) );  // the caller may free its buffers on return
    return BORA_OK;
}

int bora_flip_num_particles( bora_flip_handle s, size_t* n )
{
    if( !s || !n ) return BORA_ERR_INVALID_ARG;
    *n = s->nlive;
    return BORA_OK;
}

int bora_flip_get_particles( bora_flip_handle s, float* pos, float* vel, float* adjacency, int32_t* ids, size_t cap,
                             size_t* n, int space )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( cap < s->nlive && ( pos || vel || adjacency || ids ) ) return BORA_ERR_CAPACITY;
    if( n ) *n = s->nlive;
    if( s->np == 0 ) return BORA_OK;
    cudaStream_t st = s->st;
    const size_t np = s->np;
    BORA_TRYS( ensure_scan_scratch( s, std::max( np + 1, std::max( s->ntv, s->cap_tiles * BORA_TILE_CELLS + 2 ) ) ) );
    BORA_TRY( grow( s->stage_out, s->nlive * 32 + 64, false, st ) );
    BoraParticlesDev p = s->parts( s->cur );
    s->stats.kernel_launches += 5;
    k_live_flags<<<grid_blocks( np ), 256, 0, st>>>( np, p.id, P<uint32_t>( s->live_flag ) );
    bora_device_scan( P<uint32_t>( s->live_flag ), P<uint32_t>( s->live_flag ), np, P<uint32_t>( s->scan_scratch ),
                   P<uint32_t>( s->counters ) + 4, st );
    const size_t nl = s->nlive;
    float* opos = P<float>( s->stage_out );
    float* ovel = opos + 3 * nl;
    float* oadj = ovel + 3 * nl;
    int32_t* oid = reinterpret_cast<int32_t*>( oadj + nl );
    const float3 tr = make_float3( s->translate[0], s->translate[1], s->translate[2] );
    const float3 sc = make_float3( s->scale[0], s->scale[1], s->scale[2] );
    k_gather_live<<<grid_blocks( np ), 256, 0, st>>>( np, p, P<float>( s->adj ), P<uint32_t>( s->live_flag ), space, tr, sc,
                                                      opos, ovel, oadj, oid );
    BORA_TRYS( check_launch( s ) );
    if( pos ) BORA_TRY( cudaMemcpyAsync( pos, opos, nl * 12, cudaMemcpyDeviceToHost, st ) );
    if( vel ) BORA_TRY( cudaMemcpyAsync( vel, ovel, nl * 12, cudaMemcpyDeviceToHost, st ) );
    if( adjacency ) BORA_TRY( cudaMemcpyAsync( adjacency, oadj, nl * 4, cudaMemcpyDeviceToHost, st ) );
    if( ids ) BORA_TRY( cudaMemcpyAsync( ids, oid, nl * 4, cudaMemcpyDeviceToHost, st ) );
    BORA_TRY( cudaStreamSynchronize( st ) );
    return BORA_OK;
}

int bora_flip_export_begin( bora_flip_handle s, float* pos, float* vel, float* vorticity, float* curvature, int32_t* ids,
                            size_t cap, int space, size_t* n )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( cap < s->nlive && ( pos || vel || vorticity || curvature || ids ) ) return BORA_ERR_CAPACITY;
    if( n ) *n = s->nlive;
    if( !s->st_copy )
    {
        BORA_TRY( cudaStreamCreateWithFlags( &s->st_copy, cudaStreamNonBlocking ) );
        BORA_TRY( cudaEventCreateWithFlags( &s->ev_gathered, cudaEventDisableTiming ) );
        BORA_TRY( cudaEventCreateWithFlags( &s->ev_copied, cudaEventDisableTiming ) );
    }
    if( s->exporting ) BORA_TRY( cudaEventSynchronize( s->ev_copied ) );  // one export at a time
    s->exporting = false;
    if( s->np == 0 || s->nlive == 0 ) return BORA_OK;
    cudaStream_t st = s->st;
    const size_t np = s->np, nl = s->nlive;
    BORA_TRYS( ensure_scan_scratch( s, std::max( np + 1, std::max( s->ntv, s->cap_tiles * BORA_TILE_CELLS + 2 ) ) ) );
    BORA_TRY( grow( s->exp_buf, nl * 40 + 64, false, st ) );
    float* opos = P<float>( s->exp_buf );
    float* ovel = opos + 3 * nl;
    float* oadj = ovel + 3 * nl;
    float* ovort = oadj + nl;
    float* ocurv = ovort + nl;
    int32_t* oid = reinterpret_cast<int32_t*>( ocurv + nl );
    BoraParticlesDev p = s->parts( s->cur );
    const float3 tr = make_float3( s->translate[0], s->translate[1], s->translate[2] );
    const float3 sc = make_float3( s->scale[0], s->scale[1], s->scale[2] );
    s->stats.kernel_launches += 5;
    k_live_flags<<<grid_blocks( np ), 256, 0, st>>>( np, p.id, P<uint32_t>( s->live_flag ) );
    bora_device_scan( P<uint32_t>( s->live_flag ), P<uint32_t>( s->live_flag ), np, P<uint32_t>( s->scan_scratch ),
                   P<uint32_t>( s->counters ) + 4, st );
    k_gather_live<<<grid_blocks( np ), 256, 0, st>>>( np, p, P<float>( s->adj ), P<uint32_t>( s->live_flag ), space, tr, sc,
                                                      opos, ovel, oadj, oid );
    k_gather_attrs<<<grid_blocks( np ), 256, 0, st>>>( np, p, P<uint32_t>( s->live_flag ), ovort, ocurv, oid );
    BORA_TRYS( check_launch( s ) );
    BORA_TRY( cudaEventRecord( s->ev_gathered, st ) );
    cudaStream_t cs = s->st_copy;
    BORA_TRY( cudaStreamWaitEvent( cs, s->ev_gathered, 0 ) );
    if( pos ) BORA_TRY( cudaMemcpyAsync( pos, opos, nl * 12, cudaMemcpyDeviceToHost, cs ) );
    if( vel ) BORA_TRY( cudaMemcpyAsync( vel, ovel, nl * 12, cudaMemcpyDeviceToHost, cs ) );
    if( vorticity ) BORA_TRY( cudaMemcpyAsync( vorticity, ovort, nl * 4, cudaMemcpyDeviceToHost, cs ) );
    if( curvature ) BORA_TRY( cudaMemcpyAsync( curvature, ocurv, nl * 4, cudaMemcpyDeviceToHost, cs ) );
    if( ids ) BORA_TRY( cudaMemcpyAsync( ids, oid, nl * 4, cudaMemcpyDeviceToHost, cs ) );
    BORA_TRY( cudaEventRecord( s->ev_copied, cs ) );
    s->exporting = true;  // the next export waits for ev_copied before it gathers into exp_buf
    return BORA_OK;
}

int bora_flip_export_wait( bora_flip_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    if( s->exporting ) BORA_TRY( cudaEventSynchronize( s->ev_copied ) );
    s->exporting = false;
    return BORA_OK;
}

int bora_flip_frame_info( bora_flip_handle s, bora_frame_info* o )
{
    if( !s || !o ) return BORA_ERR_INVALID_ARG;
    o->nx = s->g.nx; o->ny = s->g.ny; o->nz = s->g.nz;
    o->tx = s->g.tx; o->ty = s->g.ty; o->tz = s->g.tz;
    o->tile = BORA_TILE;
    o->active_tiles = s->ntiles;
    for( int a = 0; a < 3; ++a ) { o->translate[a] = s->translate[a]; o->scale[a] = s->scale[a]; o->voxel_gravity[a] = s->g.gravity[a]; }
    o->voxel_wall_level = s->g.voxel_wall;
    return BORA_OK;
}

int bora_flip_get_tiles( bora_flip_handle s, int32_t* ijk, size_t cap_tiles )
{
    if( !s || ( !ijk && s->ntiles ) ) return BORA_ERR_INVALID_ARG;
    if( cap_tiles < (size_t)s->ntiles ) return BORA_ERR_CAPACITY;
    std::vector<int32_t> lin( (size_t)s->ntiles );
    if( s->ntiles )
    {
        BORA_TRY( cudaMemcpyAsync( lin.data(), s->tile_of.p, lin.size() * 4, cudaMemcpyDeviceToHost, s->st ) );
        BORA_TRY( cudaStreamSynchronize( s->st ) );
    }
    for( size_t t = 0; t < lin.size(); ++t )
    {
        ijk[3 * t] = lin[t] % s->g.tx;
        ijk[3 * t + 1] = ( lin[t] / s->g.tx ) % s->g.ty;
        ijk[3 * t + 2] = lin[t] / ( s->g.tx * s->g.ty );
    }
    return BORA_OK;
}

// The surface field's background after post-processing (Rasterization::ReinitializeSurface,
// Rasterization.cu:422), in voxel units.
constexpr float kSurfaceBackground = 10.f;

int bora_flip_export_vdb( bora_flip_handle s, int which, int32_t* origins, uint64_t* masks, float* values,
                          size_t cap_leaves, size_t* nleaves, float* transform, float* background )
{
    if( !s || !nleaves || ( which != BORA_VDB_SURFACE && which != BORA_VDB_VELOCITY ) ) return BORA_ERR_INVALID_ARG;
    *nleaves = 0;
    const float dx = s->scale[0];
    if( transform )  // FieldCast.h: linear transform of voxel size dx, translated by min + dx/2
    {
        transform[0] = dx;
        for( int a = 0; a < 3; ++a ) transform[1 + a] = s->translate[a] + dx * 0.5f;
    }
    const float bg = which == BORA_VDB_SURFACE ? kSurfaceBackground : 0.f;
    if( background ) *background = bg * dx;
    // candidate leaves: the active tiles, then (surface, water tank) the band's other tiles
    const size_t nt = (size_t)s->ntiles;
    std::vector<int32_t> lin( nt );
    if( nt )
    {
        BORA_TRY( cudaMemcpyAsync( lin.data(), s->tile_of.p, nt * 4, cudaMemcpyDeviceToHost, s->st ) );
        BORA_TRY( cudaStreamSynchronize( s->st ) );
    }
    const int tx = s->g.tx, ty = s->g.ty, tz = s->g.tz;
    std::vector<int32_t> leaf;  // per leaf: i, j, k origin, slot
    leaf.reserve( nt * 4 );
    for( size_t t = 0; t < nt; ++t )
    {
        leaf.push_back( 8 * ( lin[t] % tx ) );
        leaf.push_back( 8 * ( ( lin[t] / tx ) % ty ) );
        leaf.push_back( 8 * ( lin[t] / ( tx * ty ) ) );
        leaf.push_back( (int32_t)t );
    }
    const bool tank = which == BORA_VDB_SURFACE && s->prm.enable_water_tank;
    if( tank )
    {
        std::vector<int32_t> band;
        bora_vdb_band_tiles( s->g, s->scale, s->translate, s->prm.wall_level, band );
        std::vector<uint8_t> active( (size_t)tx * ty * tz, 0 );
        for( size_t t = 0; t < nt; ++t ) active[(size_t)lin[t]] = 1;
        for( size_t b = 0; b < band.size(); b += 3 )
        {
            const int ti = band[b], tj = band[b + 1], tk = band[b + 2];
            const bool inside = ti >= 0 && tj >= 0 && tk >= 0 && ti < tx && tj < ty && tk < tz;
            if( inside && active[( (size_t)tk * ty + tj ) * tx + ti] ) continue;
            leaf.push_back( 8 * ti );
            leaf.push_back( 8 * tj );
            leaf.push_back( 8 * tk );
            leaf.push_back( -1 );
        }
    }
    const size_t nl = leaf.size() / 4;
    if( nl == 0 ) return BORA_OK;
    const size_t comps = which == BORA_VDB_SURFACE ? 1 : 3;
    BORA_TRY( grow( s->vdb_leaf, nl * 16, false, s->st ) );
    BORA_TRY( grow( s->vdb_mask, nl * 64, false, s->st ) );
    BORA_TRY( grow( s->vdb_val, nl * 512 * comps * 4, false, s->st ) );
    std::vector<int32_t> ijk( nl * 3 ), slot( nl );
    for( size_t l = 0; l < nl; ++l )
    {
        for( int a = 0; a < 3; ++a ) ijk[3 * l + a] = leaf[4 * l + a];
        slot[l] = leaf[4 * l + 3];
    }
    int32_t* d_ijk = P<int32_t>( s->vdb_leaf );
    int32_t* d_slot = d_ijk + 3 * nl;
    BORA_TRY( cudaMemcpyAsync( d_ijk, ijk.data(), nl * 12, cudaMemcpyHostToDevice, s->st ) );
    BORA_TRY( cudaMemcpyAsync( d_slot, slot.data(), nl * 4, cudaMemcpyHostToDevice, s->st ) );
    if( which == BORA_VDB_SURFACE )
        bora_launch_vdb_surface( s->g, s->scale, s->translate, (int)nl, d_ijk, d_slot, P<float>( s->surf ), bg, tank ? 1 : 0,
                                 s->prm.wall_level, P<uint64_t>( s->vdb_mask ), P<float>( s->vdb_val ), s->st );
    else
        bora_launch_vdb_velocity( s->g, s->scale, (int)nl, d_ijk, d_slot, P<float>( s->vx ), P<float>( s->vy ),
                                  P<float>( s->vz ), P<uint64_t>( s->vdb_mask ), P<float>( s->vdb_val ), s->st );
    s->stats.kernel_launches += 1;
    BORA_TRYS( check_launch( s ) );
    std::vector<uint64_t> m( nl * 8 );
    BORA_TRY( cudaMemcpyAsync( m.data(), s->vdb_mask.p, nl * 64, cudaMemcpyDeviceToHost, s->st ) );
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    // leaves without an active voxel are not written (OpenVDB creates no leaf for them)
    std::vector<size_t> keep;
    keep.reserve( nl );
    for( size_t l = 0; l < nl; ++l )
    {
        uint64_t any = 0;
        for( int w = 0; w < 8; ++w ) any |= m[8 * l + w];
        if( any ) keep.push_back( l );
    }
    *nleaves = keep.size();
    if( !origins ) return BORA_OK;
    if( cap_leaves < keep.size() || !masks || !values ) return cap_leaves < keep.size() ? BORA_ERR_CAPACITY : BORA_ERR_INVALID_ARG;
    const size_t per = 512 * comps;
    for( size_t q = 0; q < keep.size(); ++q )
    {
        const size_t l = keep[q];
        for( int a = 0; a < 3; ++a ) origins[3 * q + a] = ijk[3 * l + a];
        for( int w = 0; w < 8; ++w ) masks[8 * q + w] = m[8 * l + w];
        BORA_TRY( cudaMemcpyAsync( values + q * per, P<float>( s->vdb_val ) + l * per, per * 4, cudaMemcpyDeviceToHost,
                                   s->st ) );
    }
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    return BORA_OK;
}

static int field_bufs( bora_flip_handle s, int which, DevBuf** b, int* ncomp, size_t* esize )
{
    *ncomp = 1;
    *esize = 4;
    switch( which )
    {
        case BORA_FIELD_MASS: b[0] = &s->mass; return BORA_OK;
        case BORA_FIELD_SURF: b[0] = &s->surf; return BORA_OK;
        case BORA_FIELD_PRES: b[0] = &s->pres; return BORA_OK;
        case BORA_FIELD_VELO: b[0] = &s->vx; b[1] = &s->vy; b[2] = &s->vz; *ncomp = 3; return BORA_OK;
        case BORA_FIELD_COMP: b[0] = &s->cx; b[1] = &s->cy; b[2] = &s->cz; *ncomp = 3; return BORA_OK;
        case BORA_FIELD_FLAG: b[0] = &s->flag; *esize = 1; return BORA_OK;
        case BORA_FIELD_RHS: b[0] = &s->rhs; return BORA_OK;
        case BORA_FIELD_CODE: b[0] = &s->code; *esize = 2; return BORA_OK;
        default: return BORA_ERR_INVALID_ARG;
    }
}

int bora_flip_get_field( bora_flip_handle s, int which, void* out, size_t bytes )
{
    if( !s || !out ) return BORA_ERR_INVALID_ARG;
    DevBuf* b[3];
    int nc;
    size_t es;
    BORA_TRYS( field_bufs( s, which, b, &nc, &es ) );
    const size_t ncell = (size_t)s->ntiles * BORA_TILE_CELLS;
    if( bytes < ncell * nc * es ) return BORA_ERR_CAPACITY;
    if( nc == 1 )
    {
        BORA_TRY( cudaMemcpyAsync( out, b[0]->p, ncell * es, cudaMemcpyDeviceToHost, s->st ) );
        BORA_TRY( cudaStreamSynchronize( s->st ) );
        return BORA_OK;
    }
    std::vector<float> tmp( ncell );
    float* o = (float*)out;
    for( int c = 0; c < nc; ++c )
    {
        BORA_TRY( cudaMemcpyAsync( tmp.data(), b[c]->p, ncell * 4, cudaMemcpyDeviceToHost, s->st ) );
        BORA_TRY( cudaStreamSynchronize( s->st ) );
        for( size_t i = 0; i < ncell; ++i ) o[3 * i + c] = tmp[i];
    }
    return BORA_OK;
}

int bora_flip_set_field( bora_flip_handle s, int which, const void* in, size_t bytes )
{
    if( !s || !in ) return BORA_ERR_INVALID_ARG;
    DevBuf* b[3];
    int nc;
    size_t es;
    BORA_TRYS( field_bufs( s, which, b, &nc, &es ) );
    const size_t ncell = (size_t)s->ntiles * BORA_TILE_CELLS;
    if( bytes < ncell * nc * es ) return BORA_ERR_CAPACITY;
    if( nc == 1 )
    {
        BORA_TRY( cudaMemcpyAsync( b[0]->p, in, ncell * es, cudaMemcpyHostToDevice, s->st ) );
        BORA_TRY( cudaStreamSynchronize( s->st ) );
        return BORA_OK;
    }
    std::vector<float> tmp( ncell );
    const float* src = (const float*)in;
    for( int c = 0; c < nc; ++c )
    {
        for( size_t i = 0; i < ncell; ++i ) tmp[i] = src[3 * i + c];
        BORA_TRY( cudaMemcpyAsync( b[c]->p, tmp.data(), ncell * 4, cudaMemcpyHostToDevice, s->st ) );
        BORA_TRY( cudaStreamSynchronize( s->st ) );
    }
    return BORA_OK;
}

int bora_flip_get_stats( bora_flip_handle s, bora_flip_stats* o )
{
    if( !s || !o ) return BORA_ERR_INVALID_ARG;
    *o = s->stats;
    o->num_particles = s->nlive;
    uint64_t bytes = 0;
    for_each_buffer( s, [&]( DevBuf& b ) { bytes += b.bytes; } );
    o->device_bytes = bytes;
    return BORA_OK;
}

int bora_flip_set_fault( bora_flip_handle s, int fault )
{
    if( !s || ( fault != BORA_FAULT_NONE && fault != BORA_FAULT_BARRIER ) ) return BORA_ERR_INVALID_ARG;
    s->fault = fault;
    return BORA_OK;
}

int bora_flip_set_profiling( bora_flip_handle s, uint32_t mask )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    s->prof_resolve();
    s->prof_mask = mask;
    for( int c = 0; c < BORA_KERNEL_CLASSES; ++c ) { s->kt_ms[c] = 0.0; s->kt_n[c] = 0; s->prof_seen[c] = 0; }
    return BORA_OK;
}

int bora_flip_set_profiling_sampling( bora_flip_handle s, uint32_t every )
{
    if( !s || every == 0 ) return BORA_ERR_INVALID_ARG;
    s->prof_every = every;
    for( int c = 0; c < BORA_KERNEL_CLASSES; ++c ) s->prof_seen[c] = 0;
    return BORA_OK;
}

int bora_flip_get_kernel_times( bora_flip_handle s, double* ms, uint64_t* launches, int n )
{
    if( !s || n < 0 || n > BORA_KERNEL_CLASSES ) return BORA_ERR_INVALID_ARG;
    BORA_TRY( cudaStreamSynchronize( s->st ) );
    s->prof_resolve();
    for( int c = 0; c < n; ++c )
    {
        if( ms ) ms[c] = s->kt_ms[c];
        if( launches ) launches[c] = s->kt_n[c];
    }
    return BORA_OK;
}

const char* bora_flip_status_string( int st )
{
    switch( st )
    {
        case BORA_OK: return "ok";
        case BORA_ERR_INVALID_ARG: return "invalid argument";
        case BORA_ERR_OUT_OF_MEMORY: return "out of device memory";
        case BORA_ERR_CUDA: return "CUDA error";
        case BORA_ERR_NO_DEVICE: return "no CUDA device";
        case BORA_ERR_INTERNAL: return "internal consistency check failed";
        case BORA_ERR_CAPACITY: return "buffer too small or size limit exceeded";
        case BORA_WARN_NOT_CONVERGED: return "pressure solve stopped before reaching its tolerance";
        default: return "unknown status";
    }
}

}  // extern "C"
