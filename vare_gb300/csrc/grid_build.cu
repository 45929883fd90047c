// Sparse-grid rebuild on the device: particle binning, tile activation, the tile table
// and the per-step counting sort of particles by dual cell.
//
// Replaces SparseFrame::buildFromPoints (base/source/SparseFrame.cu:83-155), whose
// per-particle 27-way atomicAdd marks a dense tile-count table and whose serial host
// loop compacts it, and SparseField::build (SparseField.h:221-226).
//
// Activation rule at the 8^3 tile edge: tile T is active iff some particle's tile
// (max(int(p)/8, 0), clamped to the table) lies within one tile of T in every axis.
// Active tiles take slots in linear tile order (x fastest), as the reference numbers
// its active tiles. The reference's unclamped lower loop bound (SparseFrame.cu:105-107)
// that wraps index -1 into the previous row is not reproduced.
#include "bora_internal.h"

namespace {

constexpr int kThreads = 256;

inline int grid_for( size_t n, int threads = kThreads )
{
    const size_t b = ( n + threads - 1 ) / threads;
    return (int)( b < 152 * 16 ? ( b > 0 ? b : 1 ) : 152 * 16 );  // grid-stride loops: 16 blocks per SM
}

__device__ inline uint32_t bin_one( const BoraGridDev& g, int32_t id, float x, float y, float z,
                                    uint8_t* __restrict__ tile_flag )
{
    return bora_bin_key( g.nx, g.ny, g.nz, g.tx, g.ty, g.tz, id, x, y, z, tile_flag );
}

// Four particles per thread with 16-byte loads and stores (the arrays are 256-byte
// aligned), the last n % 4 one by one.
__global__ void k_bin( BoraGridDev g, BoraParticlesDev p, size_t n, uint32_t* __restrict__ vkey,
                       uint8_t* __restrict__ tile_flag )
{
    const size_t n4 = n / 4;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for( size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n4; v += stride )
    {
        const int4 id = reinterpret_cast<const int4*>( p.id )[v];
        const float4 x = reinterpret_cast<const float4*>( p.px )[v];
        const float4 y = reinterpret_cast<const float4*>( p.py )[v];
        const float4 z = reinterpret_cast<const float4*>( p.pz )[v];
        uint4 k;
        k.x = bin_one( g, id.x, x.x, y.x, z.x, tile_flag );
        k.y = bin_one( g, id.y, x.y, y.y, z.y, tile_flag );
        k.z = bin_one( g, id.z, x.z, y.z, z.z, tile_flag );
        k.w = bin_one( g, id.w, x.w, y.w, z.w, tile_flag );
        reinterpret_cast<uint4*>( vkey )[v] = k;
    }
    for( size_t i = n4 * 4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride )
        vkey[i] = bin_one( g, p.id[i], p.px[i], p.py[i], p.pz[i], tile_flag );
}

__global__ void k_activate( BoraGridDev g, const uint8_t* __restrict__ tile_flag, uint32_t* __restrict__ act, int tank_rows )
{
    const size_t ntv = (size_t)g.tx * g.ty * g.tz;
    for( size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < ntv; t += (size_t)gridDim.x * blockDim.x )
    {
        const int ti = (int)( t % g.tx ), tj = (int)( ( t / g.tx ) % g.ty ), tk = (int)( t / ( (size_t)g.tx * g.ty ) );
        uint32_t a = tj < tank_rows ? 1u : 0u;  // the water tank keeps its rows active (SparseFrame.cu:119-129)
        for( int dk = -1; dk <= 1 && !a; ++dk )
        {
            const int k = tk + dk;
            if( k < 0 || k >= g.tz ) continue;
            for( int dj = -1; dj <= 1 && !a; ++dj )
            {
                const int j = tj + dj;
                if( j < 0 || j >= g.ty ) continue;
                for( int di = -1; di <= 1; ++di )
                {
                    const int i = ti + di;
                    if( i < 0 || i >= g.tx ) continue;
                    if( tile_flag[( (size_t)k * g.ty + j ) * g.tx + i] ) { a = 1; break; }
                }
            }
        }
        act[t] = a;
    }
}

__global__ void k_tile_assign( size_t ntv, const uint32_t* __restrict__ act, const uint32_t* __restrict__ excl,
                               int32_t* __restrict__ slot_of, int32_t* __restrict__ tile_of )
{
    for( size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < ntv; t += (size_t)gridDim.x * blockDim.x )
    {
        if( act[t] )
        {
            const int32_t s = (int32_t)excl[t];
            slot_of[t] = s;
            tile_of[s] = (int32_t)t;
        }
        else
        {
            slot_of[t] = -1;
        }
    }
}

__global__ void k_tile_nbrs( BoraGridDev g, int ntiles, const int32_t* __restrict__ slot_of,
                             const int32_t* __restrict__ tile_of, int32_t* __restrict__ nbr )
{
    const size_t total = (size_t)ntiles * 27;
    for( size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x )
    {
        const int s = (int)( q / 27 ), d = (int)( q % 27 );
        const int t = tile_of[s];
        const int ti = t % g.tx, tj = ( t / g.tx ) % g.ty, tk = t / ( g.tx * g.ty );
        const int i = ti + d % 3 - 1, j = tj + ( d / 3 ) % 3 - 1, k = tk + d / 9 - 1;
        int32_t v = -1;
        if( i >= 0 && i < g.tx && j >= 0 && j < g.ty && k >= 0 && k < g.tz )
            v = slot_of[( (size_t)k * g.ty + j ) * g.tx + i];
        nbr[q] = v;
    }
}

// Per-dual-cell particle histogram; one atomic per distinct key per warp.
__global__ void k_hist( size_t n, const uint32_t* __restrict__ vkey, const int32_t* __restrict__ slot_of,
                        uint32_t outside_key, uint32_t* __restrict__ key, uint32_t* __restrict__ count,
                        uint32_t* __restrict__ err )
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t nround = ( n + 31 ) & ~(size_t)31;
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nround; i += stride )
    {
        uint32_t k = BORA_DEAD_KEY;
        if( i < n )
        {
            const uint32_t v = vkey[i];
            if( v == BORA_DEAD_KEY - 1 ) k = outside_key;
            else if( v != BORA_DEAD_KEY )
            {
                const int32_t s = slot_of[v / BORA_TILE_CELLS];
                if( s >= 0 ) k = (uint32_t)s * BORA_TILE_CELLS + ( v % BORA_TILE_CELLS );
                else { k = outside_key; atomicAdd( err, 1u ); }  // cannot happen: dual cells lie in active tiles
            }
            key[i] = k;
        }
        const uint32_t peers = __match_any_sync( 0xffffffffu, k );
        const int lane = threadIdx.x & 31;
        if( k != BORA_DEAD_KEY && lane == __ffs( peers ) - 1 ) atomicAdd( &count[k], (uint32_t)__popc( peers ) );
    }
}

// Counting-sort scatter: every live particle gets a slot inside its dual cell's range.
// The per-key counters are consumed (they are all zero afterwards, ready for the next
// histogram).
__global__ void k_scatter( size_t n, const uint32_t* __restrict__ key, const uint32_t* __restrict__ start,
                           uint32_t* __restrict__ count, uint32_t* __restrict__ idx )
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t nround = ( n + 31 ) & ~(size_t)31;
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nround; i += stride )
    {
        const uint32_t k = i < n ? key[i] : BORA_DEAD_KEY;
        const uint32_t peers = __match_any_sync( 0xffffffffu, k );
        const int lane = threadIdx.x & 31;
        const int leader = __ffs( peers ) - 1;
        uint32_t top = 0;
        if( k != BORA_DEAD_KEY && lane == leader ) top = atomicSub( &count[k], (uint32_t)__popc( peers ) );
        top = __shfl_sync( 0xffffffffu, top, leader );
        if( k != BORA_DEAD_KEY )
        {
            const uint32_t rank = (uint32_t)__popc( peers & ( ( 1u << lane ) - 1u ) );
            const uint32_t dst = start[k] + top - (uint32_t)__popc( peers ) + rank;
            idx[dst] = (uint32_t)i;
        }
    }
}

// Order the particles of every dual cell by their source index (insertion sort of each
// bin of the permutation, in place). The counting-sort scatter fills a bin in atomic
// arrival order; this makes the order - and so every floating-point sum over a bin - a
// function of the input only. Bins larger than `max_bin` (possible only for the bin of
// particles outside the grid) keep their arrival order.
// Batcher's odd-even merge sort (Knuth, TAOCP vol. 3, 5.3.4) on 16 inputs: comparator pairs
// (a, b), a < b, in the order applied.
constexpr int kSortNet16 = 63;
__constant__ const int8_t kNet16[2 * kSortNet16] = {
    0, 1, 2, 3, 0, 2, 1, 3, 1, 2, 4, 5, 6, 7, 4, 6, 5, 7, 5, 6, 0, 4, 2, 6, 2, 4, 1, 5, 3, 7, 3, 5,
    1, 2, 3, 4, 5, 6, 8, 9, 10, 11, 8, 10, 9, 11, 9, 10, 12, 13, 14, 15, 12, 14, 13, 15, 13, 14, 8, 12, 10, 14,
    10, 12, 9, 13, 11, 15, 11, 13, 9, 10, 11, 12, 13, 14, 0, 8, 4, 12, 4, 8, 2, 10, 6, 14, 6, 10, 2, 4, 6, 8,
    10, 12, 1, 9, 5, 13, 5, 9, 3, 11, 7, 15, 7, 11, 3, 5, 7, 9, 11, 13, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12,
    13, 14 };

__global__ void k_order_bins( size_t nbins, const uint32_t* __restrict__ start, uint32_t* __restrict__ idx,
                              uint32_t max_bin )
{
    constexpr int kReg = 16;  // bins up to this size are sorted in registers
    for( size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x; b < nbins; b += (size_t)gridDim.x * blockDim.x )
    {
        const uint32_t q0 = start[b], q1 = start[b + 1];
        const uint32_t n = q1 - q0;
        if( n < 2 || n > max_bin ) continue;
        if( n <= kReg )
        {
            uint32_t v[kReg];
#pragma unroll
            for( int a = 0; a < kReg; ++a ) v[a] = a < (int)n ? idx[q0 + a] : 0xFFFFFFFFu;
            bool sorted = true;
#pragma unroll
            for( int a = 1; a < kReg; ++a ) sorted = sorted && v[a - 1] < v[a];  // padding sorts last
            if( sorted ) continue;
            // Batcher's odd-even merge sorting network for 16 inputs (63 comparators; indices
            // are distinct)
#pragma unroll
            for( int c = 0; c < kSortNet16; ++c )
            {
                const int a = kNet16[2 * c], b = kNet16[2 * c + 1];
                const uint32_t lo = min( v[a], v[b] ), hi = max( v[a], v[b] );
                v[a] = lo;
                v[b] = hi;
            }
#pragma unroll
            for( int a = 0; a < kReg; ++a )
                if( a < (int)n ) idx[q0 + a] = v[a];
            continue;
        }
        for( uint32_t q = q0 + 1; q < q1; ++q )
        {
            const uint32_t v = idx[q];
            uint32_t r = q;
            while( r > q0 && idx[r - 1] > v ) { idx[r] = idx[r - 1]; --r; }
            idx[r] = v;
        }
    }
}

// Host AoS (x,y,z) particles -> device SoA, with the world->voxel transform
// (Grid::voxelPoint / voxelVector, base/header/Grid.h:446-458) when space == 0.
__global__ void k_to_soa( size_t n, const float* __restrict__ pos, const float* __restrict__ vel, int space,
                          float3 tr, float3 sc, BoraParticlesDev p, size_t offset, int32_t first_id )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x )
    {
        float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        float u = vel ? vel[3 * i] : 0.f, v = vel ? vel[3 * i + 1] : 0.f, w = vel ? vel[3 * i + 2] : 0.f;
        if( space == 0 )
        {
            x = ( x - tr.x ) / sc.x; y = ( y - tr.y ) / sc.y; z = ( z - tr.z ) / sc.z;
            u = u / sc.x; v = v / sc.y; w = w / sc.z;
        }
        const size_t o = offset + i;
        p.px[o] = x; p.py[o] = y; p.pz[o] = z;
        p.vx[o] = u; p.vy[o] = v; p.vz[o] = w;
        p.id[o] = first_id + (int32_t)i;
    }
}

// Random.h:30-38, Rand( seed, 0, 1 ): an integer hash of the seed scaled to [0, 1].
__device__ inline float bora_rand01( unsigned int seed )
{
    unsigned int i = ( seed ^ 12345391u ) * 2654435769u;
    i ^= ( i << 6 ) ^ ( i >> 26 );
    i *= 2654435769u;
    i += ( i << 5 ) ^ ( i >> 12 );
    return ( 1.0f - 0.0f ) * (float)i / 4294967296.0f + 0.0f;  // (float)UINT_MAX rounds to 2^32
}

// FLIPMethod::fillWaterTank (FLIPMethod.cu:407-478), one thread per cell below the wall
// level: two jittered particles, the cell centre, and `per_cell` more in the 4-cell band
// under the wall. COUNT pass: particles per cell; write pass: each cell's particles at its
// prefix offset, so the order is the reference's (k, j, i) loop order. Positions take the
// reference's round trip through world space (Grid::worldPoint, then particlesToVoxel).
template <bool WRITE>
__global__ void k_tank( BoraGridDev g, int hh, float wall, int per_cell, float3 tr, float3 sc, uint32_t* count,
                        const uint32_t* __restrict__ offset, BoraParticlesDev p, size_t base, int32_t first_id )
{
    const size_t ncell = (size_t)g.nx * hh * g.nz;
    for( size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x )
    {
        const int i = (int)( c % g.nx ), j = (int)( ( c / g.nx ) % hh ), k = (int)( c / ( (size_t)g.nx * hh ) );
        const unsigned ui = (unsigned)i, uj = (unsigned)j, uk = (unsigned)k;
        const float cx = i + .5f, cy = j + .5f, cz = k + .5f;
        uint32_t m = 0;
        const size_t o = WRITE ? base + offset[c] : 0;
        auto emit = [&]( float x, float y, float z ) {
            if( !( y <= wall ) ) return;
            if( WRITE )
            {
                const float wx = x * sc.x + tr.x, wy = y * sc.y + tr.y, wz = z * sc.z + tr.z;
                p.px[o + m] = ( wx - tr.x ) / sc.x;
                p.py[o + m] = ( wy - tr.y ) / sc.y;
                p.pz[o + m] = ( wz - tr.z ) / sc.z;
                p.vx[o + m] = 0.f; p.vy[o + m] = 0.f; p.vz[o + m] = 0.f;
                p.id[o + m] = first_id + (int32_t)( offset[c] + m );
            }
            ++m;
        };
        emit( ( cx - 0.5f ) + bora_rand01( ui * 45651u + uk * 75561u + uj * 65551u ),
              ( cy - 0.5f ) + bora_rand01( ui * 51221u + uk * 99331u + uj * 11221u ),
              ( cz - 0.5f ) + bora_rand01( ui * 81221u + uk * 45331u + uj * 66551u ) );
        emit( ( cx - 0.5f ) + bora_rand01( ui * 53454u + uk * 12234u + uj * 23853u ),
              ( cy - 0.5f ) + bora_rand01( ui * 76335u + uk * 94762u + uj * 93654u ),
              ( cz - 0.5f ) + bora_rand01( ui * 98547u + uk * 23443u + uj * 53218u ) );
        emit( cx, cy, cz );
        const float band = wall - cy;
        if( band > 0.f && band < 4.f )
            for( int n = 0; n < per_cell; ++n )
            {
                const unsigned un = (unsigned)n;
                emit( ( cx - 0.5f ) + bora_rand01( ui * 45651u + uk * 75561u + uj * 65551u + un * 44222u ),
                      ( cy - 0.5f ) + bora_rand01( ui * 51221u + uk * 99331u + uj * 11221u + un * 59374u ),
                      ( cz - 0.5f ) + bora_rand01( ui * 81221u + uk * 45331u + uj * 66551u + un * 12333u ) );
            }
        if( !WRITE ) count[c] = m;
    }
}

}  // namespace

void bora_launch_tank( const BoraGridDev& g, int hh, int per_cell, float3 tr, float3 sc, uint32_t* count,
                       const uint32_t* offset, BoraParticlesDev p, size_t base, int32_t first_id, bool write,
                       cudaStream_t st )
{
    const size_t ncell = (size_t)g.nx * hh * g.nz;
    if( ncell == 0 ) return;
    if( write ) k_tank<true><<<grid_for( ncell ), kThreads, 0, st>>>( g, hh, g.voxel_wall, per_cell, tr, sc, count, offset, p, base, first_id );
    else k_tank<false><<<grid_for( ncell ), kThreads, 0, st>>>( g, hh, g.voxel_wall, per_cell, tr, sc, count, offset, p, base, first_id );
}

void bora_launch_bin( const BoraGridDev& g, BoraParticlesDev p, size_t n, uint32_t* vkey, uint8_t* tile_flag, cudaStream_t st )
{
    if( n == 0 ) return;
    k_bin<<<grid_for( ( n + 3 ) / 4 ), kThreads, 0, st>>>( g, p, n, vkey, tile_flag );
}

void bora_launch_activate( const BoraGridDev& g, const uint8_t* tile_flag, uint32_t* act, cudaStream_t st )
{
    const size_t ntv = (size_t)g.tx * g.ty * g.tz;
    // tile rows wholly below the wall level stay active with the tank on (build tile edge 8)
    int tank_rows = 0;
    if( g.enable_tank )
    {
        tank_rows = (int)g.voxel_wall / BORA_TILE;
        tank_rows = tank_rows < 0 ? 0 : ( tank_rows > g.ty ? g.ty : tank_rows );
    }
    k_activate<<<grid_for( ntv ), kThreads, 0, st>>>( g, tile_flag, act, tank_rows );
}

void bora_launch_tile_assign( const BoraGridDev& g, const uint32_t* act, const uint32_t* excl, int32_t* slot_of,
                              int32_t* tile_of, cudaStream_t st )
{
    const size_t ntv = (size_t)g.tx * g.ty * g.tz;
    k_tile_assign<<<grid_for( ntv ), kThreads, 0, st>>>( ntv, act, excl, slot_of, tile_of );
}

void bora_launch_tile_nbrs( const BoraGridDev& g, int ntiles, const int32_t* slot_of, const int32_t* tile_of,
                            int32_t* nbr, cudaStream_t st )
{
    if( ntiles <= 0 ) return;
    k_tile_nbrs<<<grid_for( (size_t)ntiles * 27 ), kThreads, 0, st>>>( g, ntiles, slot_of, tile_of, nbr );
}

void bora_launch_hist( size_t n, const uint32_t* vkey, const int32_t* slot_of, uint32_t outside_key, uint32_t* key,
                       uint32_t* count, uint32_t* err, cudaStream_t st )
{
    if( n == 0 ) return;
    k_hist<<<grid_for( n ), kThreads, 0, st>>>( n, vkey, slot_of, outside_key, key, count, err );
}

void bora_launch_scatter( size_t n, const uint32_t* key, const uint32_t* start, uint32_t* count, uint32_t* idx,
                          cudaStream_t st )
{
    if( n == 0 ) return;
    k_scatter<<<grid_for( n ), kThreads, 0, st>>>( n, key, start, count, idx );
}

void bora_launch_order_bins( size_t nbins, const uint32_t* start, uint32_t* idx, cudaStream_t st )
{
    if( nbins == 0 ) return;
    k_order_bins<<<grid_for( nbins ), kThreads, 0, st>>>( nbins, start, idx, 4096u );
}

void bora_launch_to_soa( size_t n, const float* pos, const float* vel, int space, const float* translate,
                         const float* scale, BoraParticlesDev p, size_t offset, int32_t first_id, cudaStream_t st )
{
    if( n == 0 ) return;
    const float3 tr = make_float3( translate[0], translate[1], translate[2] );
    const float3 sc = make_float3( scale[0], scale[1], scale[2] );
    k_to_soa<<<grid_for( n ), kThreads, 0, st>>>( n, pos, vel, space, tr, sc, p, offset, first_id );
}
