// G2P with the FLIP/PIC blend, Euler advection substeps with the box clamp and collider
// push-out, kill flags and gravity: FLIPMethod::updateParticles
// (base/source/FLIPMethod.cu:54-175), followed by the compaction of Array::remove
// (base/header/Array.h:996-1024, FLIPMethod.cu:293-297).
//
// Particles are visited in dual-cell order through the sort permutation and written
// to the other particle buffer in that order, so the particle store stays spatially
// sorted and each warp's trilinear reads hit the same few cells. Killed particles are
// written with id -1 and dropped by the next step's counting sort.
#include "bora_internal.h"

namespace {

struct CellLookup
{
    const BoraGridDev& g;
    const int32_t* slot_of;
    __device__ inline int index( int i, int j, int k ) const
    {
        const int s = slot_of[( (size_t)( k >> 3 ) * g.ty + ( j >> 3 ) ) * g.tx + ( i >> 3 )];
        if( s < 0 ) return -1;
        return s * BORA_TILE_CELLS + bora_local( i, j, k );
    }
};

// SparseField::lerp over a vector field (base/header/SparseField.h:150-173) and
// SparseField::lerpMin over a scalar field (SparseField.h:176-196). Corner order:
// (i,j,k),(i+1,j,k),(i,j,k+1),(i+1,j,k+1),(i,j+1,k),(i+1,j+1,k),(i,j+1,k+1),(i+1,j+1,k+1).
struct Lerp8
{
    int idx[8];  // cell index, -1 = background (inactive tile)
    float x, y, z;
    __device__ inline void setup( const CellLookup& L, float px, float py, float pz )
    {
        const int i = bora_clampi( bora_trunc( px - 0.5f ), 0, L.g.nx - 2 );
        const int j = bora_clampi( bora_trunc( py - 0.5f ), 0, L.g.ny - 2 );
        const int k = bora_clampi( bora_trunc( pz - 0.5f ), 0, L.g.nz - 2 );
        x = bora_clampf( px - ( (float)i + .5f ), 0.f, 1.f );
        y = bora_clampf( py - ( (float)j + .5f ), 0.f, 1.f );
        z = bora_clampf( pz - ( (float)k + .5f ), 0.f, 1.f );
        const int b = L.index( i, j, k );
        if( b >= 0 && ( i & 7 ) < 7 && ( j & 7 ) < 7 && ( k & 7 ) < 7 )
        {
            // the 2x2x2 block lies inside one tile
            idx[0] = b; idx[1] = b + 1; idx[2] = b + 64; idx[3] = b + 65;
            idx[4] = b + 8; idx[5] = b + 9; idx[6] = b + 72; idx[7] = b + 73;
            return;
        }
        idx[0] = b;
        idx[1] = L.index( i + 1, j, k );
        idx[2] = L.index( i, j, k + 1 );
        idx[3] = L.index( i + 1, j, k + 1 );
        idx[4] = L.index( i, j + 1, k );
        idx[5] = L.index( i + 1, j + 1, k );
        idx[6] = L.index( i, j + 1, k + 1 );
        idx[7] = L.index( i + 1, j + 1, k + 1 );
    }
    __device__ inline float get( const float* __restrict__ f, int q, float bg ) const { return idx[q] < 0 ? bg : __ldg( f + idx[q] ); }
    __device__ inline float lerp( const float* __restrict__ f ) const
    {
        const float c00 = get( f, 0, 0.f ) * ( 1.f - x ) + get( f, 1, 0.f ) * x;
        const float c01 = get( f, 2, 0.f ) * ( 1.f - x ) + get( f, 3, 0.f ) * x;
        const float c10 = get( f, 4, 0.f ) * ( 1.f - x ) + get( f, 5, 0.f ) * x;
        const float c11 = get( f, 6, 0.f ) * ( 1.f - x ) + get( f, 7, 0.f ) * x;
        const float c0 = c00 * ( 1.f - y ) + c10 * y;
        const float c1 = c01 * ( 1.f - y ) + c11 * y;
        return c0 * ( 1.f - z ) + c1 * z;
    }
    __device__ inline float lerp_min( const float* __restrict__ f, float bg ) const
    {
        float v = fminf_ref( get( f, 0, bg ), get( f, 1, bg ) );
        v = fminf_ref( v, fminf_ref( get( f, 2, bg ), get( f, 3, bg ) ) );
        v = fminf_ref( v, fminf_ref( get( f, 4, bg ), get( f, 5, bg ) ) );
        v = fminf_ref( v, fminf_ref( get( f, 6, bg ), get( f, 7, bg ) ) );
        return v;
    }
    __device__ static inline float fminf_ref( float a, float b ) { return a < b ? a : b; }  // MathUtils.h:174
};

__device__ inline bool inside_grid( const BoraGridDev& g, float x, float y, float z )
{
    return !( x < 0.f || x > (float)g.nx || y < 0.f || y > (float)g.ny || z < 0.f || z > (float)g.nz );
}

// Collider interactions of FLIPMethod::updateParticles, kept out of line: they are rare,
// and their corner arrays would otherwise spill the common path's registers.
__device__ __noinline__ float3 col_carry( const BoraGridDev* g, float3 p, float dt )
{
    if( bora_col_phi( *g, p.x, p.y, p.z ) < 0.f )  // FLIPMethod.cu:116-119
    {
        float cv[3];
        bora_col_lerp( g->cols, g->nx, g->ny, g->nz, p.x, p.y, p.z, 2, cv );
        p.x += cv[0] * dt; p.y += cv[1] * dt; p.z += cv[2] * dt;
    }
    return p;
}

// push-out along the collider normal (FLIPMethod.cu:146-157); w = 1 when it collided
__device__ __noinline__ float4 col_push( const BoraGridDev* g, float3 p )
{
    const float phi = bora_col_phi( *g, p.x, p.y, p.z );
    if( !( phi < 0.f ) ) return make_float4( p.x, p.y, p.z, 0.f );
    float nr[3];
    bora_col_lerp( g->cols, g->nx, g->ny, g->nz, p.x, p.y, p.z, 1, nr );
    // Vec3f::normalized (base/header/Vector3.h:350-354)
    const double dn = 1.0f / sqrtf( nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2] + 1e-30f );
    const float ux = (float)( nr[0] * dn ), uy = (float)( nr[1] * dn ), uz = (float)( nr[2] * dn );
    return make_float4( p.x - ux * phi, p.y - uy * phi, p.z - uz * phi, 1.f );
}

__device__ __noinline__ bool col_kill( const BoraGridDev* g, float3 p )
{
    const float phi = bora_col_phi( *g, p.x, p.y, p.z );  // FLIPMethod.cu:161-165
    return phi > 3.f || phi < 0.f;
}

__global__ void __launch_bounds__( 256 ) k_g2p( const __grid_constant__ BoraGridDev g, size_t n, const int32_t* __restrict__ slot_of,
                                                BoraCellsDev c, BoraParticlesDev src, const uint32_t* __restrict__ idx,
                                                BoraParticlesDev dst, float* __restrict__ adj, float dt,
                                                uint32_t* __restrict__ nkilled )
{
    const CellLookup L{ g, slot_of };
    const float lx = (float)g.nx + 0.5f, lz = (float)g.nz + 0.5f;
    const float wall = g.voxel_wall;
    uint32_t kills = 0;
    for( size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x )
    {
        const uint32_t pi = idx[q];
        float px = src.px[pi], py = src.py[pi], pz = src.pz[pi];
        float vx = src.vx[pi], vy = src.vy[pi], vz = src.vz[pi];
        int32_t id = src.id[pi];
        Lerp8 lp;
        lp.setup( L, px, py, pz );
        adj[q] = lp.lerp_min( c.surf, 10.f );  // surf background 10 (FLIPMethod.cu:30)
        {
            const float gx = lp.lerp( c.cx ), gy = lp.lerp( c.cy ), gz = lp.lerp( c.cz );
            const float ox = lp.lerp( c.vx ), oy = lp.lerp( c.vy ), oz = lp.lerp( c.vz );
            vx += gx - ox; vy += gy - oy; vz += gz - oz;
            vx = vx * 0.95f + gx * 0.05f;
            vy = vy * 0.95f + gy * 0.05f;
            vz = vz * 0.95f + gz * 0.05f;
        }
        if( g.enable_tank && py <= wall )
        {
            const float band = g.damping_band;
            float w = 1.f;
            if( px < band ) w = fminf( w, bora_clampf( ( px - 0.f ) / band, 0.f, 1.f ) );
            if( px > lx - band ) w = fminf( w, bora_clampf( ( lx - px ) / band, 0.f, 1.f ) );
            if( pz < band ) w = fminf( w, bora_clampf( ( pz - 0.f ) / band, 0.f, 1.f ) );
            if( pz > lz - band ) w = fminf( w, bora_clampf( ( lz - pz ) / band, 0.f, 1.f ) );
            vx *= w; vy *= w; vz *= w;
        }
        const bool hasCols = g.cols.count > 0;
        if( hasCols )
        {
            const float3 p = col_carry( &g, make_float3( px, py, pz ), dt );
            px = p.x; py = p.y; pz = p.z;
        }
        bool kill = false;
        {
            const float len = sqrtf( vx * vx + vy * vy + vz * vz );
            const int iter = 1 + bora_imin( bora_trunc( len * dt * 1.5f ), bora_imax( g.maxsubsteps, 1 ) );
            const float sub_dt = dt / (float)iter;
            bool col = false;
            for( int it = 0; it < iter; ++it )
            {
                px += vx * sub_dt; py += vy * sub_dt; pz += vz * sub_dt;
                if( py <= wall )
                {
                    if( px < 0.f ) { px = 0.f; if( vx < 0.f ) vx = 0.f; }
                    if( py < 0.f ) { py = 0.f; if( vy < 0.f ) vy = 0.f; }
                    if( pz < 0.f ) { pz = 0.f; if( vz < 0.f ) vz = 0.f; }
                    if( px > (float)g.nx ) { px = (float)g.nx; if( vx > 0.f ) vx = 0.f; }
                    if( py > (float)g.ny ) { py = (float)g.ny; if( vy > 0.f ) vy = 0.f; }
                    if( pz > (float)g.nz ) { pz = (float)g.nz; if( vz > 0.f ) vz = 0.f; }
                }
                if( hasCols )
                {
                    const float4 r = col_push( &g, make_float3( px, py, pz ) );
                    px = r.x; py = r.y; pz = r.z;
                    if( r.w != 0.f ) col = true;
                }
            }
            if( col && col_kill( &g, make_float3( px, py, pz ) ) ) kill = true;
            if( !inside_grid( g, px, py, pz ) ) kill = true;
        }
        vx += g.gravity[0] * dt; vy += g.gravity[1] * dt; vz += g.gravity[2] * dt;
        dst.px[q] = px; dst.py[q] = py; dst.pz[q] = pz;
        dst.vx[q] = vx; dst.vy[q] = vy; dst.vz[q] = vz;
        dst.id[q] = kill ? -1 : id;
        kills += kill ? 1u : 0u;
    }
    // one atomic per warp
    for( int o = 16; o > 0; o >>= 1 ) kills += __shfl_xor_sync( 0xffffffffu, kills, o );
    if( ( threadIdx.x & 31 ) == 0 && kills ) atomicAdd( nkilled, kills );
}

}  // namespace

void bora_launch_g2p( const BoraGridDev& g, size_t n, const int32_t* slot_of, BoraCellsDev c, BoraParticlesDev src,
                      const uint32_t* idx, BoraParticlesDev dst, float* adj, float dt, uint32_t* nkilled, cudaStream_t st )
{
    if( n == 0 ) return;
    size_t b = ( n + 255 ) / 256;
    if( b > 152 * 16 ) b = 152 * 16;
    k_g2p<<<(int)b, 256, 0, st>>>( g, n, slot_of, c, src, idx, dst, adj, dt, nkilled );
}
