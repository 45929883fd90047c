// G2P with the FLIP/PIC blend, Euler advection substeps with the box clamp and collider
// push-out, kill flags and gravity: FLIPMethod::updateParticles
// (base/source/FLIPMethod.cu:54-175), followed by the compaction of Array::remove
// (base/header/Array.h:996-1024, FLIPMethod.cu:293-297).
//
// Particles are visited in dual-cell order through the sort permutation and written
// to the other particle buffer in that order, so the particle store stays spatially
// sorted and each warp's trilinear reads hit the same few cells. Killed particles are
// written with id -1 and dropped by the next step's counting sort. Each written particle
// is also binned for the next rebuild (its sort key and tile flag, the rule of k_bin), so
// that the next step need not read the particles again to bin them; a tile's CTA marks the
// flags of the 27 tiles around its own in shared memory and stores each marked one once.
#include "bora_internal.h"
#include "../../include/bora_flip.h"

namespace {

// Grid values of a tile and its high-side halo layer, (8+1)^3 cells, staged in shared
// memory as two float4 per cell: (comp.x, comp.y, velo.x, velo.y) and (comp.z, velo.z, surf,
// 0), so that the lerps of both vector fields read two float4 per corner. Cells of inactive
// tiles hold the field backgrounds (0, and 10 for surf: FLIPMethod.cu:30).
constexpr int kG2PThreads = 256;
constexpr int kStageEdge = BORA_TILE + 1;
constexpr int kStageCells = kStageEdge * kStageEdge * kStageEdge;

// SparseField::lerp over a vector field (base/header/SparseField.h:150-173) and
// SparseField::lerpMin over a scalar field (SparseField.h:176-196), from the staged tile.
// Corner order: (i,j,k),(i+1,j,k),(i,j,k+1),(i+1,j,k+1),(i,j+1,k),(i+1,j+1,k),(i,j+1,k+1),
// (i+1,j+1,k+1).
struct StagedLerp
{
    int base;  // staged index of corner (i,j,k)
    float x, y, z;
    __device__ inline void setup( const BoraGridDev& g, int ti, int tj, int tk, float px, float py, float pz )
    {
        const int i = bora_clampi( bora_trunc( px - 0.5f ), 0, g.nx - 2 );
        const int j = bora_clampi( bora_trunc( py - 0.5f ), 0, g.ny - 2 );
        const int k = bora_clampi( bora_trunc( pz - 0.5f ), 0, g.nz - 2 );
        x = bora_clampf( px - ( (float)i + .5f ), 0.f, 1.f );
        y = bora_clampf( py - ( (float)j + .5f ), 0.f, 1.f );
        z = bora_clampf( pz - ( (float)k + .5f ), 0.f, 1.f );
        base = ( i - ti * BORA_TILE ) + kStageEdge * ( ( j - tj * BORA_TILE ) + kStageEdge * ( k - tk * BORA_TILE ) );
    }
    __device__ static inline int off( int q )
    {
        return ( q & 1 ) + kStageEdge * kStageEdge * ( ( q >> 1 ) & 1 ) + kStageEdge * ( q >> 2 );
    }
    __device__ static inline float4 mix( float4 a, float4 b, float t )
    {
        return make_float4( a.x * ( 1.f - t ) + b.x * t, a.y * ( 1.f - t ) + b.y * t, a.z * ( 1.f - t ) + b.z * t,
                            a.w * ( 1.f - t ) + b.w * t );
    }
    __device__ static inline float fminf_ref( float a, float b ) { return a < b ? a : b; }  // MathUtils.h:174
    // comp and velo lerped from the staged cells (comp.xy and velo.xy from fa, comp.z and
    // velo.z from fb), and lerpMin of surf; the corners' mix order and the min order are
    // SparseField's
    __device__ inline void sample( const float4* fa, const float4* fb, float4& comp, float4& velo, float& smin ) const
    {
        auto lerp = [&]( const float4* f ) {
            const float4 c00 = mix( f[base + off( 0 )], f[base + off( 1 )], x );
            const float4 c01 = mix( f[base + off( 2 )], f[base + off( 3 )], x );
            const float4 c10 = mix( f[base + off( 4 )], f[base + off( 5 )], x );
            const float4 c11 = mix( f[base + off( 6 )], f[base + off( 7 )], x );
            return mix( mix( c00, c10, y ), mix( c01, c11, y ), z );
        };
        const float4 A = lerp( fa ), B = lerp( fb );
        comp = make_float4( A.x, A.y, B.x, 0.f );
        velo = make_float4( A.z, A.w, B.y, 0.f );
        auto w = [&]( int q ) { return fb[base + off( q )].z; };
        float v = fminf_ref( w( 0 ), w( 1 ) );
        v = fminf_ref( v, fminf_ref( w( 2 ), w( 3 ) ) );
        v = fminf_ref( v, fminf_ref( w( 4 ), w( 5 ) ) );
        v = fminf_ref( v, fminf_ref( w( 6 ), w( 7 ) ) );
        smin = v;
    }
};

// The same lerps through the tile table, for the rare particles outside every tile (the
// sort's last bin: particles added outside the grid, killed by this step's bounds check).
struct GlobalLerp
{
    const BoraGridDev& g;
    const int32_t* slot_of;
    const BoraCellsDev& c;
    int idx[8];  // cell index, -1 = background (inactive tile)
    float x, y, z;
    __device__ inline int index( int i, int j, int k ) const
    {
        const int s = slot_of[( (size_t)( k >> 3 ) * g.ty + ( j >> 3 ) ) * g.tx + ( i >> 3 )];
        return s < 0 ? -1 : s * BORA_TILE_CELLS + bora_local( i, j, k );
    }
    __device__ inline void setup( float px, float py, float pz )
    {
        const int i = bora_clampi( bora_trunc( px - 0.5f ), 0, g.nx - 2 );
        const int j = bora_clampi( bora_trunc( py - 0.5f ), 0, g.ny - 2 );
        const int k = bora_clampi( bora_trunc( pz - 0.5f ), 0, g.nz - 2 );
        x = bora_clampf( px - ( (float)i + .5f ), 0.f, 1.f );
        y = bora_clampf( py - ( (float)j + .5f ), 0.f, 1.f );
        z = bora_clampf( pz - ( (float)k + .5f ), 0.f, 1.f );
        for( int q = 0; q < 8; ++q ) idx[q] = index( i + ( q & 1 ), j + ( q >> 2 ), k + ( ( q >> 1 ) & 1 ) );
    }
    __device__ inline float4 fa( int q ) const
    {
        return idx[q] < 0 ? make_float4( 0.f, 0.f, 0.f, 10.f )
                          : make_float4( c.cx[idx[q]], c.cy[idx[q]], c.cz[idx[q]], c.surf[idx[q]] );
    }
    __device__ inline float4 fb( int q ) const
    {
        return idx[q] < 0 ? make_float4( 0.f, 0.f, 0.f, 0.f ) : make_float4( c.vx[idx[q]], c.vy[idx[q]], c.vz[idx[q]], 0.f );
    }
    template <bool A>
    __device__ inline float4 lerp() const
    {
        auto f = [&]( int q ) { return A ? fa( q ) : fb( q ); };
        const float4 c00 = StagedLerp::mix( f( 0 ), f( 1 ), x );
        const float4 c01 = StagedLerp::mix( f( 2 ), f( 3 ), x );
        const float4 c10 = StagedLerp::mix( f( 4 ), f( 5 ), x );
        const float4 c11 = StagedLerp::mix( f( 6 ), f( 7 ), x );
        return StagedLerp::mix( StagedLerp::mix( c00, c10, y ), StagedLerp::mix( c01, c11, y ), z );
    }
    __device__ inline float surf_min() const
    {
        auto w = [&]( int q ) { return fa( q ).w; };
        float v = StagedLerp::fminf_ref( w( 0 ), w( 1 ) );
        v = StagedLerp::fminf_ref( v, StagedLerp::fminf_ref( w( 2 ), w( 3 ) ) );
        v = StagedLerp::fminf_ref( v, StagedLerp::fminf_ref( w( 4 ), w( 5 ) ) );
        v = StagedLerp::fminf_ref( v, StagedLerp::fminf_ref( w( 6 ), w( 7 ) ) );
        return v;
    }
    __device__ inline float4 comp() const { return lerp<true>(); }
    __device__ inline float4 velo() const { return lerp<false>(); }
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

// Grid velocity ("comp") at an arbitrary point, for the RK2 option.
__device__ inline float4 comp_at( const BoraGridDev& g, const int32_t* slot_of, const BoraCellsDev& c, float x, float y,
                                  float z )
{
    GlobalLerp l{ g, slot_of, c };
    l.setup( x, y, z );
    return l.comp();
}

// FLIPMethod::updateParticles for one particle (FLIPMethod.cu:60-170); gn and go are the
// grid's projected and pre-projection velocities lerped at the particle's position. With the
// RK2 option each substep moves the particle by the midpoint rule in the grid velocity field
// instead of by its own velocity; everything else is unchanged. kAll = false compiles the
// common case alone: no water tank, no colliders, Euler advection (the caller checks).
template <bool kAll>
__device__ inline bool advance_particle( const BoraGridDev& g, float4 gn, float4 go, const int32_t* slot_of,
                                         const BoraCellsDev& c, float& px, float& py, float& pz, float& vx, float& vy,
                                         float& vz, float dt )
{
    const float lx = (float)g.nx + 0.5f, lz = (float)g.nz + 0.5f;
    const float wall = g.voxel_wall;
    {
        vx += gn.x - go.x; vy += gn.y - go.y; vz += gn.z - go.z;
        vx = vx * 0.95f + gn.x * 0.05f;
        vy = vy * 0.95f + gn.y * 0.05f;
        vz = vz * 0.95f + gn.z * 0.05f;
    }
    if( kAll && g.enable_tank && py <= wall )
    {
        const float band = g.damping_band;
        float w = 1.f;
        if( px < band ) w = fminf( w, bora_clampf( ( px - 0.f ) / band, 0.f, 1.f ) );
        if( px > lx - band ) w = fminf( w, bora_clampf( ( lx - px ) / band, 0.f, 1.f ) );
        if( pz < band ) w = fminf( w, bora_clampf( ( pz - 0.f ) / band, 0.f, 1.f ) );
        if( pz > lz - band ) w = fminf( w, bora_clampf( ( lz - pz ) / band, 0.f, 1.f ) );
        vx *= w; vy *= w; vz *= w;
    }
    // Collider work only where a collider can be met this step: the substep positions stay
    // within |v| dt of the start (the box clamp only shortens moves of particles that start
    // inside the grid), a sampled collider value is a lerp of box distances at cell centres
    // within sqrt(3) cells, and a box distance changes by at most the distance moved. So a
    // particle whose start is farther than 2 |v| dt + 2 cells from every box sees positive
    // collider values all step long. (RK2 moves with the grid velocity: no cull.)
    bool hasCols = kAll && bora_col_active( g.cols );
    if( hasCols && g.cols.tslot && g.advection != BORA_ADVECT_RK2 && inside_grid( g, px, py, pz ) )
    {
        // sparse collider: every sample outside its tiles is the (positive) background with
        // a zero normal and velocity; a particle whose tile has no collider tile within one
        // tile is 8 cells or more from every stored sample, and the samples it reads this
        // step lie within |v| dt + 3 cells of its start
        const float move = sqrtf( vx * vx + vy * vy + vz * vz ) * dt;
        if( g.cols.tbg > 0.f && move < 5.f )
        {
            const int ti = bora_imin( bora_trunc( px ) >> 3, g.tx - 1 ), tj = bora_imin( bora_trunc( py ) >> 3, g.ty - 1 ),
                      tk = bora_imin( bora_trunc( pz ) >> 3, g.tz - 1 );
            if( !g.cols.tnear[(size_t)ti + (size_t)g.tx * ( (size_t)tj + (size_t)g.ty * tk )] ) hasCols = false;
        }
    }
    else if( hasCols && !g.cols.fphi && g.advection != BORA_ADVECT_RK2 && inside_grid( g, px, py, pz ) )
    {
        const float reach = 2.f * sqrtf( vx * vx + vy * vy + vz * vz ) * dt + 2.f;
        hasCols = false;
        for( int n = 0; n < g.cols.count; ++n )
            if( !( bora_box_sdf( g.cols.box[n], px, py, pz ) > reach ) ) hasCols = true;
    }
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
            if( kAll && g.advection == BORA_ADVECT_RK2 )
            {
                const float h = 0.5f * sub_dt;
                const float4 k1 = comp_at( g, slot_of, c, px, py, pz );
                const float4 k2 = comp_at( g, slot_of, c, px + k1.x * h, py + k1.y * h, pz + k1.z * h );
                px += k2.x * sub_dt; py += k2.y * sub_dt; pz += k2.z * sub_dt;
            }
            else
            {
                px += vx * sub_dt; py += vy * sub_dt; pz += vz * sub_dt;
            }
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
    return kill;
}

// One CTA per tile: stage the tile's grid values, then advance the particles of the
// tile's dual cells (a contiguous range of the sorted order). The CTA after the last tile
// advances the sort's outside bin through the tile table. The common-case kernel (kAll =
// false) needs 80 registers without spills and runs three CTAs per SM; the one with the
// collider, water-tank and RK2 paths runs four at 64 registers.
template <bool kAll>
__global__ void __launch_bounds__( kG2PThreads, kAll ? 4 : 3 ) k_g2p( const __grid_constant__ BoraGridDev g, BoraTilesDev t, int ntiles,
                                                       uint32_t nsorted, const uint32_t* __restrict__ start, BoraCellsDev c,
                                                       BoraParticlesDev src, const uint32_t* __restrict__ idx,
                                                       BoraParticlesDev dst, float* __restrict__ adj, float dt,
                                                       uint32_t* __restrict__ nkilled, uint32_t* __restrict__ vkey,
                                                       uint8_t* __restrict__ tile_flag )
{
    __shared__ float4 fa[kStageCells];  // comp.x, comp.y, velo.x, velo.y
    __shared__ float4 fb[kStageCells];  // comp.z, velo.z, surf, 0
    __shared__ int32_t nb[27];
    __shared__ uint8_t near_flag[27];  // activation flags of the tiles around the CTA's own
    const int s = blockIdx.x, tid = threadIdx.x;
    uint32_t kills = 0;
    int cti = -8, ctj = -8, ctk = -8;  // the CTA's tile (far from every tile: no shared flags)
    auto finish = [&]( uint32_t q, uint32_t pi, int32_t id, float px, float py, float pz, float vx, float vy, float vz,
                       bool kill ) {
        dst.px[q] = px; dst.py[q] = py; dst.pz[q] = pz;
        dst.vx[q] = vx; dst.vy[q] = vy; dst.vz[q] = vz;
        dst.id[q] = kill ? -1 : id;
        uint32_t key = BORA_DEAD_KEY;
        if( !kill && id >= 0 )
        {
            int ti, tj, tk;
            bora_bin_tile( g.tx, g.ty, g.tz, px, py, pz, ti, tj, tk );
            const int dx = ti - cti, dy = tj - ctj, dz = tk - ctk;
            if( dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1 ) near_flag[bora_dir( dx, dy, dz )] = 1;
            else tile_flag[( (size_t)tk * g.ty + tj ) * g.tx + ti] = 1;
            key = bora_bin_live_key( g.nx, g.ny, g.nz, g.tx, g.ty, px, py, pz );
        }
        vkey[q] = key;
        if( dst.vort )  // post-processing attributes ride along (FLIPMethod.cu:295-296)
        {
            dst.vort[q] = src.vort[pi];
            dst.curv[q] = src.curv[pi];
        }
        kills += kill ? 1u : 0u;
    };
    if( s == ntiles )
    {
        const uint32_t q0 = start[(size_t)ntiles * BORA_TILE_CELLS], q1 = nsorted;
        for( uint32_t q = q0 + tid; q < q1; q += kG2PThreads )
        {
            const uint32_t pi = idx[q];
            float px = src.px[pi], py = src.py[pi], pz = src.pz[pi];
            float vx = src.vx[pi], vy = src.vy[pi], vz = src.vz[pi];
            GlobalLerp smp{ g, t.slot_of, c };
            smp.setup( px, py, pz );
            adj[q] = smp.surf_min();
            const bool kill = advance_particle<kAll>( g, smp.comp(), smp.velo(), t.slot_of, c, px, py, pz, vx, vy, vz, dt );
            finish( q, pi, src.id[pi], px, py, pz, vx, vy, vz, kill );
        }
    }
    else
    {
        if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
        if( tid < 27 ) near_flag[tid] = 0;
        const int vt = t.tile_of[s];
        const int ti = vt % g.tx, tj = ( vt / g.tx ) % g.ty, tk = vt / ( g.tx * g.ty );
        cti = ti; ctj = tj; ctk = tk;
        // the thread's particles are loaded one ahead and their sorted-order indices two ahead:
        // the first particle and the second index before the staging, then each next particle
        // (from an index that has arrived) while the current one is advanced
        const uint32_t q0 = start[(size_t)s * BORA_TILE_CELLS], q1 = start[(size_t)( s + 1 ) * BORA_TILE_CELLS];
        uint32_t pin = 0, pin2 = 0;
        int32_t idn = 0;
        float pxn = 0.f, pyn = 0.f, pzn = 0.f, vxn = 0.f, vyn = 0.f, vzn = 0.f;
        auto fetch = [&]( uint32_t pi ) {
            pxn = src.px[pi]; pyn = src.py[pi]; pzn = src.pz[pi];
            vxn = src.vx[pi]; vyn = src.vy[pi]; vzn = src.vz[pi];
            idn = src.id[pi];
        };
        if( q0 + tid < q1 )
        {
            pin = idx[q0 + tid];
            fetch( pin );
        }
        if( q0 + tid + kG2PThreads < q1 ) pin2 = idx[q0 + tid + kG2PThreads];
        __syncthreads();
        for( int h = tid; h < kStageCells; h += kG2PThreads )
        {
            const int a = h % kStageEdge, b = ( h / kStageEdge ) % kStageEdge, cz = h / ( kStageEdge * kStageEdge );
            const int ns = nb[bora_dir( a >> 3, b >> 3, cz >> 3 )];
            float4 va = make_float4( 0.f, 0.f, 0.f, 0.f ), vb = make_float4( 0.f, 0.f, 10.f, 0.f );
            if( ns >= 0 )
            {
                const size_t q = (size_t)ns * BORA_TILE_CELLS + (size_t)bora_local( a, b, cz );
                va = make_float4( c.cx[q], c.cy[q], c.vx[q], c.vy[q] );
                vb = make_float4( c.cz[q], c.vz[q], c.surf[q], 0.f );
            }
            fa[h] = va;
            fb[h] = vb;
        }
        __syncthreads();
        for( uint32_t q = q0 + tid; q < q1; q += kG2PThreads )
        {
            const uint32_t pi = pin;
            const int32_t id = idn;
            float px = pxn, py = pyn, pz = pzn;
            float vx = vxn, vy = vyn, vz = vzn;
            if( q + kG2PThreads < q1 )
            {
                pin = pin2;
                fetch( pin );
                if( q + 2 * kG2PThreads < q1 ) pin2 = idx[q + 2 * kG2PThreads];
            }
            StagedLerp l;
            l.setup( g, ti, tj, tk, px, py, pz );
            float4 gn, go;
            float smin;
            l.sample( fa, fb, gn, go, smin );
            adj[q] = smin;  // surf background 10 (FLIPMethod.cu:30)
            const bool kill = advance_particle<kAll>( g, gn, go, t.slot_of, c, px, py, pz, vx, vy, vz, dt );
            finish( q, pi, id, px, py, pz, vx, vy, vz, kill );
        }
        __syncthreads();
        if( tid < 27 && near_flag[tid] )  // a marked tile is a clamped particle tile: inside the table
        {
            const int i = cti + tid % 3 - 1, j = ctj + ( tid / 3 ) % 3 - 1, k = ctk + tid / 9 - 1;
            tile_flag[( (size_t)k * g.ty + j ) * g.tx + i] = 1;
        }
    }
    // one atomic per warp
    for( int o = 16; o > 0; o >>= 1 ) kills += __shfl_xor_sync( 0xffffffffu, kills, o );
    if( ( threadIdx.x & 31 ) == 0 && kills ) atomicAdd( nkilled, kills );
}

}  // namespace

void bora_launch_g2p( const BoraGridDev& g, int ntiles, size_t nsorted, BoraTilesDev t, const uint32_t* start, BoraCellsDev c,
                      BoraParticlesDev src, const uint32_t* idx, BoraParticlesDev dst, float* adj, float dt,
                      uint32_t* nkilled, uint32_t* vkey, uint8_t* tile_flag, cudaStream_t st )
{
    if( nsorted == 0 ) return;
    // the common case (no water tank, no colliders, Euler advection) in a kernel without the
    // code of the others
    if( g.enable_tank || bora_col_active( g.cols ) || g.advection == BORA_ADVECT_RK2 )
        k_g2p<true><<<ntiles + 1, kG2PThreads, 0, st>>>( g, t, ntiles, (uint32_t)nsorted, start, c, src, idx, dst, adj, dt,
                                                         nkilled, vkey, tile_flag );
    else
        k_g2p<false><<<ntiles + 1, kG2PThreads, 0, st>>>( g, t, ntiles, (uint32_t)nsorted, start, c, src, idx, dst, adj,
                                                          dt, nkilled, vkey, tile_flag );
}
