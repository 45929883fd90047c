// FLIPMethod::postProcess (base/source/FLIPMethod.cu:300-405) on the device: the surface
// and velocity splat, the water tank's fill of enclosed air pockets, redistancing of the
// surface, and the particles' vorticity and curvature.
//
// Fields live in the step's tile storage (active slots x 512 cells). The stencil kernels
// stage a tile and a one-cell halo (10^3 cells) in shared memory; cells of inactive
// tiles read the field's background (surf 10, velocity and normals 0), as
// SparseField::operator() does (base/header/SparseField.h:57-63). Cells of an 8^3 tile
// that lie beyond the grid are never read by a cell inside it (faces use the mirrored or
// tank rule), so they are left alone.
#include "bora_internal.h"

namespace {

// Max / Min of base/header/MathUtils.h:174-198 (the sign of a zero matters in the
// redistancing update).
__device__ inline float maxr( float a, float b ) { return a > b ? a : b; }
__device__ inline float minr( float a, float b ) { return a < b ? a : b; }

__device__ inline bool inside_grid( const BoraGridDev& g, float x, float y, float z )  // Grid::inside, Grid.h:408-417
{
    return !( x < 0.f || x > (float)g.nx || y < 0.f || y > (float)g.ny || z < 0.f || z > (float)g.nz );
}

__device__ inline void tile_coords( const BoraGridDev& g, int vt, int& ti, int& tj, int& tk )
{
    ti = vt % g.tx;
    tj = ( vt / g.tx ) % g.ty;
    tk = vt / ( g.tx * g.ty );
}

// ======================================================================================
// Rasterization::ParticlesToSurfaceAndVelocity (base/source/Rasterization.cu:311-398),
// influence 1.5, droplet 0.5 (FLIPMethod.cu:320). One CTA per tile takes the particles
// of the tile's dual cells (a contiguous range of the sort) and adds their weights into
// an 11^3 shared-memory region (tile cells -1..9: a particle in dual cell d reaches
// cells (int)p-1..(int)p+1 within d-1..d+2), then adds the region to the grid. Cells
// 2..6 of the tile are reached only from the tile's own dual cells and are stored; the
// rest are added with atomics, in no fixed order, as the reference's atomics are.
constexpr int kSplatEdge = 11;
constexpr int kSplatCells = kSplatEdge * kSplatEdge * kSplatEdge;
constexpr int kSplatThreads = 256;

// max(0, (1 - (d/1.5)^2)^3) at the centre of cell (i,j,k) (Rasterization.cu:343-349,
// Vec3f::length, base/header/Vector3.h:328-331). d^2 >= 2.25 gives 0 without the
// division: then d >= 1.5, s >= 1 and the cube is <= 0.
__device__ inline float splat_weight( float px, float py, float pz, int i, int j, int k )
{
    const float dx = px - ( (float)i + .5f ), dy = py - ( (float)j + .5f ), dz = pz - ( (float)k + .5f );
    const float d2 = dx * dx + dy * dy + dz * dz;
    if( !( d2 < 2.25f ) ) return 0.f;
    const float s = sqrtf( d2 ) / 1.5f;
    const float t = 1.f - s * s;
    return maxr( 0.f, t * t * t );
}

__global__ void __launch_bounds__( kSplatThreads ) k_splat( const __grid_constant__ BoraGridDev g, BoraTilesDev t,
                                                            const uint32_t* __restrict__ start,
                                                            const uint32_t* __restrict__ idx, BoraParticlesDev p,
                                                            BoraCellsDev c )
{
    __shared__ float acc[7][kSplatCells];  // w, w x, w y, w z, w u, w v, w w
    __shared__ int32_t nb[27];
    const int s = blockIdx.x, tid = threadIdx.x;
    for( int h = tid; h < 7 * kSplatCells; h += kSplatThreads ) ( &acc[0][0] )[h] = 0.f;
    if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    const int ox = ti * BORA_TILE - 1, oy = tj * BORA_TILE - 1, oz = tk * BORA_TILE - 1;
    __syncthreads();
    const uint32_t q0 = start[(size_t)s * BORA_TILE_CELLS], q1 = start[(size_t)( s + 1 ) * BORA_TILE_CELLS];
    for( uint32_t q = q0 + tid; q < q1; q += kSplatThreads )
    {
        const uint32_t pi = idx[q];
        const float x = p.px[pi], y = p.py[pi], z = p.pz[pi];
        if( !inside_grid( g, x, y, z ) ) continue;
        const float u = p.vx[pi], v = p.vy[pi], w = p.vz[pi];
        // Grid::neighborCells (base/header/Grid.h:353-370) with offset (int)1.5 = 1
        const int xi = bora_trunc( x ), yi = bora_trunc( y ), zi = bora_trunc( z );
        const int i0 = bora_clampi( xi - 1, 0, g.nx - 1 ), i1 = bora_clampi( xi + 1, 0, g.nx - 1 );
        const int j0 = bora_clampi( yi - 1, 0, g.ny - 1 ), j1 = bora_clampi( yi + 1, 0, g.ny - 1 );
        const int k0 = bora_clampi( zi - 1, 0, g.nz - 1 ), k1 = bora_clampi( zi + 1, 0, g.nz - 1 );
        for( int k = k0; k <= k1; ++k )
            for( int j = j0; j <= j1; ++j )
                for( int i = i0; i <= i1; ++i )
                {
                    const float wt = splat_weight( x, y, z, i, j, k );
                    if( wt == 0.f ) continue;  // adds nothing: every sum starts at +0
                    const int h = ( i - ox ) + kSplatEdge * ( ( j - oy ) + kSplatEdge * ( k - oz ) );
                    atomicAdd( &acc[0][h], wt );
                    atomicAdd( &acc[1][h], wt * x );
                    atomicAdd( &acc[2][h], wt * y );
                    atomicAdd( &acc[3][h], wt * z );
                    atomicAdd( &acc[4][h], wt * u );
                    atomicAdd( &acc[5][h], wt * v );
                    atomicAdd( &acc[6][h], wt * w );
                }
    }
    __syncthreads();
    for( int h = tid; h < kSplatCells; h += kSplatThreads )
    {
        const float ws = acc[0][h];
        if( ws == 0.f ) continue;
        const int a = h % kSplatEdge, b = ( h / kSplatEdge ) % kSplatEdge, cc = h / ( kSplatEdge * kSplatEdge );
        const int sl = nb[bora_dir( a == 0 ? -1 : ( a >= 9 ? 1 : 0 ), b == 0 ? -1 : ( b >= 9 ? 1 : 0 ),
                                    cc == 0 ? -1 : ( cc >= 9 ? 1 : 0 ) )];
        if( sl < 0 ) continue;  // cannot happen: the tiles around a particle's tile are active
        const size_t n = (size_t)sl * BORA_TILE_CELLS + (size_t)bora_local( ox + a, oy + b, oz + cc );
        if( a >= 3 && a <= 7 && b >= 3 && b <= 7 && cc >= 3 && cc <= 7 )
        {
            c.surf[n] = ws;
            c.cx[n] = acc[1][h]; c.cy[n] = acc[2][h]; c.cz[n] = acc[3][h];
            c.vx[n] = acc[4][h]; c.vy[n] = acc[5][h]; c.vz[n] = acc[6][h];
        }
        else
        {
            atomicAdd( &c.surf[n], ws );
            atomicAdd( &c.cx[n], acc[1][h] ); atomicAdd( &c.cy[n], acc[2][h] ); atomicAdd( &c.cz[n], acc[3][h] );
            atomicAdd( &c.vx[n], acc[4][h] ); atomicAdd( &c.vy[n], acc[5][h] ); atomicAdd( &c.vz[n], acc[6][h] );
        }
    }
}

// Rasterization.cu:373-395 per cell: the weighted mean position's distance to the cell
// centre minus the droplet radius (5 where no weight landed), the weighted mean
// velocity; the weight sum goes to pres, the field FLIPMethod.cu:320 passes as "mass".
__global__ void k_splat_finish( const __grid_constant__ BoraGridDev g, BoraTilesDev t, size_t ncell, BoraCellsDev c )
{
    for( size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < ncell; n += (size_t)gridDim.x * blockDim.x )
    {
        int ti, tj, tk;
        tile_coords( g, t.tile_of[n / BORA_TILE_CELLS], ti, tj, tk );
        const int l = (int)( n % BORA_TILE_CELLS );
        const int i = ti * BORA_TILE + ( l & 7 ), j = tj * BORA_TILE + ( ( l >> 3 ) & 7 ), k = tk * BORA_TILE + ( l >> 6 );
        const float w = c.surf[n];
        c.pres[n] = w;
        if( w > 1e-30f )
        {
            const float x = c.cx[n] / w, y = c.cy[n] / w, z = c.cz[n] / w;
            c.cx[n] = x; c.cy[n] = y; c.cz[n] = z;
            const float dx = x - ( (float)i + .5f ), dy = y - ( (float)j + .5f ), dz = z - ( (float)k + .5f );
            c.surf[n] = sqrtf( dx * dx + dy * dy + dz * dz ) - 0.5f;  // Vec3f::distanceTo, Vector3.h:364-367
            c.vx[n] = c.vx[n] / w; c.vy[n] = c.vy[n] / w; c.vz[n] = c.vz[n] / w;
        }
        else
        {
            c.surf[n] = 5.f;
            c.vx[n] = 0.f; c.vy[n] = 0.f; c.vz[n] = 0.f;
        }
    }
}

// ======================================================================================
// The water tank's scan (FLIPMethod.cu:322-366): air cells (surf > 0; inactive tiles
// read the background 10) at or below the wall that no path of air cells connects to the
// wall layer (or to the grid's far corner, when that lies at or below the wall) become
// liquid (surf = -5). The reference finds the reached cells with a serial depth-first
// fill on the host; here the air cells of the slab j <= W form a union-find forest
// (labels only ever point to smaller indices, links by compare-and-swap), every seed
// marks its root, and unmarked roots' cells are filled. Nodes: active cells by storage
// index, then one node per inactive tile (all of its slab cells are air and connected).
constexpr uint32_t kRootMark = 0x80000000u;
constexpr uint32_t kLabelMask = 0x7FFFFFFFu;
constexpr int kUnionTries = 1 << 16;

struct TankSlab
{
    int W;          // highest slab row: min(wall, ny - 1)
    int layer;      // 1: row `W` is the wall layer (wall < ny) and seeds the fill
    int corner;     // 1: the far corner lies at or below the wall and seeds its neighbours
    uint32_t ncell; // first inactive-tile node
};

// Root of x, halving the path on the way (every store writes an ancestor of a non-root,
// so concurrent walks and links stay consistent). Loads bypass L1: links made by other
// SMs are seen sooner; a stale label is still an ancestor.
__device__ inline uint32_t uf_find( uint32_t* L, uint32_t x )
{
    uint32_t cur = __ldcg( L + x ) & kLabelMask;
    if( cur == x ) return x;
    uint32_t prev = x;
    for( ;; )
    {
        const uint32_t next = __ldcg( L + cur ) & kLabelMask;
        if( next == cur ) return cur;
        L[prev] = next;
        prev = cur;
        cur = next;
    }
}

// Link the trees of a and b (the larger root under the smaller). Each failed
// compare-and-swap moves to a strictly smaller root, so the loop ends; the bound only
// guards against a broken invariant.
__device__ inline void uf_union( uint32_t* L, uint32_t a, uint32_t b, uint32_t* err )
{
    for( int it = 0; it < kUnionTries; ++it )
    {
        a = uf_find( L, a );
        b = uf_find( L, b );
        if( a == b ) return;
        if( a > b ) { const uint32_t tmp = a; a = b; b = tmp; }
        const uint32_t old = atomicCAS( L + b, b, a );
        if( old == b ) return;
        b = old & kLabelMask;
    }
    atomicOr( err, 1u );
}

__global__ void k_uf_init( size_t nnodes, uint32_t* __restrict__ L )
{
    for( size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < nnodes; n += (size_t)gridDim.x * blockDim.x )
        L[n] = (uint32_t)n;
}

// Air cell of an active tile: link it to its air neighbours in the slab (active
// neighbours on the + side only, so each pair is linked once; inactive tiles' nodes on
// every side, as they run no thread of their own).
__global__ void k_uf_cells( const __grid_constant__ BoraGridDev g, BoraTilesDev t, size_t ncell,
                            const float* __restrict__ surf, TankSlab sl, uint32_t* L, uint32_t* err )
{
    for( size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < ncell; n += (size_t)gridDim.x * blockDim.x )
    {
        const int s = (int)( n / BORA_TILE_CELLS ), l = (int)( n % BORA_TILE_CELLS );
        const int vt = t.tile_of[s];
        int ti, tj, tk;
        tile_coords( g, vt, ti, tj, tk );
        const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
        const int i = ti * BORA_TILE + li, j = tj * BORA_TILE + lj, k = tk * BORA_TILE + lk;
        if( i >= g.nx || j > sl.W || k >= g.nz ) continue;
        if( !( surf[n] > 0.f ) ) continue;
        for( int d = 0; d < 6; ++d )
        {
            const int ax = d >> 1, sg = ( d & 1 ) ? 1 : -1;
            const int i2 = i + ( ax == 0 ? sg : 0 ), j2 = j + ( ax == 1 ? sg : 0 ), k2 = k + ( ax == 2 ? sg : 0 );
            if( i2 < 0 || j2 < 0 || k2 < 0 || i2 >= g.nx || j2 > sl.W || k2 >= g.nz ) continue;
            const int li2 = li + ( i2 - i ), lj2 = lj + ( j2 - j ), lk2 = lk + ( k2 - k );
            const int dt_ = bora_dir( li2 < 0 ? -1 : ( li2 > 7 ? 1 : 0 ), lj2 < 0 ? -1 : ( lj2 > 7 ? 1 : 0 ),
                                      lk2 < 0 ? -1 : ( lk2 > 7 ? 1 : 0 ) );
            const int s2 = t.nbr[(size_t)s * 27 + dt_];
            if( s2 >= 0 )
            {
                if( sg < 0 ) continue;
                const size_t m = (size_t)s2 * BORA_TILE_CELLS + (size_t)bora_local( i2, j2, k2 );
                if( surf[m] > 0.f ) uf_union( L, (uint32_t)n, (uint32_t)m, err );
            }
            else
            {
                const int vt2 = ( ( k2 >> 3 ) * g.ty + ( j2 >> 3 ) ) * g.tx + ( i2 >> 3 );
                uf_union( L, (uint32_t)n, sl.ncell + (uint32_t)vt2, err );
            }
        }
    }
}

// Inactive tile in the slab: link it to the inactive tiles after it on each axis that
// share air cells of the slab with it.
__global__ void k_uf_tiles( const __grid_constant__ BoraGridDev g, const int32_t* __restrict__ slot_of, TankSlab sl,
                            uint32_t* L, uint32_t* err )
{
    const size_t ntv = (size_t)g.tx * g.ty * g.tz;
    for( size_t vt = blockIdx.x * (size_t)blockDim.x + threadIdx.x; vt < ntv; vt += (size_t)gridDim.x * blockDim.x )
    {
        if( slot_of[vt] >= 0 ) continue;
        int ti, tj, tk;
        tile_coords( g, (int)vt, ti, tj, tk );
        if( tj * BORA_TILE > sl.W ) continue;
        const uint32_t a = sl.ncell + (uint32_t)vt;
        if( ti + 1 < g.tx && slot_of[vt + 1] < 0 ) uf_union( L, a, a + 1, err );
        if( tk + 1 < g.tz && slot_of[vt + (size_t)g.tx * g.ty] < 0 ) uf_union( L, a, a + (uint32_t)( g.tx * g.ty ), err );
        if( tj + 1 < g.ty && ( tj + 1 ) * BORA_TILE <= sl.W && slot_of[vt + g.tx] < 0 )
            uf_union( L, a, a + (uint32_t)g.tx, err );
    }
}

// Every label set to its root. The walk only reads: a concurrent halving store could
// otherwise replace a root that another thread has just written with an inner ancestor.
__global__ void k_uf_flatten( size_t nnodes, uint32_t* L )
{
    for( size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < nnodes; n += (size_t)gridDim.x * blockDim.x )
    {
        uint32_t x = (uint32_t)n, y = __ldcg( L + x );
        while( y != x ) { x = y; y = __ldcg( L + x ); }
        L[n] = x;
    }
}

// Node of an in-grid cell and whether it is air.
__device__ inline uint32_t tank_node( const BoraGridDev& g, const int32_t* slot_of, const float* surf, uint32_t ncell,
                                      int i, int j, int k, bool& air )
{
    const int vt = ( ( k >> 3 ) * g.ty + ( j >> 3 ) ) * g.tx + ( i >> 3 );
    const int s = slot_of[vt];
    if( s < 0 )
    {
        air = true;
        return ncell + (uint32_t)vt;
    }
    const uint32_t n = (uint32_t)s * BORA_TILE_CELLS + (uint32_t)bora_local( i, j, k );
    air = surf[n] > 0.f;
    return n;
}

// Seeds: the air cells of the wall layer and the air neighbours of the far corner.
__global__ void k_uf_seed( const __grid_constant__ BoraGridDev g, const int32_t* __restrict__ slot_of,
                           const float* __restrict__ surf, TankSlab sl, uint32_t* L )
{
    const size_t nl = (size_t)g.nx * g.nz;
    for( size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nl + 1; q += (size_t)gridDim.x * blockDim.x )
    {
        if( q < nl )
        {
            if( !sl.layer ) continue;
            bool air;
            const uint32_t n = tank_node( g, slot_of, surf, sl.ncell, (int)( q % g.nx ), sl.W, (int)( q / g.nx ), air );
            if( air ) atomicOr( L + ( L[n] & kLabelMask ), kRootMark );
        }
        else if( sl.corner )
        {
            const int ci = g.nx - 1, cj = g.ny - 1, ck = g.nz - 1;
            for( int d = 0; d < 4; ++d )  // the corner itself, then -x, -y, -z
            {
                const int i = ci - ( d == 1 ), j = cj - ( d == 2 ), k = ck - ( d == 3 );
                if( i < 0 || j < 0 || k < 0 ) continue;
                bool air;
                const uint32_t n = tank_node( g, slot_of, surf, sl.ncell, i, j, k, air );
                if( air ) atomicOr( L + ( L[n] & kLabelMask ), kRootMark );
            }
        }
    }
}

__global__ void k_uf_apply( const __grid_constant__ BoraGridDev g, BoraTilesDev t, size_t ncell, float* __restrict__ surf,
                            TankSlab sl, const uint32_t* __restrict__ L )
{
    for( size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < ncell; n += (size_t)gridDim.x * blockDim.x )
    {
        int ti, tj, tk;
        tile_coords( g, t.tile_of[n / BORA_TILE_CELLS], ti, tj, tk );
        const int l = (int)( n % BORA_TILE_CELLS );
        const int i = ti * BORA_TILE + ( l & 7 ), j = tj * BORA_TILE + ( ( l >> 3 ) & 7 ), k = tk * BORA_TILE + ( l >> 6 );
        if( i >= g.nx || j > sl.W || k >= g.nz ) continue;
        if( !( surf[n] > 0.f ) ) continue;
        if( !( L[L[n] & kLabelMask] & kRootMark ) ) surf[n] = -5.f;
    }
}

// ======================================================================================
// Stencil kernels: one CTA of 512 threads per tile, a 10^3 staged region (the tile and a
// one-cell halo), one cell per thread.
constexpr int kQ = 10;
constexpr int kQN = kQ * kQ * kQ;

__device__ inline size_t halo_index( const int32_t* nb, int h )  // storage index of region cell h, or SIZE_MAX
{
    const int a = h % kQ, b = ( h / kQ ) % kQ, cc = h / ( kQ * kQ );
    const int ns = nb[bora_dir( a == 0 ? -1 : ( a == 9 ? 1 : 0 ), b == 0 ? -1 : ( b == 9 ? 1 : 0 ),
                                cc == 0 ? -1 : ( cc == 9 ? 1 : 0 ) )];
    if( ns < 0 ) return SIZE_MAX;
    return (size_t)ns * BORA_TILE_CELLS + (size_t)bora_local( a + 7, b + 7, cc + 7 );
}

// Rasterization::ReinitializeSurface (base/source/Rasterization.cu:400-486), one step:
// Godunov upwind update of phi_t = sign(phi)(1 - |grad phi|), dt 0.3, sign =
// phi / sqrt(phi^2 + 1); differences mirrored at the grid faces, or for the water tank
// the faces read the level y - wall (minus / plus one below / above the grid).
template <bool TANK>
__global__ void __launch_bounds__( 512 ) k_redistance( const __grid_constant__ BoraGridDev g, BoraTilesDev t,
                                                        const float* __restrict__ in, float* __restrict__ out )
{
    __shared__ float r[kQN];
    __shared__ int32_t nb[27];
    const int s = blockIdx.x, tid = threadIdx.x;
    bora_pdl_trigger();
    if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    __syncthreads();
    size_t src[2];
    for( int u = 0; u < 2; ++u ) src[u] = tid + u * 512 < kQN ? halo_index( nb, tid + u * 512 ) : SIZE_MAX;
    bora_pdl_wait();
    for( int u = 0; u < 2; ++u )
        if( tid + u * 512 < kQN ) r[tid + u * 512] = src[u] == SIZE_MAX ? 10.f : in[src[u]];
    __syncthreads();
    const int li = tid & 7, lj = ( tid >> 3 ) & 7, lk = tid >> 6;
    const int i = ti * BORA_TILE + li, j = tj * BORA_TILE + lj, k = tk * BORA_TILE + lk;
    const int h = ( li + 1 ) + kQ * ( ( lj + 1 ) + kQ * ( lk + 1 ) );
    const float v = r[h];
    const size_t n = (size_t)s * BORA_TILE_CELLS + tid;
    if( i >= g.nx || j >= g.ny || k >= g.nz )
    {
        out[n] = v;
        return;
    }
    const int I = g.nx - 1, J = g.ny - 1, K = g.nz - 1;
    float vi0, vi1, vj0, vj1, vk0, vk1;
    if( TANK )
    {
        const float ll = ( (float)j + .5f ) - g.voxel_wall;
        vj0 = j == 0 ? ll - 1.f : r[h - kQ];
        vj1 = j == J ? ll + 1.f : r[h + kQ];
        vi0 = i == 0 ? ll : r[h - 1];
        vi1 = i == I ? ll : r[h + 1];
        vk0 = k == 0 ? ll : r[h - kQ * kQ];
        vk1 = k == K ? ll : r[h + kQ * kQ];
    }
    else
    {
        vi0 = i == 0 ? 2.f * v - r[h + 1] : r[h - 1];
        vi1 = i == I ? 2.f * v - r[h - 1] : r[h + 1];
        vj0 = j == 0 ? 2.f * v - r[h + kQ] : r[h - kQ];
        vj1 = j == J ? 2.f * v - r[h - kQ] : r[h + kQ];
        vk0 = k == 0 ? 2.f * v - r[h + kQ * kQ] : r[h - kQ * kQ];
        vk1 = k == K ? 2.f * v - r[h - kQ * kQ] : r[h + kQ * kQ];
    }
    const float dx0 = v - vi0, dx1 = vi1 - v, dy0 = v - vj0, dy1 = vj1 - v, dz0 = v - vk0, dz1 = vk1 - v;
    const float sign = v / sqrtf( v * v + 1.f );
    float a = maxr( dx0, 0.f ) * maxr( dx0, 0.f );
    a = a + minr( dx1, 0.f ) * minr( dx1, 0.f );
    a = a + maxr( dy0, 0.f ) * maxr( dy0, 0.f );
    a = a + minr( dy1, 0.f ) * minr( dy1, 0.f );
    a = a + maxr( dz0, 0.f ) * maxr( dz0, 0.f );
    a = a + minr( dz1, 0.f ) * minr( dz1, 0.f );
    float b = minr( dx0, 0.f ) * minr( dx0, 0.f );
    b = b + maxr( dx1, 0.f ) * maxr( dx1, 0.f );
    b = b + minr( dy0, 0.f ) * minr( dy0, 0.f );
    b = b + maxr( dy1, 0.f ) * maxr( dy1, 0.f );
    b = b + minr( dz0, 0.f ) * minr( dz0, 0.f );
    b = b + maxr( dz1, 0.f ) * maxr( dz1, 0.f );
    const float dt = 0.3f;
    out[n] = ( v - dt * maxr( sign, 0.f ) * ( sqrtf( a ) - 1.f ) ) - dt * minr( sign, 0.f ) * ( sqrtf( b ) - 1.f );
}

// FieldOP::curl of the splatted velocity (base/source/FieldOP.cu:338-369; background 0)
// into the curl arrays, and FieldOP::normalGradient of the surface (FieldOP.cu:79-110;
// background 10), normalised as Vec3f::normalized (Vector3.h:350-354), into comp.
__global__ void __launch_bounds__( 512 ) k_curl_normal( const __grid_constant__ BoraGridDev g, BoraTilesDev t,
                                                         BoraCellsDev c, float* __restrict__ wx, float* __restrict__ wy,
                                                         float* __restrict__ wz )
{
    __shared__ float fu[kQN], fv[kQN], fw[kQN], fs[kQN];
    __shared__ int32_t nb[27];
    const int s = blockIdx.x, tid = threadIdx.x;
    if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    __syncthreads();
    for( int h = tid; h < kQN; h += 512 )
    {
        const size_t q = halo_index( nb, h );
        const bool ok = q != SIZE_MAX;
        fu[h] = ok ? c.vx[q] : 0.f;
        fv[h] = ok ? c.vy[q] : 0.f;
        fw[h] = ok ? c.vz[q] : 0.f;
        fs[h] = ok ? c.surf[q] : 10.f;
    }
    __syncthreads();
    const int li = tid & 7, lj = ( tid >> 3 ) & 7, lk = tid >> 6;
    const int i = ti * BORA_TILE + li, j = tj * BORA_TILE + lj, k = tk * BORA_TILE + lk;
    if( i >= g.nx || j >= g.ny || k >= g.nz ) return;
    const int h = ( li + 1 ) + kQ * ( ( lj + 1 ) + kQ * ( lk + 1 ) );
    const size_t n = (size_t)s * BORA_TILE_CELLS + tid;
    const int I = g.nx - 1, J = g.ny - 1, K = g.nz - 1;
    const int sx = 1, sy = kQ, sz = kQ * kQ;
    // neighbour value of f on the low / high side at stride o, mirrored at a grid face
    auto lo = [&]( const float* f, bool face, int o ) { return face ? f[h] * 2.f - f[h + o] : f[h - o]; };
    auto hi = [&]( const float* f, bool face, int o ) { return face ? f[h] * 2.f - f[h - o] : f[h + o]; };
    const bool fi0 = i == 0, fi1 = i == I, fj0 = j == 0, fj1 = j == J, fk0 = k == 0, fk1 = k == K;
    const float x1y = hi( fv, fi1, sx ), x0y = lo( fv, fi0, sx ), x1z = hi( fw, fi1, sx ), x0z = lo( fw, fi0, sx );
    const float y1x = hi( fu, fj1, sy ), y0x = lo( fu, fj0, sy ), y1z = hi( fw, fj1, sy ), y0z = lo( fw, fj0, sy );
    const float z1x = hi( fu, fk1, sz ), z0x = lo( fu, fk0, sz ), z1y = hi( fv, fk1, sz ), z0y = lo( fv, fk0, sz );
    wx[n] = ( y1z - y0z ) * 0.5f - ( z1y - z0y ) * 0.5f;
    wy[n] = ( z1x - z0x ) * 0.5f - ( x1z - x0z ) * 0.5f;
    wz[n] = ( x1y - x0y ) * 0.5f - ( y1x - y0x ) * 0.5f;
    const float v = fs[h];
    const float vi0 = fi0 ? 2.f * v - fs[h + sx] : fs[h - sx], vi1 = fi1 ? 2.f * v - fs[h - sx] : fs[h + sx];
    const float vj0 = fj0 ? 2.f * v - fs[h + sy] : fs[h - sy], vj1 = fj1 ? 2.f * v - fs[h - sy] : fs[h + sy];
    const float vk0 = fk0 ? 2.f * v - fs[h + sz] : fs[h - sz], vk1 = fk1 ? 2.f * v - fs[h - sz] : fs[h + sz];
    const float gx = ( vi1 - vi0 ) * 0.5f, gy = ( vj1 - vj0 ) * 0.5f, gz = ( vk1 - vk0 ) * 0.5f;
    const float d = 1.f / sqrtf( gx * gx + gy * gy + gz * gz + 1e-30f );
    c.cx[n] = gx * d;
    c.cy[n] = gy * d;
    c.cz[n] = gz * d;
}

// FieldOP::curvature of the normals (FieldOP.cu:273-301; background 0) into pres.
__global__ void __launch_bounds__( 512 ) k_curvature( const __grid_constant__ BoraGridDev g, BoraTilesDev t, BoraCellsDev c )
{
    __shared__ float fx[kQN], fy[kQN], fz[kQN];
    __shared__ int32_t nb[27];
    const int s = blockIdx.x, tid = threadIdx.x;
    if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    __syncthreads();
    for( int h = tid; h < kQN; h += 512 )
    {
        const size_t q = halo_index( nb, h );
        const bool ok = q != SIZE_MAX;
        fx[h] = ok ? c.cx[q] : 0.f;
        fy[h] = ok ? c.cy[q] : 0.f;
        fz[h] = ok ? c.cz[q] : 0.f;
    }
    __syncthreads();
    const int li = tid & 7, lj = ( tid >> 3 ) & 7, lk = tid >> 6;
    const int i = ti * BORA_TILE + li, j = tj * BORA_TILE + lj, k = tk * BORA_TILE + lk;
    const size_t n = (size_t)s * BORA_TILE_CELLS + tid;
    if( i >= g.nx || j >= g.ny || k >= g.nz )
    {
        c.pres[n] = 0.f;
        return;
    }
    const int h = ( li + 1 ) + kQ * ( ( lj + 1 ) + kQ * ( lk + 1 ) );
    const int sy = kQ, sz = kQ * kQ;
    const float si0 = i == 0 ? fx[h] * 2.f - fx[h + 1] : fx[h - 1];
    const float si1 = i == g.nx - 1 ? fx[h] * 2.f - fx[h - 1] : fx[h + 1];
    const float sj0 = j == 0 ? fy[h] * 2.f - fy[h + sy] : fy[h - sy];
    const float sj1 = j == g.ny - 1 ? fy[h] * 2.f - fy[h - sy] : fy[h + sy];
    const float sk0 = k == 0 ? fz[h] * 2.f - fz[h + sz] : fz[h - sz];
    const float sk1 = k == g.nz - 1 ? fz[h] * 2.f - fz[h - sz] : fz[h + sz];
    c.pres[n] = ( si1 - si0 ) * 0.5f + ( sj1 - sj0 ) * 0.5f + ( sk1 - sk0 ) * 0.5f;
}

// SparseField::lerp (base/header/SparseField.h:150-173) through the tile table.
struct CellLerp
{
    int64_t q[8];  // (i,j,k) (i+1,j,k) (i,j,k+1) (i+1,j,k+1) (i,j+1,k) (i+1,j+1,k) (i,j+1,k+1) (i+1,j+1,k+1); -1 = background
    float x, y, z;
    __device__ inline void setup( const BoraGridDev& g, const int32_t* slot_of, float px, float py, float pz )
    {
        const int i = bora_clampi( bora_trunc( px - 0.5f ), 0, g.nx - 2 );
        const int j = bora_clampi( bora_trunc( py - 0.5f ), 0, g.ny - 2 );
        const int k = bora_clampi( bora_trunc( pz - 0.5f ), 0, g.nz - 2 );
        x = bora_clampf( px - ( (float)i + .5f ), 0.f, 1.f );
        y = bora_clampf( py - ( (float)j + .5f ), 0.f, 1.f );
        z = bora_clampf( pz - ( (float)k + .5f ), 0.f, 1.f );
        for( int c = 0; c < 8; ++c )
        {
            const int a = i + ( c & 1 ), b = j + ( c >> 2 ), e = k + ( ( c >> 1 ) & 1 );
            const int s = slot_of[( (size_t)( e >> 3 ) * g.ty + ( b >> 3 ) ) * g.tx + ( a >> 3 )];
            q[c] = s < 0 ? -1 : (int64_t)s * BORA_TILE_CELLS + bora_local( a, b, e );
        }
    }
    __device__ inline float lerp( const float* f, float bg ) const
    {
        float v[8];
        for( int c = 0; c < 8; ++c ) v[c] = q[c] < 0 ? bg : f[q[c]];
        const float c00 = v[0] * ( 1.f - x ) + v[1] * x;
        const float c01 = v[2] * ( 1.f - x ) + v[3] * x;
        const float c10 = v[4] * ( 1.f - x ) + v[5] * x;
        const float c11 = v[6] * ( 1.f - x ) + v[7] * x;
        const float c0 = c00 * ( 1.f - y ) + c10 * y;
        const float c1 = c01 * ( 1.f - y ) + c11 * y;
        return c0 * ( 1.f - z ) + c1 * z;
    }
};

// FLIPMethod.cu:378-403 per particle: vorticity = max(|world curl| - 0.2 (>= 0),
// vorticity (1 - dis)), curvature = the curvature field at the particle (pres, whose
// background ReinitializeSurface left at 10).
__global__ void k_particle_attributes( const __grid_constant__ BoraGridDev g, const int32_t* __restrict__ slot_of, size_t np,
                                       BoraParticlesDev p, const float* __restrict__ wx, const float* __restrict__ wy,
                                       const float* __restrict__ wz, const float* __restrict__ curvature, float3 scale,
                                       float dis )
{
    for( size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < np; q += (size_t)gridDim.x * blockDim.x )
    {
        if( p.id[q] < 0 ) continue;
        CellLerp L;
        L.setup( g, slot_of, p.px[q], p.py[q], p.pz[q] );
        const float cx = L.lerp( wx, 0.f ) * scale.x, cy = L.lerp( wy, 0.f ) * scale.y, cz = L.lerp( wz, 0.f ) * scale.z;
        float v = sqrtf( cx * cx + cy * cy + cz * cz );
        v = maxr( 0.f, v - 0.2f );
        float o = p.vort[q];
        o -= o * dis;
        p.vort[q] = maxr( v, o );
        p.curv[q] = L.lerp( curvature, 10.f );
    }
}

int blocks_for_cells( size_t n )
{
    return (int)std::max<size_t>( 1, std::min<size_t>( ( n + 255 ) / 256, (size_t)152 * 32 ) );
}

}  // namespace

void bora_launch_splat( const BoraGridDev& g, int ntiles, BoraTilesDev t, const uint32_t* start, const uint32_t* idx,
                        BoraParticlesDev p, BoraCellsDev c, cudaStream_t st )
{
    if( ntiles <= 0 ) return;
    k_splat<<<ntiles, kSplatThreads, 0, st>>>( g, t, start, idx, p, c );
    const size_t ncell = (size_t)ntiles * BORA_TILE_CELLS;
    k_splat_finish<<<blocks_for_cells( ncell ), 256, 0, st>>>( g, t, ncell, c );
}

int bora_tank_scan_launches( const BoraGridDev& g, int ntiles, BoraTilesDev t, float* surf, uint32_t* labels,
                             uint32_t* err, cudaStream_t st )
{
    if( ntiles <= 0 || !( g.voxel_wall >= 0.f ) ) return 0;
    const int wall = g.voxel_wall >= (float)g.ny ? g.ny : (int)g.voxel_wall;
    TankSlab sl;
    sl.W = std::min( wall, g.ny - 1 );
    sl.layer = wall < g.ny ? 1 : 0;
    sl.corner = wall >= g.ny - 1 ? 1 : 0;
    const size_t ncell = (size_t)ntiles * BORA_TILE_CELLS;
    const size_t ntv = (size_t)g.tx * g.ty * g.tz;
    sl.ncell = (uint32_t)ncell;
    const size_t nn = ncell + ntv;
    k_uf_init<<<blocks_for_cells( nn ), 256, 0, st>>>( nn, labels );
    k_uf_cells<<<blocks_for_cells( ncell ), 256, 0, st>>>( g, t, ncell, surf, sl, labels, err );
    k_uf_tiles<<<blocks_for_cells( ntv ), 256, 0, st>>>( g, t.slot_of, sl, labels, err );
    k_uf_flatten<<<blocks_for_cells( nn ), 256, 0, st>>>( nn, labels );
    k_uf_seed<<<blocks_for_cells( (size_t)g.nx * g.nz + 1 ), 256, 0, st>>>( g, t.slot_of, surf, sl, labels );
    k_uf_apply<<<blocks_for_cells( ncell ), 256, 0, st>>>( g, t, ncell, surf, sl, labels );
    return 6;
}

cudaError_t bora_launch_redistance( const BoraGridDev& g, int ntiles, BoraTilesDev t, const float* in, float* out,
                                    cudaStream_t st )
{
    if( ntiles <= 0 ) return cudaSuccess;
    if( g.enable_tank ) return bora_launch_pdl( k_redistance<true>, dim3( ntiles ), dim3( 512 ), 0, st, g, t, in, out );
    return bora_launch_pdl( k_redistance<false>, dim3( ntiles ), dim3( 512 ), 0, st, g, t, in, out );
}

void bora_launch_surface_fields( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, float* wx, float* wy,
                                 float* wz, cudaStream_t st )
{
    if( ntiles <= 0 ) return;
    k_curl_normal<<<ntiles, 512, 0, st>>>( g, t, c, wx, wy, wz );
    k_curvature<<<ntiles, 512, 0, st>>>( g, t, c );
}

void bora_launch_particle_attributes( const BoraGridDev& g, const int32_t* slot_of, size_t np, BoraParticlesDev p,
                                      const float* wx, const float* wy, const float* wz, const float* curvature,
                                      float3 scale, float dis, cudaStream_t st )
{
    if( np == 0 ) return;
    k_particle_attributes<<<blocks_for_cells( np ), 256, 0, st>>>( g, slot_of, np, p, wx, wy, wz, curvature, scale, dis );
}
