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

__device__ inline void tile_coords( const BoraGridDev& g, int vt, int& ti, int& tj, int& tk )
{
    ti = vt % g.tx;
    tj = ( vt / g.tx ) % g.ty;
    tk = vt / ( g.tx * g.ty );
}

// ======================================================================================
// Rasterization::ParticlesToSurfaceAndVelocity (base/source/Rasterization.cu:311-398),
// influence 1.5, droplet 0.5 (FLIPMethod.cu:320), as a gather. A particle p adds to the
// 3^3 cells around (int)p those within the kernel radius; a cell c is reached only from
// particles of dual cells c-2 .. c+1 per axis (dual cell = max(int(p - 0.5), 0), the
// sort's key). One CTA per tile owns the tile's 512 cells and walks the 11 dual-cell
// layers z = -2 .. 8 of its region: each layer's particles (11 x 11 dual cells, one
// contiguous sorted range each) are staged in shared memory, and the 256 cells the layer
// can reach (z - 1 .. z + 2) are worked on at once: a pair of z-adjacent cells per thread
// pair (the pair shares each candidate's x and y distances), the two threads of a pair
// taking two of the four candidate rows each. Layer sums go into per-cell shared sums in a
// fixed order, so the result is reproducible; no atomics, and the normalisation of
// Rasterization.cu:373-395 is applied on the way out.
constexpr int kSplatThreads = 256;
constexpr int kSplatCap = 1024;  // staged particles per pass (a layer with more takes several)
constexpr int kLayerCells = 121;  // 11 x 11 dual cells

// Kernel weight of Rasterization.cu:343-349, max(0, (1 - (d/1.5)^2)^3), evaluated as
// (1 - d^2 / 2.25)^3 with fused multiply-adds: the same function without the square root
// and the division (one weight's rounding differs by an ulp or two; the sums' order, open
// in the reference, moves them more). Zero for d^2 >= 2.25; a cell within that radius lies
// in the reference's 3^3 box around (int)p.
__global__ void __launch_bounds__( kSplatThreads ) k_splat( const __grid_constant__ BoraGridDev g, BoraTilesDev t,
                                                            const uint32_t* __restrict__ start,
                                                            const uint32_t* __restrict__ idx, BoraParticlesDev p,
                                                            BoraCellsDev c )
{
    __shared__ float4 sa[kSplatCap];  // x, y, z, u (x = -1e30: outside the grid)
    __shared__ float2 sb[kSplatCap];  // v, w
    __shared__ float accs[7][BORA_TILE_CELLS];  // per cell: w, w x, w y, w z, w u, w v, w w
    __shared__ uint32_t q0s[kLayerCells];
    __shared__ uint32_t off[kLayerCells + 1];
    __shared__ uint32_t wsum[4];
    __shared__ int32_t nb[27];
    const int s = blockIdx.x, tid = threadIdx.x;
    if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
    for( int h = tid; h < 7 * BORA_TILE_CELLS; h += kSplatThreads ) ( &accs[0][0] )[h] = 0.f;
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    // work item: cells (li, lj, zz - 1 + 2 pr) and (li, lj, zz + 2 pr); lanes l and l ^ 16
    // split its four candidate rows
    const int half = ( tid >> 4 ) & 1;
    const int item = ( tid & 15 ) | ( ( tid >> 5 ) << 4 );
    const int li = item & 7, lj = ( item >> 3 ) & 7, pr = item >> 6;
    const float cx = (float)( ti * BORA_TILE + li ) + .5f, cy = (float)( tj * BORA_TILE + lj ) + .5f;
    const float fnx = (float)g.nx, fny = (float)g.ny, fnz = (float)g.nz;
    __syncthreads();
    for( int zz = -2; zz <= 8; ++zz )
    {
        // particle ranges of the layer's dual cells (xx, yy) in -2..8, and their prefix sums
        uint32_t cnt = 0;
        if( tid < kLayerCells )
        {
            const int xx = tid % 11 - 2, yy = tid / 11 - 2;
            const int sl = nb[bora_dir( xx < 0 ? -1 : ( xx > 7 ? 1 : 0 ), yy < 0 ? -1 : ( yy > 7 ? 1 : 0 ),
                                        zz < 0 ? -1 : ( zz > 7 ? 1 : 0 ) )];
            uint32_t a = 0;
            if( sl >= 0 )
            {
                const uint32_t key = (uint32_t)sl * BORA_TILE_CELLS + (uint32_t)bora_local( xx & 7, yy & 7, zz & 7 );
                a = start[key];
                cnt = start[key + 1] - a;
            }
            q0s[tid] = a;
        }
        // exclusive scan over the 121 counts (warps 0..3)
        uint32_t inc = cnt;
        const int lane = tid & 31, wp = tid >> 5;
#pragma unroll
        for( int o = 1; o < 32; o <<= 1 )
        {
            const uint32_t y = __shfl_up_sync( 0xffffffffu, inc, o );
            if( lane >= o ) inc += y;
        }
        if( wp < 4 && lane == 31 ) wsum[wp] = inc;
        __syncthreads();
        if( tid < kLayerCells )
        {
            uint32_t base = 0;
            for( int w = 0; w < wp; ++w ) base += wsum[w];
            off[tid + 1] = base + inc;
            if( tid == 0 ) off[0] = 0;
        }
        __syncthreads();
        const uint32_t total = off[kLayerCells];
        const int z0 = zz - 1 + 2 * pr, z1 = z0 + 1;  // this item's cells
        const float cz0 = (float)( tk * BORA_TILE + z0 ) + .5f, cz1 = (float)( tk * BORA_TILE + z1 ) + .5f;
        float acc[2][7];
#pragma unroll
        for( int m = 0; m < 2; ++m )
#pragma unroll
            for( int v = 0; v < 7; ++v ) acc[m][v] = 0.f;
        for( uint32_t e0 = 0; e0 < total; e0 += kSplatCap )
        {
            const uint32_t e1 = min( total, e0 + kSplatCap );
            for( uint32_t e = e0 + tid; e < e1; e += kSplatThreads )
            {
                int lo = 0, hi = kLayerCells;  // dual cell d with off[d] <= e < off[d + 1]
                while( hi - lo > 1 )
                {
                    const int mid = ( lo + hi ) >> 1;
                    if( off[mid] <= e ) lo = mid;
                    else hi = mid;
                }
                const uint32_t pi = idx[q0s[lo] + ( e - off[lo] )];
                float x = p.px[pi];
                const float y = p.py[pi], z = p.pz[pi];
                // Grid::inside (Grid.h:408-417): a particle outside is moved out of every
                // cell's reach, so it adds weight 0 (and 0 * finite values) everywhere
                if( x < 0.f || x > fnx || y < 0.f || y > fny || z < 0.f || z > fnz ) x = -1e30f;
                sa[e - e0] = make_float4( x, y, z, p.vx[pi] );
                sb[e - e0] = make_float2( p.vy[pi], p.vz[pi] );
            }
            __syncthreads();
            // the 4 dual cells xx = li-2 .. li+1 of a row are adjacent in the staging
            for( int yy = lj - 2 + 2 * half; yy <= lj - 1 + 2 * half; ++yy )
            {
                const int d = li + 11 * ( yy + 2 );
                // the row's part of this pass, as staging indices (empty when the row lies
                // wholly before or after the pass)
                const uint32_t ga = max( off[d], e0 ), gb = min( off[d + 4], e1 );
                const uint32_t a = ga - e0, b = gb > ga ? gb - e0 : a;
                // branch-free: a particle outside the radius (or the grid) adds weight 0
                auto add = [&]( uint32_t e ) {
                    const float4 q = sa[e];
                    const float2 r = sb[e];
                    const float dx = q.x - cx, dy = q.y - cy, dz0 = q.z - cz0, dz1 = q.z - cz1;
                    const float h2 = fmaf( dy, dy, dx * dx );
                    const float t0 = fmaf( -fmaf( dz0, dz0, h2 ), 1.f / 2.25f, 1.f );
                    const float t1 = fmaf( -fmaf( dz1, dz1, h2 ), 1.f / 2.25f, 1.f );
                    const float w0 = t0 > 0.f ? t0 * t0 * t0 : 0.f, w1 = t1 > 0.f ? t1 * t1 * t1 : 0.f;
                    acc[0][0] += w0; acc[1][0] += w1;
                    acc[0][1] = fmaf( w0, q.x, acc[0][1] ); acc[1][1] = fmaf( w1, q.x, acc[1][1] );
                    acc[0][2] = fmaf( w0, q.y, acc[0][2] ); acc[1][2] = fmaf( w1, q.y, acc[1][2] );
                    acc[0][3] = fmaf( w0, q.z, acc[0][3] ); acc[1][3] = fmaf( w1, q.z, acc[1][3] );
                    acc[0][4] = fmaf( w0, q.w, acc[0][4] ); acc[1][4] = fmaf( w1, q.w, acc[1][4] );
                    acc[0][5] = fmaf( w0, r.x, acc[0][5] ); acc[1][5] = fmaf( w1, r.x, acc[1][5] );
                    acc[0][6] = fmaf( w0, r.y, acc[0][6] ); acc[1][6] = fmaf( w1, r.y, acc[1][6] );
                };
                uint32_t e = a;
                for( ; e + 2 <= b; e += 2 )
                {
                    add( e ); add( e + 1 );
                }
                if( e < b ) add( e );
            }
            __syncthreads();  // the staging buffer is reused by the next pass
        }
        // the two halves' sums, added in a fixed order into the cells' running sums (each
        // cell is owned by one item in a layer)
#pragma unroll
        for( int m = 0; m < 2; ++m )
        {
            const int zc = m == 0 ? z0 : z1;
#pragma unroll
            for( int v = 0; v < 7; ++v )
            {
                const float other = __shfl_xor_sync( 0xffffffffu, acc[m][v], 16 );
                if( half == 0 && zc >= 0 && zc <= 7 ) accs[v][li + 8 * lj + 64 * zc] += acc[m][v] + other;
            }
        }
        __syncthreads();  // the layer tables are rewritten next
    }
    // Rasterization.cu:373-395: mean position's distance to the centre - 0.5 (5 where no
    // weight landed), mean velocity; the weight sum goes to pres ("mass", FLIPMethod.cu:320)
#pragma unroll
    for( int m = 0; m < 2; ++m )
    {
        const int l = tid + 256 * m;
        const int i = ti * BORA_TILE + ( l & 7 ), j = tj * BORA_TILE + ( ( l >> 3 ) & 7 ), k = tk * BORA_TILE + ( l >> 6 );
        const size_t n = (size_t)s * BORA_TILE_CELLS + l;
        const bool real = i < g.nx && j < g.ny && k < g.nz;
        const float w = real ? accs[0][l] : 0.f;
        c.pres[n] = w;
        if( w > 1e-30f )
        {
            const float x = accs[1][l] / w, y = accs[2][l] / w, z = accs[3][l] / w;
            c.cx[n] = x; c.cy[n] = y; c.cz[n] = z;
            const float dx = x - ( (float)i + .5f ), dy = y - ( (float)j + .5f ), dz = z - ( (float)k + .5f );
            c.surf[n] = sqrtf( dx * dx + dy * dy + dz * dz ) - 0.5f;  // Vec3f::distanceTo, Vector3.h:364-367
            c.vx[n] = accs[4][l] / w; c.vy[n] = accs[5][l] / w; c.vz[n] = accs[6][l] / w;
        }
        else
        {
            c.cx[n] = real ? accs[1][l] : 0.f; c.cy[n] = real ? accs[2][l] : 0.f; c.cz[n] = real ? accs[3][l] : 0.f;
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

// One Godunov upwind step of Rasterization::ReinitializeSurface
// (base/source/Rasterization.cu:400-486) at a cell with value v and neighbours
// (i0, i1, j0, j1, k0, k1): phi_t = sign(phi)(1 - |grad phi|), dt 0.3,
// sign = phi / sqrt(phi^2 + 1). Of the reference's two terms
// dt max(sign,0)(sqrt(a) - 1) and dt min(sign,0)(sqrt(b) - 1) one has a zero factor; its
// value is the signed zero (+0) * (sqrt(x) - 1), whose sign is that of x - 1, so only the
// other square root is taken.
__device__ inline float godunov_step( float v, float vi0, float vi1, float vj0, float vj1, float vk0, float vk1 )
{
    const float dx0 = v - vi0, dx1 = vi1 - v, dy0 = v - vj0, dy1 = vj1 - v, dz0 = v - vk0, dz1 = vk1 - v;
    const float sign = v / sqrtf( v * v + 1.f );
    const float dt = 0.3f;
    const float ps = maxr( sign, 0.f ), ns = minr( sign, 0.f );
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
    const float zp = a < 1.f ? -0.f : 0.f, zn = b < 1.f ? -0.f : 0.f;
    const bool pos = ps != 0.f;  // sign > 0: the first term is live
    const bool neg = ns != 0.f;  // sign < 0: the second
    const float t1 = pos ? dt * ps * ( sqrtf( a ) - 1.f ) : zp;
    const float t2 = neg ? dt * ns * ( sqrtf( b ) - 1.f ) : zn;
    return ( v - t1 ) - t2;
}

// Redistancing, one step over all tiles: a persistent grid walks the tiles; each tile's
// 10^3 region (the tile and a one-cell halo, background 10 for inactive tiles) is read
// into registers one tile ahead, so the loads of the next tile overlap the arithmetic of
// the current one.
constexpr int kRedistThreads = 512;

template <bool TANK>
__global__ void __launch_bounds__( kRedistThreads ) k_redistance( const __grid_constant__ BoraGridDev g, BoraTilesDev t,
                                                                   int ntiles, const float* __restrict__ in,
                                                                   float* __restrict__ out )
{
    __shared__ float r[kQN];
    __shared__ int32_t nbb[2][27];
    __shared__ int tcb[2][3];  // tile coordinates, double-buffered like the neighbour tables
    const int tid = threadIdx.x, G = gridDim.x;
    bora_pdl_trigger();
    if( tid < 27 )
    {
        nbb[0][tid] = blockIdx.x < ntiles ? t.nbr[(size_t)blockIdx.x * 27 + tid] : -1;
        nbb[1][tid] = blockIdx.x + G < ntiles ? t.nbr[(size_t)( blockIdx.x + G ) * 27 + tid] : -1;
    }
    else if( tid == 32 || tid == 33 )
    {
        const int q = tid - 32, sq = blockIdx.x + q * G;
        if( sq < ntiles ) tile_coords( g, t.tile_of[sq], tcb[q][0], tcb[q][1], tcb[q][2] );
    }
    __syncthreads();
    bora_pdl_wait();  // `in` is the previous step's output
    // this thread's two region cells: tile direction and local index, the same for every tile
    int rdir[2], rloc[2];
    for( int u = 0; u < 2; ++u )
    {
        const int hh = tid + u * kRedistThreads;
        const int a = hh % kQ, b = ( hh / kQ ) % kQ, c = hh / ( kQ * kQ );
        rdir[u] = hh < kQN ? bora_dir( a == 0 ? -1 : ( a == 9 ? 1 : 0 ), b == 0 ? -1 : ( b == 9 ? 1 : 0 ),
                                       c == 0 ? -1 : ( c == 9 ? 1 : 0 ) )
                           : -1;
        rloc[u] = bora_local( a + 7, b + 7, c + 7 );
    }
    float pf[2];
    auto issue = [&]( const int32_t* nb ) {
        for( int u = 0; u < 2; ++u )
        {
            const int ns = rdir[u] >= 0 ? nb[rdir[u]] : -1;
            pf[u] = ns >= 0 ? in[(size_t)ns * BORA_TILE_CELLS + rloc[u]] : 10.f;
        }
    };
    issue( nbb[0] );
    const int li = tid & 7, lj = ( tid >> 3 ) & 7, lk = tid >> 6;
    const int h = ( li + 1 ) + kQ * ( ( lj + 1 ) + kQ * ( lk + 1 ) );
    const int I = g.nx - 1, J = g.ny - 1, K = g.nz - 1;
    int n = 0;
    for( int s = blockIdx.x; s < ntiles; s += G, ++n )
    {
        for( int u = 0; u < 2; ++u )
            if( tid + u * kRedistThreads < kQN ) r[tid + u * kRedistThreads] = pf[u];
        const int32_t nb2 = tid < 27 && s + 2 * G < ntiles ? t.nbr[(size_t)( s + 2 * G ) * 27 + tid] : -1;
        int tc2[3] = { 0, 0, 0 };
        if( tid == 32 && s + 2 * G < ntiles ) tile_coords( g, t.tile_of[s + 2 * G], tc2[0], tc2[1], tc2[2] );
        __syncthreads();
        if( s + G < ntiles ) issue( nbb[( n + 1 ) & 1] );
        const int ti = tcb[n & 1][0], tj = tcb[n & 1][1], tk = tcb[n & 1][2];
        const int i = ti * BORA_TILE + li, j = tj * BORA_TILE + lj, k = tk * BORA_TILE + lk;
        const float v = r[h];
        float res = v;
        if( i < g.nx && j < g.ny && k < g.nz )
        {
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
            res = godunov_step( v, vi0, vi1, vj0, vj1, vk0, vk1 );
        }
        out[(size_t)s * BORA_TILE_CELLS + tid] = res;
        __syncthreads();  // tile s's tables and region are no longer read
        if( tid < 27 ) nbb[n & 1][tid] = nb2;
        if( tid == 32 ) { tcb[n & 1][0] = tc2[0]; tcb[n & 1][1] = tc2[1]; tcb[n & 1][2] = tc2[2]; }
    }
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

template <bool TANK>
int redistance_grid( int ntiles )
{
    static BoraPerDevice per_sm;
    const int b = per_sm.get( [] {
        int v = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor( &v, k_redistance<TANK>, kRedistThreads, 0 ) == cudaSuccess && v > 0 ? v : 1;
    } );
    int dev = 0, sms = 0;
    cudaGetDevice( &dev );
    cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
    return std::max( 1, std::min( ntiles, b * std::max( sms, 1 ) ) );
}

cudaError_t bora_launch_redistance( const BoraGridDev& g, int ntiles, BoraTilesDev t, const float* in, float* out,
                                    cudaStream_t st )
{
    if( ntiles <= 0 ) return cudaSuccess;
    if( g.enable_tank )
        return bora_launch_pdl( k_redistance<true>, dim3( redistance_grid<true>( ntiles ) ), dim3( kRedistThreads ), 0, st,
                                g, t, ntiles, in, out );
    return bora_launch_pdl( k_redistance<false>, dim3( redistance_grid<false>( ntiles ) ), dim3( kRedistThreads ), 0, st,
                            g, t, ntiles, in, out );
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
