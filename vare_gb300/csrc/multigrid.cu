// Geometric multigrid V-cycle preconditioner for the pressure PCG, with FP16 storage
// and FP32 arithmetic (the mixed-precision form of the projection).
//
// The reference's pressure solve is unpreconditioned FP32 CG
// (base/source/LinearSystemSolver.cpp:12-50); its only preconditioner is a serial MIC(0)
// (base/source/BLAS.cu:211-331). This V-cycle replaces both for the mixed form.
//
// Hierarchy: level 0 is the fine grid of active 8^3 tiles; levels 1..3 keep the tile
// layout with 4^3, 2^3 and 1 cell per tile (neighbours across tiles through the tile
// neighbour table); levels >= 4 are small dense grids over the tile grid halved per
// level. A coarse cell is air (Dirichlet) if any child is air (inactive tiles count as
// air), else fluid if any child is fluid, else solid. Every level applies the reference's
// 7-point rule (diagonal 6 + #air - #solid/wall, -1 per fluid neighbour,
// FluidProjection.cu:234-244) to its own cell types; coarse operators are the
// rediscretisation with spacing 2^l, i.e. the same stencil divided by 4^l.
//
// All quantities are kept in "stencil units" (the level equation S z = r' with
// S = diag*z - sum of fluid neighbours): restriction averages the children's residuals
// and multiplies by 4, prolongation injects the coarse correction. Smoothing is two
// Jacobi sweeps before and after with Chebyshev weights (kOmegaA, kOmegaB below); the
// coarsest level (<= 512 cells) gets 16 damped Jacobi sweeps. Level residuals and corrections are stored as FP16: the fine residual
// is scaled by 1/||r||_2 on entry so every stored value is O(1). Residuals restricted to
// non-fluid coarse cells are never read (their z is zero), so the restriction does not
// look at the coarse types.
#include <algorithm>

#include <cuda_fp16.h>

#include "bora_internal.h"
#include "reduce.cuh"

namespace {

// Smoothing: the two Jacobi sweeps of each pre- and post-smoother take the weights of the
// degree-2 Chebyshev polynomial in D^-1 A over [0.35, 2] (roots 1.175 -+ 0.825 cos(pi/4)):
// the pre-smoother sweeps with kOmegaA then kOmegaB, the post-smoother with kOmegaB then
// kOmegaA. The two factors commute, so each level's post-smoother is the adjoint of its
// pre-smoother and the V-cycle stays symmetric. Against two sweeps of damped Jacobi
// (omega 0.9) this cut the PCG iterations of the dam-break scenes by a fifth at the same
// cost per V-cycle. The coarsest level keeps damped Jacobi with kOmega.
constexpr float kOmega = 0.9f;
constexpr float kOmegaA = 0.5687f;  // 1 / (1.175 + 0.825 cos(pi/4))
constexpr float kOmegaB = 1.6902f;  // 1 / (1.175 - 0.825 cos(pi/4))

__device__ inline int code_diag( uint16_t c ) { return ( c >> 8 ) & 15; }

// Index of the face neighbour q (0:-x 1:+x 2:-y 3:+y 4:-z 5:+z) of a cell on level L,
// or -1 when it lies in an inactive tile / beyond the stored grid.
struct LevelNav
{
    BoraLevelDev L;
    const int32_t* nbr;      // tile neighbour table (tiled levels)
    const int32_t* tile_of;  // slot -> virtual tile (tiled levels)
    int tx, ty;              // tile grid (tiled levels)

    __device__ inline void coords( long long cell, int& i, int& j, int& k ) const
    {
        if( L.kind == 1 )
        {
            i = (int)( cell % L.dx );
            j = (int)( ( cell / L.dx ) % L.dy );
            k = (int)( cell / ( (long long)L.dx * L.dy ) );
            return;
        }
        const int E = L.E, E3 = E * E * E;
        const int s = (int)( cell / E3 ), loc = (int)( cell % E3 );
        const int vt = tile_of[s];
        i = ( vt % tx ) * E + loc % E;
        j = ( ( vt / tx ) % ty ) * E + ( loc / E ) % E;
        k = ( vt / ( tx * ty ) ) * E + loc / ( E * E );
    }
    __device__ inline bool real( int i, int j, int k ) const { return i < L.nx && j < L.ny && k < L.nz; }

    // neighbour cell index, -1 inactive/outside storage; *edge = true beyond the domain
    __device__ inline long long nbr_index( long long cell, int i, int j, int k, int q, bool* edge ) const
    {
        const int di = q == 0 ? -1 : ( q == 1 ? 1 : 0 );
        const int dj = q == 2 ? -1 : ( q == 3 ? 1 : 0 );
        const int dk = q == 4 ? -1 : ( q == 5 ? 1 : 0 );
        const int a = i + di, b = j + dj, c = k + dk;
        *edge = ( a < 0 || b < 0 || c < 0 || a >= L.nx || b >= L.ny || c >= L.nz );
        if( *edge ) return -1;
        if( L.kind == 1 ) return (long long)a + (long long)L.dx * ( b + (long long)L.dy * c );
        const int E = L.E, E3 = E * E * E;
        const int s = (int)( cell / E3 );
        const int la = ( ( i % E ) + di ), lb = ( ( j % E ) + dj ), lc = ( ( k % E ) + dk );
        if( la >= 0 && la < E && lb >= 0 && lb < E && lc >= 0 && lc < E )
            return (long long)s * E3 + la + E * ( lb + E * lc );
        const int ox = la < 0 ? -1 : ( la >= E ? 1 : 0 );
        const int oy = lb < 0 ? -1 : ( lb >= E ? 1 : 0 );
        const int oz = lc < 0 ? -1 : ( lc >= E ? 1 : 0 );
        const int ns = nbr[(size_t)s * 27 + bora_dir( ox, oy, oz )];
        if( ns < 0 ) return -1;
        const int wa = ( la + E ) % E, wb = ( lb + E ) % E, wc = ( lc + E ) % E;
        return (long long)ns * E3 + wa + E * ( wb + E * wc );
    }
};

// ---- set-up: cell types and stencil codes of coarse levels ---------------------------

// Types of level `C` from level `F` (one finer). C tiled with E_C = E_F / 2 (children in
// the same tile), or C dense: children are the finer level's cells (dense) or tiles
// (F tiled with E = 1, through slot_of).
__global__ void k_mg_types( BoraLevelDev F, BoraLevelDev C, const int32_t* __restrict__ slot_of,
                            const int32_t* __restrict__ tile_of, int tx, int ty, int tz )
{
    for( long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < (long long)C.ncells;
         cell += (long long)gridDim.x * blockDim.x )
    {
        int i, j, k;
        if( C.kind == 1 )
        {
            i = (int)( cell % C.dx ); j = (int)( ( cell / C.dx ) % C.dy ); k = (int)( cell / ( (long long)C.dx * C.dy ) );
        }
        else
        {
            const int E = C.E, E3 = E * E * E;
            const int s = (int)( cell / E3 ), loc = (int)( cell % E3 );
            const int vt = tile_of[s];
            i = ( vt % tx ) * E + loc % E;
            j = ( ( vt / tx ) % ty ) * E + ( loc / E ) % E;
            k = ( vt / ( tx * ty ) ) * E + loc / ( E * E );
        }
        if( i >= C.nx || j >= C.ny || k >= C.nz ) { C.type[cell] = BORA_MASKED; continue; }
        bool anyF = false, anyA = false;
        for( int o = 0; o < 8; ++o )
        {
            const int a = 2 * i + ( o & 1 ), b = 2 * j + ( ( o >> 1 ) & 1 ), c = 2 * k + ( o >> 2 );
            if( a >= F.nx || b >= F.ny || c >= F.nz ) continue;  // beyond the finer grid: wall-like
            uint8_t t;
            if( C.kind == 0 )
            {
                const int E = F.E;
                const int s = (int)( cell / ( C.E * C.E * C.E ) );
                t = F.type[(long long)s * E * E * E + ( a % E ) + E * ( ( b % E ) + E * ( c % E ) )];
            }
            else if( F.kind == 1 )
            {
                t = F.type[(long long)a + (long long)F.dx * ( b + (long long)F.dy * c )];
            }
            else  // F tiled with one cell per tile: children are tiles
            {
                if( a >= tx || b >= ty || c >= tz ) continue;
                const int s = slot_of[( (size_t)c * ty + b ) * tx + a];
                t = s < 0 ? (uint8_t)BORA_AIR : F.type[s];
            }
            if( t == BORA_FLUID ) anyF = true;
            else if( t == BORA_AIR ) anyA = true;
        }
        C.type[cell] = anyA ? BORA_AIR : ( anyF ? BORA_FLUID : BORA_SOLID );
    }
}

// Stencil codes of level L from its types (same bit layout as the fine code).
__global__ void k_mg_codes( LevelNav nav, float voxel_wall )
{
    const BoraLevelDev& L = nav.L;
    for( long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < (long long)L.ncells;
         cell += (long long)gridDim.x * blockDim.x )
    {
        if( L.type[cell] != BORA_FLUID ) { L.code[cell] = 0; continue; }
        int i, j, k;
        nav.coords( cell, i, j, k );
        // FluidProjection.cu:208 evaluated at the cell's lowest fine row
        const int wall = (float)( j << L.level ) + 0.5f <= voxel_wall + 1.f ? BORA_WALL : BORA_AIR;
        int diag = 6;
        uint32_t mask = 0;
        for( int q = 0; q < 6; ++q )
        {
            bool edge;
            const long long n = nav.nbr_index( cell, i, j, k, q, &edge );
            int t = edge ? wall : ( n < 0 ? BORA_AIR : (int)L.type[n] );
            if( t == BORA_MASKED ) t = BORA_SOLID;
            if( t == BORA_AIR ) diag += 1;
            else if( t == BORA_SOLID || t == BORA_WALL ) diag -= 1;
            else if( t == BORA_FLUID ) mask |= 1u << q;
        }
        L.code[cell] = (uint16_t)( BORA_CODE_FLUID | ( (uint32_t)diag << 8 ) | mask );
    }
}

// ---- V-cycle -----------------------------------------------------------------------
//
// Navigation is specialised per level kind: tiled levels use the tile edge E as a
// compile-time constant (bit arithmetic, neighbours across tiles through the tile
// neighbour table), dense levels use their small extents. Kernels only visit the
// neighbours that the stencil code marks as fluid, which always exist.

__device__ inline float scale_of( const double* ring, int slot )
{
    const double rr = ring[slot];
    return rr > 0.0 ? (float)( 1.0 / sqrt( rr ) ) : 1.f;
}

template <int E>
struct TiledNav
{
    static constexpr int LE = E == 8 ? 3 : ( E == 4 ? 2 : ( E == 2 ? 1 : 0 ) );
    static constexpr int E3 = E * E * E;
    const int32_t* nbr;
    // dense parent level (E == 1 only)
    const int32_t* tile_of;
    int tx, ty, cdx, cdy;

    __device__ inline long long nb( long long cell, int q ) const
    {
        const long long s = cell >> ( 3 * LE );
        const int l = (int)( cell & ( E3 - 1 ) );
        const int li = l & ( E - 1 ), lj = ( l >> LE ) & ( E - 1 ), lk = l >> ( 2 * LE );
        int dir, ll;
        switch( q )
        {
            case 0: if( li > 0 ) return cell - 1; dir = 12; ll = l + ( E - 1 ); break;
            case 1: if( li < E - 1 ) return cell + 1; dir = 14; ll = l - ( E - 1 ); break;
            case 2: if( lj > 0 ) return cell - E; dir = 10; ll = l + E * ( E - 1 ); break;
            case 3: if( lj < E - 1 ) return cell + E; dir = 16; ll = l - E * ( E - 1 ); break;
            case 4: if( lk > 0 ) return cell - E * E; dir = 4; ll = l + E * E * ( E - 1 ); break;
            default: if( lk < E - 1 ) return cell + E * E; dir = 22; ll = l - E * E * ( E - 1 ); break;
        }
        const int ns = nbr[s * 27 + dir];
        return ns < 0 ? -1 : (long long)ns * E3 + ll;
    }
    // parent on the next coarser level: same tile with edge E/2, or (E == 1) a dense cell
    __device__ inline long long parent( long long cell ) const
    {
        const long long s = cell >> ( 3 * LE );
        const int l = (int)( cell & ( E3 - 1 ) );
        if( E > 1 )
        {
            constexpr int H = E > 1 ? E / 2 : 1;
            const int li = l & ( E - 1 ), lj = ( l >> LE ) & ( E - 1 ), lk = l >> ( 2 * LE );
            return s * ( H * H * H ) + ( li >> 1 ) + H * ( ( lj >> 1 ) + H * ( lk >> 1 ) );
        }
        const int vt = tile_of[s];
        const int ti = vt % tx, tj = ( vt / tx ) % ty, tk = vt / ( tx * ty );
        return (long long)( ti >> 1 ) + (long long)cdx * ( ( tj >> 1 ) + (long long)cdy * ( tk >> 1 ) );
    }
};

struct DenseNav
{
    int dx, dy, dz;   // storage extent = cells inside the domain
    int cdx, cdy;     // coarser dense level
    __device__ inline long long nb( long long cell, int q ) const
    {
        const int c = (int)cell;  // dense levels hold far fewer than 2^31 cells
        const int i = c % dx, j = ( c / dx ) % dy, k = c / ( dx * dy );
        switch( q )
        {
            case 0: return i > 0 ? cell - 1 : -1;
            case 1: return i < dx - 1 ? cell + 1 : -1;
            case 2: return j > 0 ? cell - dx : -1;
            case 3: return j < dy - 1 ? cell + dx : -1;
            case 4: return k > 0 ? cell - (long long)dx * dy : -1;
            default: return k < dz - 1 ? cell + (long long)dx * dy : -1;
        }
    }
    __device__ inline long long parent( long long cell ) const
    {
        const int c = (int)cell;
        const int i = c % dx, j = ( c / dx ) % dy, k = c / ( dx * dy );
        return (long long)( ( i >> 1 ) + cdx * ( ( j >> 1 ) + cdy * ( k >> 1 ) ) );
    }
};

// Level residual r' of a cell: level 0 reads the PCG residual (FP32) times the scale,
// coarser levels read their FP16 residual.
struct RIn
{
    const float* r0;
    float s;
    const __half* rh;
    __device__ inline float operator()( long long c ) const { return r0 ? r0[c] * s : __half2float( rh[c] ); }
};

__device__ inline float ldh( const __half* z, long long c ) { return __half2float( z[c] ); }

// The per-level operations below are written as device functions over a strided cell
// range, so that the same code runs as one grid-wide kernel per operation (large levels)
// or, for the small tail of the hierarchy, inside one CTA that walks several levels with
// CTA barriers in between (k_mg_tail).

// z = two damped-Jacobi sweeps from zero: z1 = w r'/d, z2 = z1 + w (r' - S z1)/d, with
// each neighbour's z1 recomputed from its own r' and diagonal.
template <class Nav>
__device__ inline void smooth0_cells( const Nav& nav, const BoraLevelDev& L, const RIn& R, uint32_t* err, long long i0,
                                      long long stride )
{
    for( long long cell = i0; cell < (long long)L.ncells; cell += stride )
    {
        const uint16_t cc = L.code[cell];
        float z2 = 0.f;
        const int dg = code_diag( cc );
        if( ( cc & BORA_CODE_FLUID ) && dg > 0 )
        {
            const float rc = R( cell );
            const float z1 = kOmegaA * rc / (float)dg;
            float sum = 0.f;
#pragma unroll
            for( int q = 0; q < 6; ++q )
            {
                if( !( cc & ( 1u << q ) ) ) continue;
                const long long n = nav.nb( cell, q );
                if( n < 0 ) { atomicOr( err, 4u ); continue; }
                const int dn = code_diag( L.code[n] );
                if( dn > 0 ) sum += kOmegaA * R( n ) / (float)dn;
            }
            z2 = z1 + kOmegaB * ( rc - ( (float)dg * z1 - sum ) ) / (float)dg;
        }
        L.z0[cell] = __float2half_rn( z2 );
    }
}

// Restriction, one thread per (coarse cell, child): each thread forms its child's
// residual r' - S z (z = the pre-smoothed z0), the 8 lanes of a coarse cell add up by
// shuffles, and r'_C = 4 * mean = 0.5 * sum. Child enumeration:
//   mode 0: C tiled (edge EC), F tiled (edge 2 EC) in the same tile;
//   mode 1: C dense, F tiled with one cell per tile (children are tiles, via slot_of);
//   mode 2: C dense, F dense.
// i0 and stride are multiples of 8 apart within a warp (every lane of a warp runs the
// same number of iterations).
template <class FNav, int MODE, int EC>
__device__ inline void restrict_cells( const FNav& fnav, const BoraLevelDev& F, const BoraLevelDev& C, const RIn& R,
                                       const int32_t* __restrict__ slot_of, int tx, int ty, int tz, uint32_t* err,
                                       long long i0, long long stride )
{
    const long long total = (long long)C.ncells * 8;
    const long long tround = ( total + 31 ) & ~31LL;
    for( long long t = i0; t < tround; t += stride )
    {
        const long long pc = t >> 3;
        const int o = (int)( t & 7 );
        float res = 0.f;
        if( t < total )  // the value of a non-fluid coarse cell is never read
        {
            long long fc = -1;
            if( MODE == 0 )
            {
                constexpr int LC = EC == 4 ? 2 : ( EC == 2 ? 1 : 0 );
                constexpr int EF = 2 * EC;
                const long long s = pc >> ( 3 * LC );
                const int l = (int)( pc & ( EC * EC * EC - 1 ) );
                const int ci = l & ( EC - 1 ), cj = ( l >> LC ) & ( EC - 1 ), ck = l >> ( 2 * LC );
                fc = s * ( EF * EF * EF ) + ( 2 * ci + ( o & 1 ) ) + EF * ( ( 2 * cj + ( ( o >> 1 ) & 1 ) ) +
                                                                           EF * ( 2 * ck + ( o >> 2 ) ) );
            }
            else
            {
                const int I = (int)( pc % C.dx ), J = (int)( ( pc / C.dx ) % C.dy ), K = (int)( pc / ( (long long)C.dx * C.dy ) );
                const int a = 2 * I + ( o & 1 ), b = 2 * J + ( ( o >> 1 ) & 1 ), c = 2 * K + ( o >> 2 );
                if( MODE == 1 )
                {
                    if( a < tx && b < ty && c < tz ) fc = slot_of[( (size_t)c * ty + b ) * tx + a];
                }
                else if( a < F.dx && b < F.dy && c < F.dz )
                {
                    fc = (long long)a + (long long)F.dx * ( b + (long long)F.dy * c );
                }
            }
            if( fc >= 0 )  // children beyond the domain are masked cells: their code is 0
            {
                const uint16_t cf = F.code[fc];
                if( cf & BORA_CODE_FLUID )
                {
                    float sum = 0.f;
#pragma unroll
                    for( int q = 0; q < 6; ++q )
                    {
                        if( !( cf & ( 1u << q ) ) ) continue;
                        const long long n = fnav.nb( fc, q );
                        if( n < 0 ) { atomicOr( err, 8u ); continue; }
                        sum += ldh( F.z0, n );
                    }
                    res = R( fc ) - ( (float)code_diag( cf ) * ldh( F.z0, fc ) - sum );
                }
            }
        }
        res += __shfl_xor_sync( 0xffffffffu, res, 1 );
        res += __shfl_xor_sync( 0xffffffffu, res, 2 );
        res += __shfl_xor_sync( 0xffffffffu, res, 4 );
        if( t < total && o == 0 ) C.r[pc] = __float2half_rn( 0.5f * res );
    }
}

// Coarsest level (<= 512 cells): Jacobi sweeps from zero in shared memory; threads 0..511
// of the CTA own one cell each, every thread of the CTA takes part in the barriers.
struct CoarsestSmem
{
    float zs[2][512], rs[512];
    int16_t nbs[512][6];
};

template <class Nav>
__device__ inline void coarsest_cells( const Nav& nav, const BoraLevelDev& L, int sweeps, uint32_t* err, CoarsestSmem& sm )
{
    const int c = threadIdx.x;
    const bool mine = c < 512;
    const bool valid = c < (int)L.ncells;
    uint16_t cc = 0;
    if( valid )
    {
        cc = L.code[c];
        sm.rs[c] = __half2float( L.r[c] );
        for( int q = 0; q < 6; ++q )
        {
            long long n = -1;
            if( cc & ( 1u << q ) )
            {
                n = nav.nb( c, q );
                if( n < 0 || n >= (long long)L.ncells ) { atomicOr( err, 16u ); n = -1; }
            }
            sm.nbs[c][q] = (int16_t)n;
        }
    }
    if( mine ) { sm.zs[0][c] = 0.f; sm.zs[1][c] = 0.f; }
    __syncthreads();
    int cur = 0;
    const int dg = code_diag( cc );
    const bool act = valid && ( cc & BORA_CODE_FLUID ) && dg > 0;
    for( int it = 0; it < sweeps; ++it )
    {
        float zn = 0.f;
        if( act )
        {
            float sum = 0.f;
            for( int q = 0; q < 6; ++q )
                if( sm.nbs[c][q] >= 0 ) sum += sm.zs[cur][sm.nbs[c][q]];
            const float z = sm.zs[cur][c];
            zn = z + kOmega * ( sm.rs[c] - ( (float)dg * z - sum ) ) / (float)dg;
        }
        if( mine ) sm.zs[cur ^ 1][c] = zn;
        __syncthreads();
        cur ^= 1;
    }
    if( valid ) L.z0[c] = __float2half_rn( sm.zs[cur][c] );
}

// z_a = z0 + P e (injection of the coarse correction C.z0), then one Jacobi sweep;
// neighbours' z_a are formed the same way. Writes z1.
template <class Nav>
__device__ inline void prolong_smooth_cells( const Nav& nav, const BoraLevelDev& F, const __half* __restrict__ ec,
                                             const RIn& R, uint32_t* err, long long i0, long long stride )
{
    for( long long cell = i0; cell < (long long)F.ncells; cell += stride )
    {
        const uint16_t cc = F.code[cell];
        float zb = 0.f;
        const int dg = code_diag( cc );
        if( ( cc & BORA_CODE_FLUID ) && dg > 0 )
        {
            const float za = ldh( F.z0, cell ) + ldh( ec, nav.parent( cell ) );
            float sum = 0.f;
#pragma unroll
            for( int q = 0; q < 6; ++q )
            {
                if( !( cc & ( 1u << q ) ) ) continue;
                const long long n = nav.nb( cell, q );
                if( n < 0 ) { atomicOr( err, 32u ); continue; }
                sum += ldh( F.z0, n ) + ldh( ec, nav.parent( n ) );
            }
            zb = za + kOmegaB * ( R( cell ) - ( (float)dg * za - sum ) ) / (float)dg;
        }
        F.z1[cell] = __float2half_rn( zb );
    }
}

// Final Jacobi sweep of a level: z = z1 + w (r' - S z1)/d, written to z0. On level 0 the
// result is unscaled to FP32 into zout and r.z is accumulated (double-float).
template <class Nav>
__device__ inline DF smooth_last_cells( const Nav& nav, const BoraLevelDev& L, const RIn& R, float* __restrict__ zout,
                                        uint32_t* err, long long i0, long long stride )
{
    DF rz{ 0.f, 0.f };
    for( long long cell = i0; cell < (long long)L.ncells; cell += stride )
    {
        const uint16_t cc = L.code[cell];
        float zc = 0.f;
        const int dg = code_diag( cc );
        if( ( cc & BORA_CODE_FLUID ) && dg > 0 )
        {
            const float zb = ldh( L.z1, cell );
            float sum = 0.f;
#pragma unroll
            for( int q = 0; q < 6; ++q )
            {
                if( !( cc & ( 1u << q ) ) ) continue;
                const long long n = nav.nb( cell, q );
                if( n < 0 ) { atomicOr( err, 64u ); continue; }
                sum += ldh( L.z1, n );
            }
            zc = zb + kOmegaA * ( R( cell ) - ( (float)dg * zb - sum ) ) / (float)dg;
        }
        if( zout )
        {
            const float zf = zc / R.s;  // undo the FP16 scaling of the residual
            zout[cell] = zf;
            if( cc & BORA_CODE_FLUID ) rz = df_add( rz, df_prod( R.r0[cell], zf ) );
        }
        else
        {
            L.z0[cell] = __float2half_rn( zc );
        }
    }
    return rz;
}

// Grid-wide kernels, one per operation.
__device__ inline long long gtid() { return blockIdx.x * (long long)blockDim.x + threadIdx.x; }
__device__ inline long long gstride() { return (long long)gridDim.x * blockDim.x; }

template <class Nav>
__global__ void __launch_bounds__( 256 ) k_mg_smooth0( Nav nav, BoraLevelDev L, const float* __restrict__ r0,
                                                       int slot_rr, const double* __restrict__ ring, uint32_t* err )
{
    __shared__ float s_scale;
    if( threadIdx.x == 0 ) s_scale = r0 ? scale_of( ring, slot_rr ) : 1.f;
    __syncthreads();
    smooth0_cells( nav, L, RIn{ r0, s_scale, L.r }, err, gtid(), gstride() );
}

template <class FNav, int MODE, int EC>
__global__ void __launch_bounds__( 256 ) k_mg_restrict( FNav fnav, BoraLevelDev F, BoraLevelDev C,
                                                        const float* __restrict__ r0, int slot_rr,
                                                        const double* __restrict__ ring,
                                                        const int32_t* __restrict__ slot_of, int tx, int ty, int tz,
                                                        uint32_t* err )
{
    __shared__ float s_scale;
    if( threadIdx.x == 0 ) s_scale = r0 ? scale_of( ring, slot_rr ) : 1.f;
    __syncthreads();
    restrict_cells<FNav, MODE, EC>( fnav, F, C, RIn{ r0, s_scale, F.r }, slot_of, tx, ty, tz, err, gtid(), gstride() );
}

template <class Nav>
__global__ void __launch_bounds__( 512 ) k_mg_coarsest( Nav nav, BoraLevelDev L, int sweeps, uint32_t* err )
{
    __shared__ CoarsestSmem sm;
    coarsest_cells( nav, L, sweeps, err, sm );
}

template <class Nav>
__global__ void __launch_bounds__( 256 ) k_mg_prolong_smooth( Nav nav, BoraLevelDev F, const __half* __restrict__ ec,
                                                              const float* __restrict__ r0, int slot_rr,
                                                              const double* __restrict__ ring, uint32_t* err )
{
    __shared__ float s_scale;
    if( threadIdx.x == 0 ) s_scale = r0 ? scale_of( ring, slot_rr ) : 1.f;
    __syncthreads();
    prolong_smooth_cells( nav, F, ec, RIn{ r0, s_scale, F.r }, err, gtid(), gstride() );
}

template <class Nav>
__global__ void __launch_bounds__( 256 ) k_mg_smooth_last( Nav nav, BoraLevelDev L, const float* __restrict__ r0,
                                                           int slot_rr, BoraReduceDev red, float* __restrict__ zout,
                                                           int slot_rz )
{
    __shared__ float s_scale;
    if( threadIdx.x == 0 ) s_scale = r0 ? scale_of( red.ring, slot_rr ) : 1.f;
    __syncthreads();
    const DF rz = smooth_last_cells( nav, L, RIn{ r0, s_scale, L.r }, zout, red.err, gtid(), gstride() );
    if( zout ) reduce2_publish_warp( df_warp_sum( rz ), 0.0, 0, red, slot_rz, -1 );
}

// The small tail of the hierarchy in one thread-block cluster: levels that are dense or
// tiled with one cell per tile (only the first), down to the coarsest and back up, with a
// cluster barrier between the operations (the cluster's CTAs are co-scheduled, and the
// barrier orders their global-memory writes at cluster scope). The coarsest level runs
// in the cluster's first CTA. (Walking the levels below the first in one CTA's shared
// memory was slower: a 4096-cell level then runs on one SM.)
constexpr int kTailLevels = 8;
constexpr int kTailThreads = 1024;
constexpr int kTailCtasMax = 16;  // non-portable cluster size, where the device supports it
constexpr size_t kTailMaxCells = 32768;

__device__ inline void cluster_barrier()
{
    asm volatile( "barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory" );
}

struct TailDesc
{
    BoraLevelDev L[kTailLevels];
    int n;            // tail levels; the last is the coarsest of the hierarchy
    int first_tiled;  // L[0] is tiled with one cell per tile
    const int32_t* nbr;
    const int32_t* tile_of;
    const int32_t* slot_of;
    int tx, ty, tz;
    int sweeps;       // coarsest sweeps
};

__global__ void __launch_bounds__( kTailThreads ) k_mg_tail( const __grid_constant__ TailDesc d, uint32_t* err )
{
    __shared__ CoarsestSmem sm;
    bora_pdl_trigger();
    bora_pdl_wait();
    const long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    auto with_level = [&]( int t, auto&& f ) {
        const int cdx = t + 1 < d.n ? d.L[t + 1].dx : 0, cdy = t + 1 < d.n ? d.L[t + 1].dy : 0;
        if( t == 0 && d.first_tiled ) f( TiledNav<1>{ d.nbr, d.tile_of, d.tx, d.ty, cdx, cdy } );
        else f( DenseNav{ d.L[t].dx, d.L[t].dy, d.L[t].dz, cdx, cdy } );
    };
    for( int t = 0; t + 1 < d.n; ++t )
    {
        const RIn R{ nullptr, 1.f, d.L[t].r };
        with_level( t, [&]( auto nav ) { smooth0_cells( nav, d.L[t], R, err, i0, st ); } );
        cluster_barrier();
        with_level( t, [&]( auto nav ) {
            if( t == 0 && d.first_tiled )
                restrict_cells<decltype( nav ), 1, 1>( nav, d.L[t], d.L[t + 1], R, d.slot_of, d.tx, d.ty, d.tz, err, i0, st );
            else
                restrict_cells<decltype( nav ), 2, 1>( nav, d.L[t], d.L[t + 1], R, d.slot_of, d.tx, d.ty, d.tz, err, i0, st );
        } );
        cluster_barrier();
    }
    if( blockIdx.x == 0 ) with_level( d.n - 1, [&]( auto nav ) { coarsest_cells( nav, d.L[d.n - 1], d.sweeps, err, sm ); } );
    cluster_barrier();
    for( int t = d.n - 2; t >= 0; --t )
    {
        const RIn R{ nullptr, 1.f, d.L[t].r };
        with_level( t, [&]( auto nav ) { prolong_smooth_cells( nav, d.L[t], d.L[t + 1].z0, R, err, i0, st ); } );
        cluster_barrier();
        with_level( t, [&]( auto nav ) { (void)smooth_last_cells( nav, d.L[t], R, nullptr, err, i0, st ); } );
        cluster_barrier();
    }
}

// ---- tiled levels with E >= 2 -----------------------------------------------------------
// Levels 0, 1 and 2 (E = 8, 4, 2) run as stencil passes (mg_passes.cu).

// PCG update without a preconditioner sweep: r -= alpha q; r.r (e += alpha d is applied by
// the next direction kernel or the refinement step).
__device__ __forceinline__ void pcg_update_noprec_body( size_t ncells, const BoraSolverDev& sv, const BoraReduceDev& red,
                                                        int slot_rz, int slot_dq, int slot_rr_out, unsigned bid, unsigned G )
{
    __shared__ float s_alpha;
    bora_pdl_trigger();
    bora_pdl_wait();
    if( threadIdx.x == 0 ) s_alpha = slot_rz < 0 ? 0.f : (float)( red.ring[slot_rz] / red.ring[slot_dq] );
    __syncthreads();
    const float alpha = s_alpha;
    DF rr{ 0.f, 0.f };
    const size_t n4 = ncells / 4;
    float4* __restrict__ r4 = reinterpret_cast<float4*>( sv.r );
    const float4* __restrict__ q4 = reinterpret_cast<const float4*>( sv.q );
    for( size_t v = bid * (size_t)blockDim.x + threadIdx.x; v < n4; v += (size_t)G * blockDim.x )
    {
        float4 r = r4[v];
        const float4 q = q4[v];
        r.x = fmaf( -alpha, q.x, r.x ); r.y = fmaf( -alpha, q.y, r.y ); r.z = fmaf( -alpha, q.z, r.z ); r.w = fmaf( -alpha, q.w, r.w );
        r4[v] = r;
        rr = df_add_f( rr, dot4( r, r ) );
    }
    reduce2_publish_warp( df_warp_sum( rr ), 0.0, 0, red, slot_rr_out, -1, bid, G );
}

__global__ void __launch_bounds__( 256 ) k_pcg_update_noprec( size_t ncells, BoraSolverDev sv, BoraReduceDev red,
                                                              int slot_rz, int slot_dq, int slot_rr_out )
{
    pcg_update_noprec_body( ncells, sv, red, slot_rz, slot_dq, slot_rr_out, blockIdx.x, gridDim.x );
}

__global__ void __launch_bounds__( 256 ) k_pcg_update_noprec_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    const BoraMemberSlots& q = L.sl[k];
    pcg_update_noprec_body( (size_t)m.ntiles * 512, m.sv, m.red, q.rz_in, q.dq_in, q.rr_out, bid,
                            (unsigned)m.grid[kGridUpd] );
}

int sm_count()
{
    static BoraPerDevice sms;
    return sms.get( [] {
        int dev = 0, n = 0;
        cudaGetDevice( &dev );
        cudaDeviceGetAttribute( &n, cudaDevAttrMultiProcessorCount, dev );
        return n > 0 ? n : 152;
    } );
}

int blocks_for( size_t n )
{
    return (int)std::max<size_t>( 1, std::min<size_t>( ( n + 255 ) / 256, (size_t)sm_count() * 8 ) );
}

LevelNav nav_of( const BoraGridDev& g, const BoraLevelDev& L, BoraTilesDev t )
{
    return LevelNav{ L, t.nbr, t.tile_of, g.tx, g.ty };
}

}  // namespace

void bora_mg_setup( const BoraGridDev& g, BoraLevelDev* levels, int nlevels, BoraTilesDev t, void* mid_image,
                    uint32_t* err, cudaStream_t st )
{
    (void)err;
    for( int l = 1; l < nlevels; ++l )
    {
        const BoraLevelDev& F = levels[l - 1];
        const BoraLevelDev& C = levels[l];
        k_mg_types<<<blocks_for( C.ncells ), 256, 0, st>>>( F, C, t.slot_of, t.tile_of, g.tx, g.ty, g.tz );
        k_mg_codes<<<blocks_for( C.ncells ), 256, 0, st>>>( nav_of( g, C, t ), g.voxel_wall );
    }
    const int ntiles = levels[0].kind == 0 ? (int)( levels[0].ncells / 512 ) : 0;
    bora_mg_mid_setup( g, levels, nlevels, t, ntiles, mid_image, st );
}

namespace {

TiledNav<8> tnav8( BoraTilesDev t ) { return TiledNav<8>{ t.nbr, t.tile_of, 0, 0, 0, 0 }; }

// Launch a level-templated kernel with the navigation of level l.
template <class F>
void with_nav( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, int l, BoraTilesDev t, F&& f )
{
    const BoraLevelDev& L = levels[l];
    const int cdx = l + 1 < nlevels ? levels[l + 1].dx : 0;
    const int cdy = l + 1 < nlevels ? levels[l + 1].dy : 0;
    if( L.kind == 1 ) { f( DenseNav{ L.dx, L.dy, L.dz, cdx, cdy } ); return; }
    switch( L.E )
    {
        case 8: f( TiledNav<8>{ t.nbr, t.tile_of, g.tx, g.ty, cdx, cdy } ); break;
        case 4: f( TiledNav<4>{ t.nbr, t.tile_of, g.tx, g.ty, cdx, cdy } ); break;
        case 2: f( TiledNav<2>{ t.nbr, t.tile_of, g.tx, g.ty, cdx, cdy } ); break;
        default: f( TiledNav<1>{ t.nbr, t.tile_of, g.tx, g.ty, cdx, cdy } ); break;
    }
}

}  // namespace

namespace {

// First level of the one-CTA tail: the longest suffix of levels that are dense (or, first
// only, tiled with one cell per tile) with at most kTailMaxCells cells; nlevels when the
// coarsest level does not qualify (tiny scenes whose coarsest level is still tiled).
int tail_start( const BoraLevelDev* levels, int nlevels )
{
    auto eligible = []( const BoraLevelDev& L ) { return L.ncells <= kTailMaxCells && ( L.kind == 1 || L.E == 1 ); };
    const int last = nlevels - 1;
    if( !eligible( levels[last] ) ) return nlevels;
    int first = last;
    while( first > 0 && eligible( levels[first - 1] ) && levels[first].kind == 1 && last - first + 2 <= kTailLevels ) --first;
    return first;
}

bool pass_level( const BoraLevelDev& L ) { return L.kind == 0 && L.E >= 2; }

// CTAs of the tail cluster: 16 where the device can co-schedule such a cluster of this
// kernel, else the portable 8.
int tail_cluster_size()
{
    static BoraPerDevice size;
    return size.get( [] {
        int n = 8;
        if( cudaFuncSetAttribute( k_mg_tail, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 ) == cudaSuccess )
        {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3( kTailCtasMax );
            cfg.blockDim = dim3( kTailThreads );
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = kTailCtasMax;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            if( cudaOccupancyMaxActiveClusters( &clusters, k_mg_tail, &cfg ) == cudaSuccess && clusters > 0 ) n = kTailCtasMax;
        }
        cudaGetLastError();  // a refused query leaves no error behind
        return n;
    } );
}

}  // namespace

int bora_mg_vcycle_launches( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t,
                             const void* mid_image )
{
    if( nlevels < 2 ) return 0;
    const int ntiles = levels[0].kind == 0 ? (int)( levels[0].ncells / 512 ) : 0;
    const int first = bora_mg_mid_vcycle( g, levels, nlevels, t, ntiles, mid_image, nullptr, 16, nullptr, false )
                          ? 3
                          : tail_start( levels, nlevels );
    const int stop = std::min( first, nlevels - 1 );
    int n = 1;  // the tail kernel, or the coarsest-level kernel
    for( int l = 0; l < stop; ++l ) n += 4;
    if( !( stop > 0 && pass_level( levels[0] ) ) ) n += 1;  // the residual update on its own
    return n;
}

void bora_mg_vcycle( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, const void* mid_image,
                     float* r, const float* q, float* z, float* scratch, BoraReduceDev red, int slot_rz_in,
                     int slot_dq_in, int slot_rr_out, int slot_scale, int slot_rz, int coarse_sweeps, cudaStream_t st )
{
    if( nlevels < 2 ) return;  // the caller always builds at least two levels
    if( levels[0].ncells == 0 ) return;
    const int last = nlevels - 1;
    const int ntiles = levels[0].kind == 0 ? (int)( levels[0].ncells / 512 ) : 0;
    // level 3 .. coarsest in one cluster out of distributed shared memory (mg_mid.cu) when
    // the hierarchy fits it; otherwise the tail levels run from global memory (k_mg_tail)
    const bool mid = bora_mg_mid_vcycle( g, levels, nlevels, t, ntiles, mid_image, red.err, coarse_sweeps, st, false ) != 0;
    const int first = mid ? 3 : tail_start( levels, nlevels );  // levels [first, last] run in one kernel
    const int stop = std::min( first, last );                     // levels [0, stop) restrict/prolong here
    // the residual update runs in level 0's down passes; when level 0 itself is in the tail
    // kernel, it runs first on its own, and the V-cycle is scaled by its r.r
    int slot_rr = slot_scale;
    if( !( stop > 0 && pass_level( levels[0] ) ) )
    {
        BoraSolverDev sv{};
        sv.r = r;
        sv.q = const_cast<float*>( q );
        bora_launch_pcg_update_noprec( ntiles, sv, red, slot_rz_in, slot_dq_in, slot_rr_out, st );
        slot_rr = slot_rr_out;
    }
    // down: pre-smooth and restrict
    for( int l = 0; l < stop; ++l )
    {
        const BoraLevelDev& F = levels[l];
        const BoraLevelDev& C = levels[l + 1];
        const float* r0 = l == 0 ? r : nullptr;
        if( pass_level( F ) )
        {
            bora_mg_pass_down( levels, l, t, ntiles, r, q, scratch, red, slot_rr, slot_rz_in, slot_dq_in, slot_rr_out, st );
            continue;
        }
        with_nav( g, levels, nlevels, l, t, [&]( auto nav ) {
            k_mg_smooth0<<<blocks_for( F.ncells ), 256, 0, st>>>( nav, F, r0, slot_rr, red.ring, red.err );
            const int nb = blocks_for( C.ncells * 8 );
            using N = decltype( nav );
            if( C.kind == 1 )
            {
                if( F.kind == 1 )
                    k_mg_restrict<N, 2, 1><<<nb, 256, 0, st>>>( nav, F, C, r0, slot_rr, red.ring, t.slot_of, g.tx, g.ty, g.tz, red.err );
                else
                    k_mg_restrict<N, 1, 1><<<nb, 256, 0, st>>>( nav, F, C, r0, slot_rr, red.ring, t.slot_of, g.tx, g.ty, g.tz, red.err );
            }
            else
                k_mg_restrict<N, 0, 1><<<nb, 256, 0, st>>>( nav, F, C, r0, slot_rr, red.ring, t.slot_of, g.tx, g.ty, g.tz, red.err );
        } );
    }
    if( mid )
    {
        bora_mg_mid_vcycle( g, levels, nlevels, t, ntiles, mid_image, red.err, coarse_sweeps, st, true );
    }
    else if( first <= last )
    {
        TailDesc d{};
        d.n = last - first + 1;
        for( int q = 0; q < d.n; ++q ) d.L[q] = levels[first + q];
        d.first_tiled = levels[first].kind == 0;
        d.nbr = t.nbr; d.tile_of = t.tile_of; d.slot_of = t.slot_of;
        d.tx = g.tx; d.ty = g.ty; d.tz = g.tz;
        d.sweeps = coarse_sweeps;
        const int ctas = tail_cluster_size();
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3( ctas );
        cfg.blockDim = dim3( kTailThreads );
        cfg.stream = st;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = ctas;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 2;
        cudaLaunchKernelEx( &cfg, k_mg_tail, d, red.err );
    }
    else
    {
        with_nav( g, levels, nlevels, last, t, [&]( auto nav ) {
            k_mg_coarsest<<<1, 512, 0, st>>>( nav, levels[last], coarse_sweeps, red.err );
        } );
    }
    // up: prolong + two sweeps
    for( int l = stop - 1; l >= 0; --l )
    {
        const BoraLevelDev& F = levels[l];
        const float* r0 = l == 0 ? r : nullptr;
        if( pass_level( F ) )
        {
            // a coarser level that ran its passes left its correction in z1, the others in z0
            const bool cf = l + 1 < stop && pass_level( levels[l + 1] );
            const __half* ec = cf ? levels[l + 1].z1 : levels[l + 1].z0;
            bora_mg_pass_up( levels, l, ec, t, ntiles, r, scratch, red, slot_rr, z, slot_rz, st );
            continue;
        }
        with_nav( g, levels, nlevels, l, t, [&]( auto nav ) {
            k_mg_prolong_smooth<<<blocks_for( F.ncells ), 256, 0, st>>>( nav, F, levels[l + 1].z0, r0, slot_rr, red.ring,
                                                                         red.err );
            k_mg_smooth_last<<<blocks_for( F.ncells ), 256, 0, st>>>( nav, F, r0, slot_rr, red, l == 0 ? z : nullptr,
                                                                      slot_rz );
        } );
    }
}

void bora_member_grids( int ntiles, int* grid, const int* v )
{
    bora_projection_grids( ntiles, grid );
    grid[kGridUpd] = blocks_for( (size_t)std::max( ntiles, 0 ) * 512 / 4 );
    grid[kGridPass0] = bora_mg_pass_grid( 8, ntiles, v[0] );
    grid[kGridPass0R] = bora_mg_pass_grid( 8, ntiles, -1 );
    grid[kGridPass1] = bora_mg_pass_grid( 4, ntiles, v[1] );
    grid[kGridPass2] = bora_mg_pass_grid( 2, ntiles, v[2] );
}

void bora_launch_pcg_update_noprec_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks > 0 ) bora_launch_pdl( k_pcg_update_noprec_batch, dim3( blocks ), dim3( 256 ), 0, st, L );
}


void bora_launch_pcg_update_noprec( int ntiles, BoraSolverDev s, BoraReduceDev red, int slot_rz, int slot_dq,
                                    int slot_rr_out, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    bora_launch_pdl( k_pcg_update_noprec, blocks_for( nc / 4 ), 256, 0, st, nc, s, red, slot_rz, slot_dq, slot_rr_out );
}
