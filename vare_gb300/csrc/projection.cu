// Pressure projection over active 8^3 tiles: right-hand side and stencil build, a
// matrix-free PCG with a block-MIC(0) preconditioner, FP64 reductions and FP64
// iterative refinement, and the pressure-gradient velocity update.
//
// Replaces FluidProjection::buildLinearSystem / solve (sparse,
// base/source/FluidProjection.cu:165-381), LinearSystemSolver::cg/pcg
// (base/source/LinearSystemSolver.cpp:12-105) and the BLAS kernels they call
// (base/source/BLAS.cu:12-331). The reference assembles a 7-entry ELL matrix
// (float values + size_t columns, 84 B per row) after a serial host relabel of the
// fluid cells; here the operator is applied from a 16-bit per-cell stencil code
// (neighbour-is-fluid mask + integer diagonal), which encodes the same matrix.
#include "bora_internal.h"

namespace {

// ---------------------------------------------------------------------------------
// Shared-memory halo of a tile: region of (8+2H)^3 cells around tile s.
// Cells outside the grid or in inactive tiles read as "background" (air, zero).
template <int H>
struct Halo
{
    static constexpr int E = BORA_TILE + 2 * H;
    static constexpr int N = E * E * E;
    __device__ static inline int at( int a, int b, int c ) { return a + E * ( b + E * c ); }  // a,b,c in [0,E)
};

// Resolve halo-region cell h (0..N-1) of tile (ti,tj,tk): returns the global field
// index or -1 (outside the grid or inactive tile).
template <int H>
__device__ inline long long halo_index( const BoraGridDev& g, const int32_t* nb, int ti, int tj, int tk, int h )
{
    constexpr int E = Halo<H>::E;
    const int a = h % E, b = ( h / E ) % E, c = h / ( E * E );
    const int i = ti * BORA_TILE - H + a, j = tj * BORA_TILE - H + b, k = tk * BORA_TILE - H + c;
    if( i < 0 || j < 0 || k < 0 || i >= g.nx || j >= g.ny || k >= g.nz ) return -1;
    const int s = nb[bora_dir( ( i >> 3 ) - ti, ( j >> 3 ) - tj, ( k >> 3 ) - tk )];
    if( s < 0 ) return -1;
    return (long long)s * BORA_TILE_CELLS + bora_local( i, j, k );
}

__device__ inline void tile_coords( const BoraGridDev& g, int vt, int& ti, int& tj, int& tk )
{
    ti = vt % g.tx;
    tj = ( vt / g.tx ) % g.ty;
    tk = vt / ( g.tx * g.ty );
}

__device__ inline float absr( float x ) { return x < 0.f ? -x : x; }  // MathUtils.h:129 Abs

// ---------------------------------------------------------------------------------
// Right-hand side and stencil code (FluidProjection.cu:203-266).
__global__ void __launch_bounds__( 512 ) k_rhs( BoraGridDev g, BoraTilesDev t, BoraCellsDev c )
{
    using HL = Halo<1>;
    __shared__ int32_t nb[27];
    __shared__ uint8_t sf[HL::N];
    __shared__ float sx[HL::N], sy[HL::N], sz[HL::N];
    const int s = blockIdx.x;
    if( threadIdx.x < 27 ) nb[threadIdx.x] = t.nbr[(size_t)s * 27 + threadIdx.x];
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    __syncthreads();
    for( int h = threadIdx.x; h < HL::N; h += blockDim.x )
    {
        const long long gi = halo_index<1>( g, nb, ti, tj, tk, h );
        if( gi < 0 ) { sf[h] = BORA_AIR; sx[h] = sy[h] = sz[h] = 0.f; }
        else { sf[h] = c.flag[gi]; sx[h] = c.vx[gi]; sy[h] = c.vy[gi]; sz[h] = c.vz[gi]; }
    }
    __syncthreads();
    const int l = threadIdx.x;
    const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
    const int i = ti * 8 + li, j = tj * 8 + lj, k = tk * 8 + lk;
    const size_t cell = (size_t)s * BORA_TILE_CELLS + l;
    const int h = HL::at( li + 1, lj + 1, lk + 1 );
    if( sf[h] != BORA_FLUID )
    {
        c.b[cell] = 0.f;
        c.code[cell] = 0;
        return;
    }
    const int EI = g.nx - 1, EJ = g.ny - 1, EK = g.nz - 1;
    const int wall = (float)j + 0.5f <= g.voxel_wall + 1.f ? BORA_WALL : BORA_AIR;
    const int hi0 = h - 1, hi1 = h + 1, hj0 = h - HL::E, hj1 = h + HL::E, hk0 = h - HL::E * HL::E, hk1 = h + HL::E * HL::E;
    const int t_i0 = i == 0 ? wall : sf[hi0];
    const int t_i1 = i == EI ? wall : sf[hi1];
    const int t_j0 = j == 0 ? wall : sf[hj0];
    const int t_j1 = j == EJ ? wall : sf[hj1];
    const int t_k0 = k == 0 ? wall : sf[hk0];
    const int t_k1 = k == EK ? wall : sf[hk1];
    const float vx = sx[h], vy = sy[h], vz = sz[h];
    const float i0_j_k = i == 0 ? 2.f * vx - sx[hi1] : sx[hi0];
    const float i1_j_k = i == EI ? 2.f * vx - sx[hi0] : sx[hi1];
    const float i_j0_k = j == 0 ? 2.f * vy - sy[hj1] : sy[hj0];
    const float i_j1_k = j == EJ ? 2.f * vy - sy[hj0] : sy[hj1];
    const float i_j_k0 = k == 0 ? 2.f * vz - sz[hk1] : sz[hk0];
    const float i_j_k1 = k == EK ? 2.f * vz - sz[hk0] : sz[hk1];
    const float v_i0 = t_i0 == BORA_AIR ? 2.f * vx - i1_j_k : t_i0 == BORA_WALL ? absr( vx ) : i0_j_k;
    const float v_i1 = t_i1 == BORA_AIR ? 2.f * vx - i0_j_k : t_i1 == BORA_WALL ? -absr( vx ) : i1_j_k;
    const float v_j0 = t_j0 == BORA_AIR ? 2.f * vy - i_j1_k : t_j0 == BORA_WALL ? absr( vy ) : i_j0_k;
    const float v_j1 = t_j1 == BORA_AIR ? 2.f * vy - i_j0_k : t_j1 == BORA_WALL ? -absr( vy ) : i_j1_k;
    const float v_k0 = t_k0 == BORA_AIR ? 2.f * vz - i_j_k1 : t_k0 == BORA_WALL ? absr( vz ) : i_j_k0;
    const float v_k1 = t_k1 == BORA_AIR ? 2.f * vz - i_j_k0 : t_k1 == BORA_WALL ? -absr( vz ) : i_j_k1;
    const float d = -( ( v_i1 - v_i0 ) * 0.5f + ( v_j1 - v_j0 ) * 0.5f + ( v_k1 - v_k0 ) * 0.5f );
    int diag = 6;
    uint32_t mask = 0;
    const int tt[6] = { t_i0, t_i1, t_j0, t_j1, t_k0, t_k1 };
#pragma unroll
    for( int q = 0; q < 6; ++q )
    {
        if( tt[q] == BORA_AIR ) diag += 1;
        else if( tt[q] == BORA_SOLID || tt[q] == BORA_WALL ) diag -= 1;
        else if( tt[q] == BORA_FLUID ) mask |= 1u << q;
    }
    c.b[cell] = d;
    c.code[cell] = (uint16_t)( BORA_CODE_FLUID | ( (uint32_t)diag << 8 ) | mask );
}

// ---------------------------------------------------------------------------------
// Deterministic FP64 block reduction published through a ring slot: every block writes
// its partial, the last block to arrive sums the partials in block order.
__device__ inline double warp_sum( double v )
{
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) v += __shfl_xor_sync( 0xffffffffu, v, o );
    return v;
}
__device__ inline double warp_max( double v )
{
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) v = fmax( v, __shfl_xor_sync( 0xffffffffu, v, o ) );
    return v;
}

// op1: 0 = sum, 1 = max for the second value. Slots < 0 are skipped.
__device__ void reduce2_publish( double v0, double v1, int op1, BoraReduceDev red, int slot0, int slot1 )
{
    __shared__ double w0[32], w1[32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = ( blockDim.x + 31 ) >> 5;
    v0 = warp_sum( v0 );
    v1 = op1 ? warp_max( v1 ) : warp_sum( v1 );
    if( lane == 0 ) { w0[wid] = v0; w1[wid] = v1; }
    __syncthreads();
    if( threadIdx.x == 0 )
    {
        double a = 0.0, b = 0.0;
        for( int q = 0; q < nw; ++q ) { a += w0[q]; b = op1 ? fmax( b, w1[q] ) : b + w1[q]; }
        red.partials[2 * (size_t)blockIdx.x] = a;
        red.partials[2 * (size_t)blockIdx.x + 1] = b;
        __threadfence();
        const int key = slot0 >= 0 ? slot0 : slot1;
        const unsigned prev = atomicAdd( &red.done[key % BORA_RING], 1u );
        last = ( prev == gridDim.x - 1 );
    }
    __syncthreads();
    if( !last ) return;
    __threadfence();
    double a = 0.0, b = 0.0;
    if( wid == 0 )
    {
        // lane-strided partial sums in fixed order, then a fixed-shape warp tree
        for( unsigned q = lane; q < gridDim.x; q += 32 )
        {
            a += __ldcg( &red.partials[2 * (size_t)q] );
            const double pb = __ldcg( &red.partials[2 * (size_t)q + 1] );
            b = op1 ? fmax( b, pb ) : b + pb;
        }
        a = warp_sum( a );
        b = op1 ? warp_max( b ) : warp_sum( b );
        if( lane == 0 )
        {
            if( slot0 >= 0 ) red.ring[slot0] = a;
            if( slot1 >= 0 ) red.ring[slot1] = b;
            const int key = slot0 >= 0 ? slot0 : slot1;
            red.done[key % BORA_RING] = 0;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------------
// Wavefront tables of an 8^3 tile: cells ordered by plane i+j+k (0..21).
__constant__ uint16_t c_plane_cells[512];
__constant__ uint16_t c_plane_start[23];

struct PlaneTables
{
    uint16_t cells[512];
    uint16_t start[23];
    PlaneTables()
    {
        int n = 0;
        for( int s = 0; s <= 21; ++s )
        {
            start[s] = (uint16_t)n;
            for( int l = 0; l < 512; ++l )
            {
                const int i = l & 7, j = ( l >> 3 ) & 7, k = l >> 6;
                if( i + j + k == s ) cells[n++] = (uint16_t)l;
            }
        }
        start[22] = (uint16_t)n;
    }
};

bool g_tables_ready[64] = { false };

void ensure_tables()
{
    int dev = 0;
    cudaGetDevice( &dev );
    if( dev < 0 || dev >= 64 || g_tables_ready[dev] ) return;
    static const PlaneTables tbl;
    cudaMemcpyToSymbol( c_plane_cells, tbl.cells, sizeof( tbl.cells ) );
    cudaMemcpyToSymbol( c_plane_start, tbl.start, sizeof( tbl.start ) );
    g_tables_ready[dev] = true;
}

__device__ inline int code_diag( uint16_t c ) { return ( c >> 8 ) & 15; }

// Block-MIC(0) pivots (MIC(0) of BLAS.cu:211-262 with tau = 0.97, restricted to the
// couplings inside each 8^3 tile so that tiles factor independently). One warp per tile.
constexpr int kTilesPerCta = 4;

__global__ void __launch_bounds__( 32 * kTilesPerCta ) k_mic_factor( int ntiles, const uint16_t* __restrict__ code,
                                                                     float* __restrict__ minv )
{
    __shared__ float sm[kTilesPerCta][512];
    __shared__ uint16_t sc[kTilesPerCta][512];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = blockIdx.x * kTilesPerCta + w;
    if( s >= ntiles ) return;
    const size_t base = (size_t)s * 512;
    for( int l = lane; l < 512; l += 32 ) { sc[w][l] = code[base + l]; sm[w][l] = 0.f; }
    __syncwarp();
    const float tau = 0.97f;
    for( int p = 0; p <= 21; ++p )
    {
        for( int q = c_plane_start[p] + lane; q < c_plane_start[p + 1]; q += 32 )
        {
            const int l = c_plane_cells[q];
            const uint16_t cc = sc[w][l];
            if( !( cc & BORA_CODE_FLUID ) ) continue;
            const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
            const float diag = (float)code_diag( cc );
            float e = diag, e2 = 0.f;
            if( li > 0 && ( cc & 1u ) )
            {
                const int m = l - 1;
                const uint16_t cm = sc[w][m];
                const float M = sm[w][m];
                const float a = ( lj < 7 && ( cm & 8u ) ) ? 1.f : 0.f;    // m+y inside the tile and fluid
                const float b = ( lk < 7 && ( cm & 32u ) ) ? 1.f : 0.f;   // m+z
                e -= M * M;
                e2 += ( a + b ) * ( M * M );
            }
            if( lj > 0 && ( cc & 4u ) )
            {
                const int m = l - 8;
                const uint16_t cm = sc[w][m];
                const float M = sm[w][m];
                const float a = ( li < 7 && ( cm & 2u ) ) ? 1.f : 0.f;    // m+x
                const float b = ( lk < 7 && ( cm & 32u ) ) ? 1.f : 0.f;   // m+z
                e -= M * M;
                e2 += ( a + b ) * ( M * M );
            }
            if( lk > 0 && ( cc & 16u ) )
            {
                const int m = l - 64;
                const uint16_t cm = sc[w][m];
                const float M = sm[w][m];
                const float a = ( li < 7 && ( cm & 2u ) ) ? 1.f : 0.f;    // m+x
                const float b = ( lj < 7 && ( cm & 8u ) ) ? 1.f : 0.f;    // m+y
                e -= M * M;
                e2 += ( a + b ) * ( M * M );
            }
            e -= tau * e2;
            if( e < diag * 0.25f ) e = diag;
            sm[w][l] = 1.f / sqrtf( e + 1e-30f );
        }
        __syncwarp();
    }
    for( int l = lane; l < 512; l += 32 ) minv[base + l] = sm[w][l];
}

// ---------------------------------------------------------------------------------
// PCG update: e += alpha d; r -= alpha q; z = M^-1 r (block-MIC(0) forward and backward
// sweeps in shared memory); rz = r.z and rr = r.r in FP64. One warp per tile.
__global__ void __launch_bounds__( 32 * kTilesPerCta ) k_pcg_update( int ntiles, const uint16_t* __restrict__ code,
                                                                     BoraSolverDev sv, int dsel, BoraReduceDev red,
                                                                     int slot_rz_in, int slot_dq_in, int slot_rz_out,
                                                                     int slot_rr_out )
{
    __shared__ float sr[kTilesPerCta][512];
    __shared__ float sy[kTilesPerCta][512];
    __shared__ float sm[kTilesPerCta][512];
    __shared__ uint16_t sc[kTilesPerCta][512];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = blockIdx.x * kTilesPerCta + w;
    double prz = 0.0, prr = 0.0;
    const float alpha = slot_rz_in < 0 ? 0.f : (float)( red.ring[slot_rz_in] / red.ring[slot_dq_in] );
    if( s < ntiles )
    {
        const size_t base = (size_t)s * 512;
        const float* dvec = sv.d[dsel];
        for( int l4 = lane; l4 < 128; l4 += 32 )
        {
            const size_t o = base + 4 * (size_t)l4;
            float4 e = *reinterpret_cast<const float4*>( sv.e + o );
            float4 r = *reinterpret_cast<const float4*>( sv.r + o );
            const float4 d = *reinterpret_cast<const float4*>( dvec + o );
            const float4 q = *reinterpret_cast<const float4*>( sv.q + o );
            e.x = fmaf( alpha, d.x, e.x ); e.y = fmaf( alpha, d.y, e.y ); e.z = fmaf( alpha, d.z, e.z ); e.w = fmaf( alpha, d.w, e.w );
            r.x = fmaf( -alpha, q.x, r.x ); r.y = fmaf( -alpha, q.y, r.y ); r.z = fmaf( -alpha, q.z, r.z ); r.w = fmaf( -alpha, q.w, r.w );
            *reinterpret_cast<float4*>( sv.e + o ) = e;
            *reinterpret_cast<float4*>( sv.r + o ) = r;
            sr[w][4 * l4] = r.x; sr[w][4 * l4 + 1] = r.y; sr[w][4 * l4 + 2] = r.z; sr[w][4 * l4 + 3] = r.w;
            const float4 mv = *reinterpret_cast<const float4*>( sv.minv + o );
            sm[w][4 * l4] = mv.x; sm[w][4 * l4 + 1] = mv.y; sm[w][4 * l4 + 2] = mv.z; sm[w][4 * l4 + 3] = mv.w;
            const ushort4 cv = *reinterpret_cast<const ushort4*>( code + o );
            sc[w][4 * l4] = cv.x; sc[w][4 * l4 + 1] = cv.y; sc[w][4 * l4 + 2] = cv.z; sc[w][4 * l4 + 3] = cv.w;
        }
        __syncwarp();
        // forward: y_c = (r_c + sum_{lower m} M_m y_m) M_c   (A_mc = -1)
        for( int p = 0; p <= 21; ++p )
        {
            for( int q = c_plane_start[p] + lane; q < c_plane_start[p + 1]; q += 32 )
            {
                const int l = c_plane_cells[q];
                const uint16_t cc = sc[w][l];
                float y = 0.f;
                if( cc & BORA_CODE_FLUID )
                {
                    float t = sr[w][l];
                    if( ( l & 7 ) > 0 && ( cc & 1u ) ) t = fmaf( sm[w][l - 1], sy[w][l - 1], t );
                    if( ( ( l >> 3 ) & 7 ) > 0 && ( cc & 4u ) ) t = fmaf( sm[w][l - 8], sy[w][l - 8], t );
                    if( ( l >> 6 ) > 0 && ( cc & 16u ) ) t = fmaf( sm[w][l - 64], sy[w][l - 64], t );
                    y = t * sm[w][l];
                }
                sy[w][l] = y;
            }
            __syncwarp();
        }
        // backward: z_c = (y_c + M_c sum_{upper u} z_u) M_c ; z overwrites sy in place
        for( int p = 21; p >= 0; --p )
        {
            for( int q = c_plane_start[p] + lane; q < c_plane_start[p + 1]; q += 32 )
            {
                const int l = c_plane_cells[q];
                const uint16_t cc = sc[w][l];
                if( cc & BORA_CODE_FLUID )
                {
                    float acc = 0.f;
                    if( ( l & 7 ) < 7 && ( cc & 2u ) ) acc += sy[w][l + 1];
                    if( ( ( l >> 3 ) & 7 ) < 7 && ( cc & 8u ) ) acc += sy[w][l + 8];
                    if( ( l >> 6 ) < 7 && ( cc & 32u ) ) acc += sy[w][l + 64];
                    const float M = sm[w][l];
                    sy[w][l] = fmaf( M, acc, sy[w][l] ) * M;
                }
            }
            __syncwarp();
        }
        for( int l4 = lane; l4 < 128; l4 += 32 )
        {
            const size_t o = base + 4 * (size_t)l4;
            const float4 z = make_float4( sy[w][4 * l4], sy[w][4 * l4 + 1], sy[w][4 * l4 + 2], sy[w][4 * l4 + 3] );
            *reinterpret_cast<float4*>( sv.z + o ) = z;
            const float r0 = sr[w][4 * l4], r1 = sr[w][4 * l4 + 1], r2 = sr[w][4 * l4 + 2], r3 = sr[w][4 * l4 + 3];
            prz += (double)r0 * z.x + (double)r1 * z.y + (double)r2 * z.z + (double)r3 * z.w;
            prr += (double)r0 * r0 + (double)r1 * r1 + (double)r2 * r2 + (double)r3 * r3;
        }
    }
    reduce2_publish( prz, prr, 0, red, slot_rz_out, slot_rr_out );
}

// ---------------------------------------------------------------------------------
// PCG direction: d' = z + beta d; q = A d'; dq = d'.q. One CTA (512 threads) per tile;
// d is double-buffered so that neighbour tiles read the previous direction.
__global__ void __launch_bounds__( 512 ) k_pcg_direction( BoraGridDev g, BoraTilesDev t, const uint16_t* __restrict__ code,
                                                          BoraSolverDev sv, int dsel_in, BoraReduceDev red,
                                                          int slot_rz_new, int slot_rz_old, int slot_dq_out )
{
    __shared__ int32_t nb[27];
    __shared__ float sd[512];
    const int s = blockIdx.x;
    if( threadIdx.x < 27 ) nb[threadIdx.x] = t.nbr[(size_t)s * 27 + threadIdx.x];
    const float beta = slot_rz_old < 0 ? 0.f : (float)( red.ring[slot_rz_new] / red.ring[slot_rz_old] );
    const float* dold = sv.d[dsel_in];
    float* dnew = sv.d[dsel_in ^ 1];
    const int l = threadIdx.x;
    const size_t cell = (size_t)s * 512 + l;
    const float dn = fmaf( beta, dold[cell], sv.z[cell] );
    sd[l] = dn;
    dnew[cell] = dn;
    __syncthreads();
    const uint16_t cc = code[cell];
    double pdq = 0.0;
    if( cc & BORA_CODE_FLUID )
    {
        const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
        float acc = 0.f;
        // neighbour value: inside the tile from shared memory, else recomputed from the
        // neighbour tile's z and previous d (identical arithmetic to its own CTA)
        auto nbv = [&]( int q, int inside_off, int dx, int dy, int dz, int lo ) -> float {
            if( inside_off ) return sd[l + lo];
            const int ns = nb[bora_dir( dx, dy, dz )];
            const int ll = bora_local( li + dx, lj + dy, lk + dz );
            const size_t nc = (size_t)ns * 512 + ll;
            return fmaf( beta, dold[nc], sv.z[nc] );
        };
        if( cc & 1u ) acc += nbv( 0, li > 0, -1, 0, 0, -1 );
        if( cc & 2u ) acc += nbv( 1, li < 7, 1, 0, 0, 1 );
        if( cc & 4u ) acc += nbv( 2, lj > 0, 0, -1, 0, -8 );
        if( cc & 8u ) acc += nbv( 3, lj < 7, 0, 1, 0, 8 );
        if( cc & 16u ) acc += nbv( 4, lk > 0, 0, 0, -1, -64 );
        if( cc & 32u ) acc += nbv( 5, lk < 7, 0, 0, 1, 64 );
        const float qv = fmaf( (float)code_diag( cc ), dn, -acc );
        sv.q[cell] = qv;
        pdq = (double)dn * (double)qv;
    }
    else
    {
        sv.q[cell] = 0.f;
    }
    reduce2_publish( pdq, 0.0, 0, red, slot_dq_out, -1 );
}

// ---------------------------------------------------------------------------------
__global__ void k_solve_init( size_t ncells, const float* __restrict__ b, BoraSolverDev sv, BoraReduceDev red,
                              int slot_norm2, int slot_max )
{
    double n2 = 0.0, mx = 0.0;
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)gridDim.x * blockDim.x )
    {
        const float bv = b[i];
        sv.r[i] = bv;
        sv.x[i] = 0.0;
        sv.e[i] = 0.f;
        sv.d[0][i] = 0.f;
        sv.d[1][i] = 0.f;
        sv.q[i] = 0.f;
        n2 += (double)bv * bv;
        mx = fmax( mx, (double)fabsf( bv ) );
    }
    reduce2_publish( n2, mx, 1, red, slot_norm2, slot_max );
}

__global__ void k_refine_accumulate( size_t ncells, const uint16_t* __restrict__ code, BoraSolverDev sv )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)gridDim.x * blockDim.x )
    {
        if( code[i] & BORA_CODE_FLUID ) sv.x[i] += (double)sv.e[i];
        sv.e[i] = 0.f;
        sv.d[0][i] = 0.f;
        sv.d[1][i] = 0.f;
        sv.q[i] = 0.f;
    }
}

// r = b - A x in FP64 (A from the stencil code); r stored in FP32.
__global__ void __launch_bounds__( 512 ) k_refine_residual( BoraGridDev g, BoraTilesDev t, const float* __restrict__ b,
                                                            const uint16_t* __restrict__ code, BoraSolverDev sv,
                                                            BoraReduceDev red, int slot_norm2, int slot_max )
{
    __shared__ int32_t nb[27];
    __shared__ double sxv[512];
    const int s = blockIdx.x;
    if( threadIdx.x < 27 ) nb[threadIdx.x] = t.nbr[(size_t)s * 27 + threadIdx.x];
    const int l = threadIdx.x;
    const size_t cell = (size_t)s * 512 + l;
    sxv[l] = sv.x[cell];
    __syncthreads();
    const uint16_t cc = code[cell];
    double n2 = 0.0, mx = 0.0;
    if( cc & BORA_CODE_FLUID )
    {
        const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
        auto nbv = [&]( int inside_off, int dx, int dy, int dz, int lo ) -> double {
            if( inside_off ) return sxv[l + lo];
            const int ns = nb[bora_dir( dx, dy, dz )];
            return sv.x[(size_t)ns * 512 + bora_local( li + dx, lj + dy, lk + dz )];
        };
        double acc = 0.0;
        if( cc & 1u ) acc += nbv( li > 0, -1, 0, 0, -1 );
        if( cc & 2u ) acc += nbv( li < 7, 1, 0, 0, 1 );
        if( cc & 4u ) acc += nbv( lj > 0, 0, -1, 0, -8 );
        if( cc & 8u ) acc += nbv( lj < 7, 0, 1, 0, 8 );
        if( cc & 16u ) acc += nbv( lk > 0, 0, 0, -1, -64 );
        if( cc & 32u ) acc += nbv( lk < 7, 0, 0, 1, 64 );
        const double rv = (double)b[cell] - ( (double)code_diag( cc ) * sxv[l] - acc );
        sv.r[cell] = (float)rv;
        n2 = rv * rv;
        mx = fabs( rv );
    }
    else
    {
        sv.r[cell] = 0.f;
    }
    reduce2_publish( n2, mx, 1, red, slot_norm2, slot_max );
}

__global__ void k_write_pressure( size_t ncells, const uint16_t* __restrict__ code, const double* __restrict__ x,
                                  float* __restrict__ pres )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)gridDim.x * blockDim.x )
        pres[i] = ( code[i] & BORA_CODE_FLUID ) ? (float)x[i] : 0.f;
}

// ---------------------------------------------------------------------------------
// Velocity update (FluidProjection.cu:293-378): air cells next to fluid take the mean
// of their fluid neighbours' pressure, then fluid cells subtract the central-difference
// pressure gradient with the reference's ghost rules; other cells keep the P2G velocity.
__global__ void __launch_bounds__( 512 ) k_vel_update( BoraGridDev g, BoraTilesDev t, BoraCellsDev c )
{
    using H2 = Halo<2>;
    using H1 = Halo<1>;
    __shared__ int32_t nb[27];
    __shared__ uint8_t sf[H2::N];
    __shared__ float sp[H2::N];
    __shared__ float pa[H1::N];
    __shared__ uint8_t fa[H1::N];
    const int s = blockIdx.x;
    if( threadIdx.x < 27 ) nb[threadIdx.x] = t.nbr[(size_t)s * 27 + threadIdx.x];
    int ti, tj, tk;
    tile_coords( g, t.tile_of[s], ti, tj, tk );
    __syncthreads();
    for( int h = threadIdx.x; h < H2::N; h += blockDim.x )
    {
        const long long gi = halo_index<2>( g, nb, ti, tj, tk, h );
        if( gi < 0 ) { sf[h] = BORA_AIR; sp[h] = 0.f; }
        else
        {
            const uint8_t f = c.flag[gi];
            sf[h] = f;
            sp[h] = f == BORA_FLUID ? c.pres[gi] : 0.f;
        }
    }
    __syncthreads();
    const int EI = g.nx - 1, EJ = g.ny - 1, EK = g.nz - 1;
    for( int h = threadIdx.x; h < H1::N; h += blockDim.x )
    {
        const int a = h % H1::E, b = ( h / H1::E ) % H1::E, cc = h / ( H1::E * H1::E );
        const int i = ti * 8 - 1 + a, j = tj * 8 - 1 + b, k = tk * 8 - 1 + cc;
        const int h2 = H2::at( a + 1, b + 1, cc + 1 );
        const uint8_t f = sf[h2];
        float p = sp[h2];
        if( f == BORA_AIR && i >= 0 && j >= 0 && k >= 0 && i <= EI && j <= EJ && k <= EK )
        {
            float press = 0.f;
            int count = 0;
            if( i > 0 && sf[h2 - 1] == BORA_FLUID ) { press += sp[h2 - 1]; count++; }
            if( i < EI && sf[h2 + 1] == BORA_FLUID ) { press += sp[h2 + 1]; count++; }
            if( j > 0 && sf[h2 - H2::E] == BORA_FLUID ) { press += sp[h2 - H2::E]; count++; }
            if( j < EJ && sf[h2 + H2::E] == BORA_FLUID ) { press += sp[h2 + H2::E]; count++; }
            if( k > 0 && sf[h2 - H2::E * H2::E] == BORA_FLUID ) { press += sp[h2 - H2::E * H2::E]; count++; }
            if( k < EK && sf[h2 + H2::E * H2::E] == BORA_FLUID ) { press += sp[h2 + H2::E * H2::E]; count++; }
            if( count > 0 ) p = press / (float)count;
        }
        pa[h] = p;
        fa[h] = f;
    }
    __syncthreads();
    const int l = threadIdx.x;
    const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
    const int i = ti * 8 + li, j = tj * 8 + lj, k = tk * 8 + lk;
    const size_t cell = (size_t)s * BORA_TILE_CELLS + l;
    const int h = H1::at( li + 1, lj + 1, lk + 1 );
    const uint8_t f = fa[h];
    if( f == BORA_MASKED ) { c.pres[cell] = 0.f; c.cx[cell] = 0.f; c.cy[cell] = 0.f; c.cz[cell] = 0.f; return; }
    const float p = pa[h];
    c.pres[cell] = p;
    float vx = c.vx[cell], vy = c.vy[cell], vz = c.vz[cell];
    if( f == BORA_FLUID )
    {
        const int wall = (float)j + 0.5f <= g.voxel_wall + 1.f ? BORA_SOLID : BORA_AIR;
        const int hi0 = h - 1, hi1 = h + 1, hj0 = h - H1::E, hj1 = h + H1::E, hk0 = h - H1::E * H1::E, hk1 = h + H1::E * H1::E;
        const int t_i0 = i == 0 ? wall : fa[hi0];
        const int t_i1 = i == EI ? wall : fa[hi1];
        const int t_j0 = j == 0 ? wall : fa[hj0];
        const int t_j1 = j == EJ ? wall : fa[hj1];
        const int t_k0 = k == 0 ? wall : fa[hk0];
        const int t_k1 = k == EK ? wall : fa[hk1];
        const float i0_j_k = i == 0 ? 2.f * p - pa[hi1] : pa[hi0];
        const float i1_j_k = i == EI ? 2.f * p - pa[hi0] : pa[hi1];
        const float i_j0_k = j == 0 ? 2.f * p - pa[hj1] : pa[hj0];
        const float i_j1_k = j == EJ ? 2.f * p - pa[hj0] : pa[hj1];
        const float i_j_k0 = k == 0 ? 2.f * p - pa[hk1] : pa[hk0];
        const float i_j_k1 = k == EK ? 2.f * p - pa[hk0] : pa[hk1];
        const float p_i0 = t_i0 == BORA_SOLID ? 2.f * p - i1_j_k : t_i0 == BORA_AIR ? -i0_j_k : i0_j_k;
        const float p_i1 = t_i1 == BORA_SOLID ? 2.f * p - i0_j_k : t_i1 == BORA_AIR ? -i1_j_k : i1_j_k;
        const float p_j0 = t_j0 == BORA_SOLID ? 2.f * p - i_j1_k : t_j0 == BORA_AIR ? -i_j0_k : i_j0_k;
        const float p_j1 = t_j1 == BORA_SOLID ? 2.f * p - i_j0_k : t_j1 == BORA_AIR ? -i_j1_k : i_j1_k;
        const float p_k0 = t_k0 == BORA_SOLID ? 2.f * p - i_j_k1 : t_k0 == BORA_AIR ? -i_j_k0 : i_j_k0;
        const float p_k1 = t_k1 == BORA_SOLID ? 2.f * p - i_j_k0 : t_k1 == BORA_AIR ? -i_j_k1 : i_j_k1;
        vx -= ( p_i1 - p_i0 ) * 0.5f;
        vy -= ( p_j1 - p_j0 ) * 0.5f;
        vz -= ( p_k1 - p_k0 ) * 0.5f;
    }
    c.cx[cell] = vx;
    c.cy[cell] = vy;
    c.cz[cell] = vz;
}

int grid_for( size_t n, int threads )
{
    const size_t b = ( n + threads - 1 ) / threads;
    return (int)( b < 152 * 8 ? ( b > 0 ? b : 1 ) : 152 * 8 );
}

}  // namespace

size_t bora_reduce_max_blocks() { return 152 * 8 > 0 ? (size_t)1 << 22 : 0; }

void bora_launch_rhs( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, cudaStream_t st )
{
    if( ntiles > 0 ) k_rhs<<<ntiles, 512, 0, st>>>( g, t, c );
}

void bora_launch_vel_update( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, cudaStream_t st )
{
    if( ntiles > 0 ) k_vel_update<<<ntiles, 512, 0, st>>>( g, t, c );
}

void bora_launch_mic_factor( const BoraGridDev&, int ntiles, const uint16_t* code, float* minv, cudaStream_t st )
{
    ensure_tables();
    if( ntiles > 0 ) k_mic_factor<<<( ntiles + kTilesPerCta - 1 ) / kTilesPerCta, 32 * kTilesPerCta, 0, st>>>( ntiles, code, minv );
}

void bora_launch_solve_init( int ntiles, const float* b, const uint16_t*, BoraSolverDev s, BoraReduceDev red,
                             int slot_norm2, int slot_max, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    k_solve_init<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, b, s, red, slot_norm2, slot_max );
}

void bora_launch_pcg_update( int ntiles, const uint16_t* code, BoraSolverDev s, int dsel, BoraReduceDev red,
                             int slot_rz_in, int slot_dq_in, int slot_rz_out, int slot_rr_out, cudaStream_t st )
{
    ensure_tables();
    const int nb = ( ntiles + kTilesPerCta - 1 ) / kTilesPerCta;
    k_pcg_update<<<nb > 0 ? nb : 1, 32 * kTilesPerCta, 0, st>>>( ntiles, code, s, dsel, red, slot_rz_in, slot_dq_in,
                                                                   slot_rz_out, slot_rr_out );
}

void bora_launch_pcg_direction( const BoraGridDev& g, int ntiles, BoraTilesDev t, const uint16_t* code, BoraSolverDev s,
                                int dsel_in, BoraReduceDev red, int slot_rz_new, int slot_rz_old, int slot_dq_out,
                                cudaStream_t st )
{
    if( ntiles > 0 )
        k_pcg_direction<<<ntiles, 512, 0, st>>>( g, t, code, s, dsel_in, red, slot_rz_new, slot_rz_old, slot_dq_out );
}

void bora_launch_refine_accumulate( int ntiles, const uint16_t* code, BoraSolverDev s, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    if( nc ) k_refine_accumulate<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, code, s );
}

void bora_launch_refine_residual( const BoraGridDev& g, int ntiles, BoraTilesDev t, const float* b, const uint16_t* code,
                                  BoraSolverDev s, BoraReduceDev red, int slot_norm2, int slot_max, cudaStream_t st )
{
    if( ntiles > 0 ) k_refine_residual<<<ntiles, 512, 0, st>>>( g, t, b, code, s, red, slot_norm2, slot_max );
}

void bora_launch_write_pressure( int ntiles, const uint16_t* code, const double* x, float* pres, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    if( nc ) k_write_pressure<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, code, x, pres );
}
