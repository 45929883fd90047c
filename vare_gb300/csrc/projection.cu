// Pressure projection over active 8^3 tiles: right-hand side and stencil build, a
// matrix-free PCG with a block-MIC(0) preconditioner, FP64-accurate (double-float)
// reductions and double-float iterative refinement, and the pressure-gradient velocity
// update.
//
// Replaces FluidProjection::buildLinearSystem / solve (sparse,
// base/source/FluidProjection.cu:165-381), LinearSystemSolver::cg/pcg
// (base/source/LinearSystemSolver.cpp:12-105) and the BLAS kernels they call
// (base/source/BLAS.cu:12-331). The reference assembles a 7-entry ELL matrix
// (float values + size_t columns, 84 B per row) after a serial host relabel of the
// fluid cells; here the operator is applied from a 16-bit per-cell stencil code
// (neighbour-is-fluid mask + integer diagonal), which encodes the same matrix.
#include <algorithm>

#include "bora_internal.h"
#include "reduce.cuh"

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
__global__ void __launch_bounds__( 512 ) k_rhs( BoraGridDev g, BoraTilesDev t, BoraCellsDev c, uint32_t* nfluid )
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
#pragma unroll 2
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
    const bool fluid = sf[h] == BORA_FLUID;
    const unsigned fl = __ballot_sync( 0xffffffffu, fluid );  // unknowns of the system, counted per warp
    if( ( threadIdx.x & 31 ) == 0 && fl ) atomicAdd( nfluid, (uint32_t)__popc( fl ) );
    if( !fluid )
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
// Wavefront tables of an 8^3 tile: cells ordered by plane i+j+k (0..21). Kept in global
// memory and copied to shared memory by every CTA that sweeps planes (lanes of a warp
// read different entries, which a constant-memory table would serialise).
__device__ uint16_t g_plane_cells[512];
__device__ uint16_t g_plane_start[23];

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

void ensure_tables()
{
    static BoraPerDevice ready;
    ready.get( [] {
        static const PlaneTables tbl;
        cudaMemcpyToSymbol( g_plane_cells, tbl.cells, sizeof( tbl.cells ) );
        cudaMemcpyToSymbol( g_plane_start, tbl.start, sizeof( tbl.start ) );
        cudaDeviceSynchronize();  // the tables are in place before any stream's kernel reads them
        return 1;
    } );
}

int num_sms()
{
    static BoraPerDevice sms;
    return sms.get( [] {
        int dev = 0, n = 0;
        cudaGetDevice( &dev );
        cudaDeviceGetAttribute( &n, cudaDevAttrMultiProcessorCount, dev );
        return n > 0 ? n : 152;
    } );
}

__device__ inline void load_plane_tables( uint16_t* pc, uint16_t* ps )
{
    for( int q = threadIdx.x; q < 512; q += blockDim.x ) pc[q] = g_plane_cells[q];
    if( threadIdx.x < 23 ) ps[threadIdx.x] = g_plane_start[threadIdx.x];
}

__device__ inline int code_diag( uint16_t c ) { return ( c >> 8 ) & 15; }

// Block-MIC(0) pivots (MIC(0) of BLAS.cu:211-262 with tau = 0.97, restricted to the
// couplings inside each 8^3 tile so that tiles factor independently). One warp per
// tile, persistent over tiles.
constexpr int kTilesPerCta = 4;

__global__ void __launch_bounds__( 32 * kTilesPerCta ) k_mic_factor( int ntiles, const uint16_t* __restrict__ code,
                                                                     float* __restrict__ minv )
{
    __shared__ float sm[kTilesPerCta][512];
    __shared__ uint16_t sc[kTilesPerCta][512];
    __shared__ uint16_t pc[512], ps[23];
    load_plane_tables( pc, ps );
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float tau = 0.97f;
    for( int s = blockIdx.x * kTilesPerCta + w; s < ntiles; s += gridDim.x * kTilesPerCta )
    {
        const size_t base = (size_t)s * 512;
        for( int l = lane; l < 512; l += 32 ) { sc[w][l] = code[base + l]; sm[w][l] = 0.f; }
        __syncwarp();
        for( int p = 0; p <= 21; ++p )
        {
            for( int q = ps[p] + lane; q < ps[p + 1]; q += 32 )
            {
                const int l = pc[q];
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
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// PCG update: r -= alpha q; z = M^-1 r (block-MIC(0) forward and backward sweeps over the
// tile's 22 wavefront planes i+j+k = p); rz = r.z and rr = r.r, FP64-accurate. The matching
// e += alpha d is applied by the next direction kernel (which reads d anyway) or by the
// refinement step. One warp per tile, persistent over tiles (every warp gets the same
// number of tiles; the next tile's r, q and pivots are loaded into registers during the
// current tile's sweeps, the one after into L2); alpha is formed once per CTA.
//
// Sweep schedule: each lane owns two x-rows of the tile, (j, kq) and (j, kq + 4) with
// j = lane & 7, kq = lane >> 3, i.e. tile rows lane and lane + 32; the tile's values and
// pivots are staged in shared memory at cell address i + 8 j + 73 k, where the plane pitch
// 73 makes every step's 32 accesses fall in distinct banks. Step u of a sweep handles cell
// i = u - (j + k) - 1 of every row at once, so a lane's cell address is its own row offset
// plus the compile-time u, and the -y, -z (+y, +z) neighbours sit 8 and 73 cells below
// (above) it, computed in the previous step. The -x (+x) neighbour is the lane's own previous
// step, kept in registers. Steps outside a row's eight cells compute with pivot 0 (so they
// yield 0 and feed the row's first cell a zero neighbour) and store nothing; neighbours
// outside the tile (j = 0 / 7, k = 0 / 7) are masked, and zeroed guard cells keep every read
// inside the warp's buffers and finite. The floating-point operations per cell are those of
// the wavefront form: forward y_c = (r_c + M_x y_x + M_y y_y + M_z y_z) M_c as three chained
// FMAs in the order -x, -y, -z; backward z_c = (y_c + M_c (z_x + z_y + z_z)) M_c with the sum
// in the order +x, +y, +z. Non-fluid cells have M = 0 (k_mic_factor) and r = 0.
namespace micsweep {
constexpr int kPlane = 73;                          // buffer pitch of a z-plane (64 cells + 9)
constexpr int kGuard = 80;                          // cells before the tile (reads reach -73)
constexpr int kBuf = kGuard + 7 * kPlane + 64 + kPlane + 7;  // reads reach 574 + 73
constexpr int kWarps = 4;  // 4 x 5.9 KB of buffers per CTA; five CTAs per SM at 96 registers
}  // namespace micsweep
constexpr int kUpdWarps = micsweep::kWarps;

// The update of the warp's tiles first, first + tstride, ...: r -= alpha q, z = M^-1 r; r.z and
// r.r accumulated into prz, prr. sv_w, sp_w: the warp's two sweep buffers (kBuf floats each,
// zeroed before the first call; the sweeps keep their guard cells zero).
__device__ __forceinline__ void pcg_update_tiles( int ntiles, const BoraSolverDev& sv, float alpha, int first, int tstride,
                                                  float* sv_w, float* sp_w, DF& prz, DF& prr )
{
    using namespace micsweep;
    const int lane = threadIdx.x & 31;
    float* const V = sv_w + kGuard;  // tile cell (i, j, k) at V[i + 8 j + kPlane k]
    float* const P = sp_w + kGuard;
    const int j = lane & 7, kq = lane >> 3, sA = j + kq;  // plane offset of row A; row B: sA + 4
    const bool has_ym = j > 0, has_yp = j < 7, has_zmA = kq > 0, has_zpB = kq < 3;
    // cell of row A at step u: VA + u (row B: VB + u)
    const int rA = 8 * j + kPlane * kq, rB = rA + 4 * kPlane;  // element 0 of rows A and B
    const int oA = rA - sA - 1, oB = rB - ( sA + 4 ) - 1;
    float4* const r4 = reinterpret_cast<float4*>( sv.r );
    float4* const z4 = reinterpret_cast<float4*>( sv.z );
    const float4* __restrict__ q4 = reinterpret_cast<const float4*>( sv.q );
    const float4* __restrict__ m4 = reinterpret_cast<const float4*>( sv.minv );
    // Step u of a row with plane offset s. The operands that do not depend on the previous
    // step (the cell's own value and pivot, the neighbours' pivots) are read one step ahead,
    // so that only the two neighbour values computed in the previous step are waited for.
    struct FwdOps { float r, p, py, pz; };
    auto fwd_load = [&]( int o, bool zm ) -> FwdOps {
        return { V[o], P[o], has_ym ? P[o - 8] : 0.f, zm ? P[o - kPlane] : 0.f };
    };
    // y = (r + M_x y_x + M_y y_y + M_z y_z) M
    auto fwd_step = [&]( int o, int u, int s, const FwdOps& c, float& y, float& m ) {
        const bool act = (unsigned)( u - s - 1 ) < 8u;
        const float vy = V[o - 8], vz = V[o - kPlane];
        float t = fmaf( m, y, c.r );
        t = fmaf( c.py, vy, t );
        t = fmaf( c.pz, vz, t );
        m = act ? c.p : 0.f;
        y = t * m;
        if( act ) V[o] = y;
    };
    struct BwdOps { float y, p; };
    auto bwd_load = [&]( int o ) -> BwdOps { return { V[o], P[o] }; };
    // z = (y + M (z_x + z_y + z_z)) M
    auto bwd_step = [&]( int o, int u, int s, bool zp, const BwdOps& c, float& z ) {
        const bool act = (unsigned)( u - s - 1 ) < 8u;
        const float zy = has_yp ? V[o + 8] : 0.f, zz = zp ? V[o + kPlane] : 0.f;
        float acc = 0.f;
        acc += z;
        acc += zy;
        acc += zz;
        const float m = act ? c.p : 0.f;
        z = fmaf( m, acc, c.y ) * m;
        if( act ) V[o] = z;
    };
    // global traffic in whole-warp 512-byte float4 runs: float4 c = lane + 32 m of a tile holds
    // cells 4c .. 4c + 3, which sit at buffer address 4c + 9 k, k = c >> 4
    const int cbase = 4 * lane + 9 * ( lane >> 4 );  // + 146 m
    auto prefetch_tile = [&]( int s ) {  // the tile's r, q and pivots into L2
        if( s < ntiles && lane < 3 )
        {
            const float* src = ( lane == 0 ? sv.r : lane == 1 ? sv.q : sv.minv ) + (size_t)s * 512;
            asm volatile( "cp.async.bulk.prefetch.L2.global [%0], 2048;" ::"l"( src ) : "memory" );
        }
    };
    // the next tile's r, q and pivots are loaded into registers before this tile's sweeps
    float4 rn[4], qn[4], mn[4];
    auto load_tile = [&]( int s ) {
        if( s >= ntiles ) return;
#pragma unroll
        for( int m = 0; m < 4; ++m )
        {
            const size_t o = (size_t)s * 128 + lane + 32 * m;
            rn[m] = r4[o];
            qn[m] = q4[o];
            mn[m] = m4[o];
        }
    };
    load_tile( first );
    for( int s = first; s < ntiles; s += tstride )
    {
        const size_t b4 = (size_t)s * 128 + lane;
        float4 r[4];
#pragma unroll
        for( int m = 0; m < 4; ++m )
        {
            r[m] = rn[m];
            const float4 q = qn[m];
            const float4 mv = mn[m];
            r[m].x = fmaf( -alpha, q.x, r[m].x ); r[m].y = fmaf( -alpha, q.y, r[m].y );
            r[m].z = fmaf( -alpha, q.z, r[m].z ); r[m].w = fmaf( -alpha, q.w, r[m].w );
            r4[b4 + 32 * m] = r[m];
            const int c = cbase + 146 * m;
            V[c] = r[m].x; V[c + 1] = r[m].y; V[c + 2] = r[m].z; V[c + 3] = r[m].w;
            P[c] = mv.x; P[c + 1] = mv.y; P[c + 2] = mv.z; P[c + 3] = mv.w;
            prr = df_add_f( prr, dot4( r[m], r[m] ) );
        }
        load_tile( s + tstride );
        prefetch_tile( s + 2 * tstride );
        __syncwarp();
        // forward: row A holds cells at u = 1 .. 18, row B at u = 5 .. 22
        {
            float yA = 0.f, mA = 0.f, yB = 0.f, mB = 0.f;  // the -x neighbour (previous step)
            FwdOps cA = fwd_load( oA + 1, has_zmA ), cB = { 0.f, 0.f, 0.f, 0.f };
#pragma unroll
            for( int u = 1; u <= 22; ++u )
            {
                FwdOps nA = { 0.f, 0.f, 0.f, 0.f }, nB = { 0.f, 0.f, 0.f, 0.f };
                if( u + 1 <= 18 ) nA = fwd_load( oA + u + 1, has_zmA );
                if( u + 1 >= 5 && u + 1 <= 22 ) nB = fwd_load( oB + u + 1, true );
                if( u <= 18 ) fwd_step( oA + u, u, sA, cA, yA, mA );
                if( u >= 5 ) fwd_step( oB + u, u, sA + 4, cB, yB, mB );
                cA = nA;
                cB = nB;
                __syncwarp();
            }
        }
        // backward, in place over y
        {
            float zA = 0.f, zB = 0.f;  // the +x neighbour (previous step)
            BwdOps cB = bwd_load( oB + 22 ), cA = { 0.f, 0.f };
#pragma unroll
            for( int u = 22; u >= 1; --u )
            {
                BwdOps nA = { 0.f, 0.f }, nB = { 0.f, 0.f };
                if( u - 1 >= 5 ) nB = bwd_load( oB + u - 1 );
                if( u - 1 >= 1 && u - 1 <= 18 ) nA = bwd_load( oA + u - 1 );
                if( u >= 5 ) bwd_step( oB + u, u, sA + 4, has_zpB, cB, zB );
                if( u <= 18 ) bwd_step( oA + u, u, sA, true, cA, zA );
                cA = nA;
                cB = nB;
                __syncwarp();
            }
        }
#pragma unroll
        for( int m = 0; m < 4; ++m )
        {
            const int c = cbase + 146 * m;
            const float4 z = make_float4( V[c], V[c + 1], V[c + 2], V[c + 3] );
            z4[b4 + 32 * m] = z;
            prz = df_add_f( prz, dot4( r[m], z ) );
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__( 32 * kUpdWarps, 5 ) k_pcg_update( int ntiles, BoraSolverDev sv, BoraReduceDev red,
                                                                  int slot_rz_in, int slot_dq_in, int slot_rz_out,
                                                                  int slot_rr_out )
{
    using namespace micsweep;
    __shared__ __align__( 16 ) float sval[kUpdWarps][kBuf];
    __shared__ __align__( 16 ) float spiv[kUpdWarps][kBuf];
    __shared__ float s_alpha;
    bora_pdl_trigger();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for( int q = lane; q < kBuf; q += 32 ) { sval[w][q] = 0.f; spiv[w][q] = 0.f; }
    bora_pdl_wait();  // the previous kernel's results are complete from here
    if( threadIdx.x == 0 ) s_alpha = slot_rz_in < 0 ? 0.f : (float)( red.ring[slot_rz_in] / red.ring[slot_dq_in] );
    __syncthreads();
    DF prz{ 0.f, 0.f }, prr{ 0.f, 0.f };
    pcg_update_tiles( ntiles, sv, s_alpha, blockIdx.x * kUpdWarps + w, gridDim.x * kUpdWarps, sval[w], spiv[w], prz, prr );
    reduce2_publish_df( prz, prr, red, slot_rz_out, slot_rr_out );
}

// Global index of the face neighbour of cell (slot s, local l) in direction q
// (0:-x 1:+x 2:-y 3:+y 4:-z 5:+z), or SIZE_MAX when the neighbour tile is not active
// (a stencil code that names a fluid neighbour there is inconsistent; callers record
// it and skip the access).
__device__ inline size_t face_nbr( const int32_t* __restrict__ nbr, size_t cell, int s, int l, int q )
{
    const int li = l & 7, lj = ( l >> 3 ) & 7, lk = l >> 6;
    int dir, ll;
    switch( q )
    {
        case 0: if( li > 0 ) return cell - 1; dir = 12; ll = l + 7; break;
        case 1: if( li < 7 ) return cell + 1; dir = 14; ll = l - 7; break;
        case 2: if( lj > 0 ) return cell - 8; dir = 10; ll = l + 56; break;
        case 3: if( lj < 7 ) return cell + 8; dir = 16; ll = l - 56; break;
        case 4: if( lk > 0 ) return cell - 64; dir = 4; ll = l + 448; break;
        default: if( lk < 7 ) return cell + 64; dir = 22; ll = l - 448; break;
    }
    const int ns = nbr[(size_t)s * 27 + dir];
    return ns < 0 ? (size_t)-1 : (size_t)ns * 512 + ll;
}

// ---------------------------------------------------------------------------------
// PCG direction: e += alpha d (the previous update's step, pending); d' = z + beta d;
// q = A d'; dq = d'.q (d double-buffered). One warp per tile, persistent over tiles. Each
// lane owns two x-rows of the tile, (j, kq) and (j, kq + 4) with j = lane & 7, kq = lane >> 3
// (tile rows lane and lane + 32), read and written as 16-byte vectors. The stencil's x
// neighbours are the lane's own registers, its y and z neighbours inside the tile come from
// other lanes by shuffles, and the cells of the six face-neighbour tiles that the tile's
// boundary rows need are loaded by the lanes that own those rows (d' formed the same way;
// an inactive neighbour tile contributes 0). Non-fluid cells hold d = z = 0, so the stencil
// sum runs over all six neighbours in the fixed order -x, +x, -y, +y, -z, +z; the dot
// product adds d'.q of cells (i, j, k) and (i, j, k + 4) in float, then into a double-float
// sum.
constexpr int kDirWarps = 4;

// The direction step of the warp's tiles bid * kDirWarps + warp, then every G * kDirWarps:
// returns the thread's d'.q. upd_e: the previous update's e += alpha d is still pending.
__device__ __forceinline__ DF pcg_direction_tiles( int ntiles, const int32_t* __restrict__ nbr,
                                                   const uint16_t* __restrict__ code, const BoraSolverDev& sv, int dsel_in,
                                                   float beta, float alpha, bool upd_e, unsigned bid, unsigned G )
{
    const float* __restrict__ dold = dsel_in ? sv.d[1] : sv.d[0];  // selects keep sv out of local memory
    float* __restrict__ dnew = dsel_in ? sv.d[0] : sv.d[1];
    const int lane = threadIdx.x & 31, j = lane & 7, kq = lane >> 3;
    constexpr unsigned kAll = 0xffffffffu;
    // d' of 8 consecutive cells starting at cell c of tile slot t (0 when t < 0)
    auto halo8 = [&]( int t, int c, float* v ) {
        if( t < 0 ) { for( int i = 0; i < 8; ++i ) v[i] = 0.f; return; }
        const size_t g = (size_t)t * 512 + c;
        const float4 d0 = *reinterpret_cast<const float4*>( dold + g ), d1 = *reinterpret_cast<const float4*>( dold + g + 4 );
        const float4 z0 = *reinterpret_cast<const float4*>( sv.z + g ), z1 = *reinterpret_cast<const float4*>( sv.z + g + 4 );
        v[0] = fmaf( beta, d0.x, z0.x ); v[1] = fmaf( beta, d0.y, z0.y ); v[2] = fmaf( beta, d0.z, z0.z ); v[3] = fmaf( beta, d0.w, z0.w );
        v[4] = fmaf( beta, d1.x, z1.x ); v[5] = fmaf( beta, d1.y, z1.y ); v[6] = fmaf( beta, d1.z, z1.z ); v[7] = fmaf( beta, d1.w, z1.w );
    };
    auto halo1 = [&]( int t, int c ) { return t < 0 ? 0.f : fmaf( beta, dold[(size_t)t * 512 + c], sv.z[(size_t)t * 512 + c] ); };
    DF pdq{ 0.f, 0.f };
    for( int s = (int)bid * kDirWarps + ( threadIdx.x >> 5 ); s < ntiles; s += (int)G * kDirWarps )
    {
        const int32_t* __restrict__ nb = nbr + (size_t)s * 27;  // tile tables: not written by the solver chain
        const int smx = nb[bora_dir( -1, 0, 0 )], spx = nb[bora_dir( 1, 0, 0 )];
        const int smy = nb[bora_dir( 0, -1, 0 )], spy = nb[bora_dir( 0, 1, 0 )];
        const int smz = nb[bora_dir( 0, 0, -1 )], spz = nb[bora_dir( 0, 0, 1 )];
        const size_t gA = (size_t)s * 512 + 8 * lane, gB = gA + 256;
        // own rows: d' = z + beta d and the pending e += alpha d, both stored right away
        float dA[8], dB[8];
        uint16_t cA[8], cB[8];
#pragma unroll
        for( int r = 0; r < 2; ++r )
        {
            const size_t g = r ? gB : gA;
            float* dn = r ? dB : dA;
            uint16_t* cc = r ? cB : cA;
            halo8( s, (int)( g - (size_t)s * 512 ), dn );
            reinterpret_cast<float4*>( dnew + g )[0] = make_float4( dn[0], dn[1], dn[2], dn[3] );
            reinterpret_cast<float4*>( dnew + g )[1] = make_float4( dn[4], dn[5], dn[6], dn[7] );
            const uint4 cw = *reinterpret_cast<const uint4*>( code + g );
            const uint32_t w4[4] = { cw.x, cw.y, cw.z, cw.w };
#pragma unroll
            for( int i = 0; i < 4; ++i ) { cc[2 * i] = (uint16_t)( w4[i] & 0xffffu ); cc[2 * i + 1] = (uint16_t)( w4[i] >> 16 ); }
            if( upd_e )
            {
                const float4 d0 = *reinterpret_cast<const float4*>( dold + g ), d1 = *reinterpret_cast<const float4*>( dold + g + 4 );
                float4 e0 = *reinterpret_cast<const float4*>( sv.e + g ), e1 = *reinterpret_cast<const float4*>( sv.e + g + 4 );
                e0.x = fmaf( alpha, d0.x, e0.x ); e0.y = fmaf( alpha, d0.y, e0.y ); e0.z = fmaf( alpha, d0.z, e0.z ); e0.w = fmaf( alpha, d0.w, e0.w );
                e1.x = fmaf( alpha, d1.x, e1.x ); e1.y = fmaf( alpha, d1.y, e1.y ); e1.z = fmaf( alpha, d1.z, e1.z ); e1.w = fmaf( alpha, d1.w, e1.w );
                reinterpret_cast<float4*>( sv.e + g )[0] = e0;
                reinterpret_cast<float4*>( sv.e + g )[1] = e1;
            }
        }
        // neighbour-tile cells: x ends of both rows; the y face row of lanes j = 0 / 7 (row A
        // here, row B after row A's stencil); the z face row of row A at k = 0 (-z) and of row
        // B at k = 7 (+z)
        const float xmA = halo1( smx, 8 * lane + 7 ), xpA = halo1( spx, 8 * lane );
        const float xmB = halo1( smx, 256 + 8 * lane + 7 ), xpB = halo1( spx, 256 + 8 * lane );
        const int yt = j == 0 ? smy : ( j == 7 ? spy : -1 );
        const int yc = 8 * ( lane - j ) + ( j == 0 ? 56 : 0 );  // row (7 or 0, kq) of the neighbour tile
        float yh[8], zh[8];
        halo8( yt, yc, yh );
        {
            const int zt = kq == 0 ? smz : ( kq == 3 ? spz : -1 );
            const int zc = 8 * j + ( kq == 0 ? 448 : 0 );  // row (j, 7) or (j, 0) of the neighbour tile
            halo8( zt, zc, zh );
        }
        // q = A d' and d'.q, row A then row B (both rows' d' feed the z shuffles)
        float q[8], tA[8];
#pragma unroll
        for( int i = 0; i < 8; ++i )
        {
            float ymA = __shfl_up_sync( kAll, dA[i], 1 ), ypA = __shfl_down_sync( kAll, dA[i], 1 );
            if( j == 0 ) ymA = yh[i];
            if( j == 7 ) ypA = yh[i];
            float zmA = __shfl_up_sync( kAll, dA[i], 8 );
            if( kq == 0 ) zmA = zh[i];
            const float zpA = __shfl_sync( kAll, kq == 0 ? dB[i] : dA[i], ( lane + 8 ) & 31 );
            const float xmA_ = i > 0 ? dA[i > 0 ? i - 1 : 0] : xmA, xpA_ = i < 7 ? dA[i < 7 ? i + 1 : 7] : xpA;
            q[i] = 0.f;
            tA[i] = 0.f;
            if( cA[i] & BORA_CODE_FLUID )
            {
                float acc = 0.f;
                acc += xmA_; acc += xpA_; acc += ymA; acc += ypA; acc += zmA; acc += zpA;
                q[i] = fmaf( (float)code_diag( cA[i] ), dA[i], -acc );
                tA[i] = fmaf( dA[i], q[i], 0.f );
            }
        }
        reinterpret_cast<float4*>( sv.q + gA )[0] = make_float4( q[0], q[1], q[2], q[3] );
        reinterpret_cast<float4*>( sv.q + gA )[1] = make_float4( q[4], q[5], q[6], q[7] );
        halo8( yt, yc + 256, yh );
#pragma unroll
        for( int i = 0; i < 8; ++i )
        {
            float ymB = __shfl_up_sync( kAll, dB[i], 1 ), ypB = __shfl_down_sync( kAll, dB[i], 1 );
            if( j == 0 ) ymB = yh[i];
            if( j == 7 ) ypB = yh[i];
            const float zmB = __shfl_sync( kAll, kq == 3 ? dA[i] : dB[i], ( lane + 24 ) & 31 );
            float zpB = __shfl_down_sync( kAll, dB[i], 8 );
            if( kq == 3 ) zpB = zh[i];
            const float xmB_ = i > 0 ? dB[i > 0 ? i - 1 : 0] : xmB, xpB_ = i < 7 ? dB[i < 7 ? i + 1 : 7] : xpB;
            q[i] = 0.f;
            float t = tA[i];
            if( cB[i] & BORA_CODE_FLUID )
            {
                float acc = 0.f;
                acc += xmB_; acc += xpB_; acc += ymB; acc += ypB; acc += zmB; acc += zpB;
                q[i] = fmaf( (float)code_diag( cB[i] ), dB[i], -acc );
                t = fmaf( dB[i], q[i], t );
            }
            pdq = df_add_f( pdq, t );
        }
        reinterpret_cast<float4*>( sv.q + gB )[0] = make_float4( q[0], q[1], q[2], q[3] );
        reinterpret_cast<float4*>( sv.q + gB )[1] = make_float4( q[4], q[5], q[6], q[7] );
    }
    return pdq;
}

__device__ __forceinline__ void pcg_direction_body( int ntiles, const int32_t* __restrict__ nbr,
                                                    const uint16_t* __restrict__ code, const BoraSolverDev& sv, int dsel_in,
                                                    const BoraReduceDev& red, int slot_rz_new, int slot_rz_old,
                                                    int slot_dq_out, int slot_a_rz, int slot_a_dq, unsigned bid, unsigned G )
{
    __shared__ float s_beta, s_alpha;
    bora_pdl_trigger();
    bora_pdl_wait();  // the previous kernel's results (ring, z, d, e) are complete from here
    if( threadIdx.x == 0 )
    {
        s_beta = slot_rz_old < 0 ? 0.f : (float)( red.ring[slot_rz_new] / red.ring[slot_rz_old] );
        s_alpha = slot_a_rz < 0 ? 0.f : (float)( red.ring[slot_a_rz] / red.ring[slot_a_dq] );
    }
    __syncthreads();
    const DF pdq = pcg_direction_tiles( ntiles, nbr, code, sv, dsel_in, s_beta, s_alpha, slot_a_rz >= 0, bid, G );
    reduce2_publish_warp( df_warp_sum( pdq ), 0.0, 0, red, slot_dq_out, -1, bid, G );
}

__global__ void __launch_bounds__( 32 * kDirWarps, 7 ) k_pcg_direction( int ntiles, const int32_t* __restrict__ nbr,
                                                                    const uint16_t* __restrict__ code, BoraSolverDev sv,
                                                                    int dsel_in, BoraReduceDev red, int slot_rz_new,
                                                                    int slot_rz_old, int slot_dq_out, int slot_a_rz,
                                                                    int slot_a_dq )
{
    pcg_direction_body( ntiles, nbr, code, sv, dsel_in, red, slot_rz_new, slot_rz_old, slot_dq_out, slot_a_rz, slot_a_dq,
                        blockIdx.x, gridDim.x );
}

// Batched: each simulation on its own grid of m.grid[kGridDir] blocks.
__global__ void __launch_bounds__( 32 * kDirWarps ) k_pcg_direction_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    const BoraMemberSlots& q = L.sl[k];
    pcg_direction_body( m.ntiles, m.nbr, m.code, m.sv, q.dsel, m.red, q.rz_new, q.rz_old, q.dq, q.a_rz, q.a_dq, bid,
                        (unsigned)m.grid[kGridDir] );
}

// ---------------------------------------------------------------------------------
// Persistent plain PCG: one cooperative launch runs a refinement pass's inner iterations -
// the first update (z = M^-1 r), then direction and update per iteration - with a grid-wide
// barrier after each phase instead of a kernel boundary. The phases are the kernels' own tile
// loops; a phase's sums are formed per block (warps in a fixed order), stored, and after the
// barrier every block adds all blocks' values in the same fixed order, so each block holds
// the same bits without a second barrier. The pass stops after the update whose ||r|| reaches
// the target (checked in the kernel, the same in every block) or after max_inner iterations.
//
// Every barrier wait is bounded: a block that has spun `limit` times, or that sees another
// block's error, sets BORA_REDUCE_ERR_BARRIER in the error word and returns; every other block
// then runs out of its own waits and returns too, and the host reports BORA_ERR_INTERNAL.
struct PcgPersistArgs
{
    int ntiles;
    const int32_t* nbr;
    const uint16_t* code;
    BoraSolverDev sv;
    BoraReduceDev red;
    int dsel;                  // the current search-direction buffer
    int slot_rz_prev;          // r.z before the last update of the previous pass, or -1 (restart)
    int max_inner;
    double target;             // stop once ||r|| <= target
    int slot_a_rz, slot_a_dq;  // out: the last update's alpha = a_rz / a_dq (its e += alpha d is pending)
    int slot_rr;               // out: the last r.r
    uint32_t* iters;           // out: iterations run
    unsigned* bar;             // barrier count and generation (zeroed before the launch)
    unsigned expect;           // blocks a barrier waits for (gridDim.x)
    unsigned limit;            // spins per barrier wait
    double* part;              // 3 * gridDim.x block sums
};

__device__ __forceinline__ bool grid_barrier( const PcgPersistArgs& a )
{
    __shared__ int s_ok;
    __syncthreads();
    if( threadIdx.x == 0 )
    {
        volatile unsigned* gen = a.bar + 1;
        volatile uint32_t* err = a.red.err;
        int ok = 1;
        const unsigned g = *gen;
        __threadfence();
        if( atomicAdd( a.bar, 1u ) == a.expect - 1 )
        {
            atomicExch( a.bar, 0u );
            __threadfence();
            atomicAdd( a.bar + 1, 1u );
        }
        else
        {
            for( unsigned n = 0; *gen == g; ++n )
            {
                if( n >= a.limit || *err )
                {
                    atomicOr( a.red.err, (uint32_t)BORA_REDUCE_ERR_BARRIER );
                    ok = 0;
                    break;
                }
                __nanosleep( 128 );
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The block's total of v (valid in every lane of every warp), stored at part[blockIdx.x].
__device__ __forceinline__ void block_sum_store( double v, double* part )
{
    __shared__ double w[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if( lane == 0 ) w[wid] = v;
    __syncthreads();
    if( threadIdx.x == 0 )
    {
        double t = 0.0;
        for( int q = 0; q < nw; ++q ) t += w[q];
        part[blockIdx.x] = t;
    }
    __syncthreads();  // w is reused by the next call
}

// The sum of part[0 .. nb) in a fixed order (the first warp: lane-strided, then a fixed
// shuffle tree), returned in every thread.
__device__ __forceinline__ double grid_sum( const double* part, unsigned nb )
{
    __shared__ double s_total;
    if( threadIdx.x < 32 )
    {
        double t = 0.0;
        for( unsigned q = threadIdx.x; q < nb; q += 32 ) t += __ldcg( part + q );
        t = warp_sum( t );
        if( threadIdx.x == 0 ) s_total = t;
    }
    __syncthreads();
    const double v = s_total;
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__( 32 * kUpdWarps, 3 ) k_pcg_persistent( const __grid_constant__ PcgPersistArgs a )
{
    using namespace micsweep;
    static_assert( kUpdWarps == kDirWarps, "both phases run one tile per warp" );
    __shared__ __align__( 16 ) float sval[kUpdWarps][kBuf];
    __shared__ __align__( 16 ) float spiv[kUpdWarps][kBuf];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for( int q = lane; q < kBuf; q += 32 ) { sval[w][q] = 0.f; spiv[w][q] = 0.f; }
    __syncwarp();
    const unsigned G = gridDim.x;
    double* const pd = a.part;                // d'.q
    double* const pz = a.part + G;            // r.z
    double* const pr = a.part + 2 * (size_t)G;  // r.r
    const int first = blockIdx.x * kUpdWarps + w, stride = G * kUpdWarps;
    double rz_prev = a.slot_rz_prev >= 0 ? a.red.ring[a.slot_rz_prev] : -1.0;
    // the pass's first update: z = M^-1 r (alpha 0)
    DF prz{ 0.f, 0.f }, prr{ 0.f, 0.f };
    pcg_update_tiles( a.ntiles, a.sv, 0.f, first, stride, sval[w], spiv[w], prz, prr );
    block_sum_store( df_warp_sum( prz ), pz );
    block_sum_store( df_warp_sum( prr ), pr );
    if( !grid_barrier( a ) ) return;
    double rz = grid_sum( pz, G ), rr = grid_sum( pr, G );
    double a_rz = -1.0, a_dq = 1.0;
    int dsel = a.dsel, it = 0;
    while( it < a.max_inner )
    {
        const float beta = rz_prev < 0.0 ? 0.f : (float)( rz / rz_prev );
        const float alpha_e = a_rz < 0.0 ? 0.f : (float)( a_rz / a_dq );
        const DF pdq = pcg_direction_tiles( a.ntiles, a.nbr, a.code, a.sv, dsel, beta, alpha_e, a_rz >= 0.0, blockIdx.x, G );
        block_sum_store( df_warp_sum( pdq ), pd );
        if( !grid_barrier( a ) ) return;
        const double dq = grid_sum( pd, G );
        dsel ^= 1;
        prz = DF{ 0.f, 0.f };
        prr = DF{ 0.f, 0.f };
        pcg_update_tiles( a.ntiles, a.sv, (float)( rz / dq ), first, stride, sval[w], spiv[w], prz, prr );
        block_sum_store( df_warp_sum( prz ), pz );
        block_sum_store( df_warp_sum( prr ), pr );
        if( !grid_barrier( a ) ) return;
        a_rz = rz;
        a_dq = dq;
        rz_prev = rz;
        rz = grid_sum( pz, G );
        rr = grid_sum( pr, G );
        ++it;
        if( !( rr > 0.0 ) || sqrt( rr ) <= a.target ) break;
    }
    if( blockIdx.x == 0 && threadIdx.x == 0 )
    {
        a.red.ring[a.slot_a_rz] = a_rz;
        a.red.ring[a.slot_a_dq] = a_dq;
        a.red.ring[a.slot_rr] = rr;
        if( a.red.mirror )
        {
            a.red.mirror[a.slot_a_rz] = a_rz;
            a.red.mirror[a.slot_a_dq] = a_dq;
            a.red.mirror[a.slot_rr] = rr;
        }
        *a.iters = (uint32_t)it;
    }
}

// ---------------------------------------------------------------------------------
__device__ __forceinline__ void solve_init_body( size_t ncells, const float* __restrict__ b, const BoraSolverDev& sv,
                                                 const BoraReduceDev& red, int slot_norm2, int slot_max, unsigned bid,
                                                 unsigned G )
{
    DF n2{ 0.f, 0.f };
    float mx = 0.f;
    for( size_t i = bid * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)G * blockDim.x )
    {
        const float bv = b[i];
        sv.r[i] = bv;
        sv.x[i] = make_float2( 0.f, 0.f );
        sv.e[i] = 0.f;
        sv.d[0][i] = 0.f;
        sv.d[1][i] = 0.f;
        sv.q[i] = 0.f;
        n2 = df_add( n2, df_prod( bv, bv ) );
        mx = fmaxf( mx, fabsf( bv ) );
    }
    reduce2_publish_dfmax( n2, mx, red, slot_norm2, slot_max, bid, G );
}

// The warm start of a solve: x = the last step's pressure on fluid cells whose tile was active
// then (slot_prev: the previous tile table, virtual tile -> slot), 0 elsewhere.
__global__ void k_solve_warm( size_t ncells, const uint16_t* __restrict__ code, const int32_t* __restrict__ tile_of,
                              const int32_t* __restrict__ slot_prev, const float* __restrict__ pres, float2* __restrict__ x )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)gridDim.x * blockDim.x )
    {
        float v = 0.f;
        if( code[i] & BORA_CODE_FLUID )
        {
            const int os = slot_prev[tile_of[i >> 9]];
            if( os >= 0 ) v = pres[(size_t)os * BORA_TILE_CELLS + ( i & ( BORA_TILE_CELLS - 1 ) )];
        }
        x[i] = make_float2( v, 0.f );
    }
}

__global__ void k_solve_init( size_t ncells, const float* __restrict__ b, BoraSolverDev sv, BoraReduceDev red,
                              int slot_norm2, int slot_max )
{
    solve_init_body( ncells, b, sv, red, slot_norm2, slot_max, blockIdx.x, gridDim.x );
}

__global__ void k_solve_init_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    const BoraMemberSlots& q = L.sl[k];
    solve_init_body( (size_t)m.ntiles * 512, m.b, m.sv, m.red, q.n2, q.mx, bid, (unsigned)m.grid[kGridCells] );
}

// x += e (+ the last update's pending alpha d), then clear e and q; the direction d is kept
// (the next refinement pass continues the recurrence from it).
__device__ __forceinline__ void refine_accumulate_body( size_t ncells, const uint16_t* __restrict__ code,
                                                        const BoraSolverDev& sv, int dsel, const double* __restrict__ ring,
                                                        int slot_a_rz, int slot_a_dq, unsigned bid, unsigned G )
{
    __shared__ float s_alpha;
    if( threadIdx.x == 0 ) s_alpha = slot_a_rz < 0 ? 0.f : (float)( ring[slot_a_rz] / ring[slot_a_dq] );
    __syncthreads();
    const float alpha = s_alpha;
    const float* __restrict__ d = dsel ? sv.d[1] : sv.d[0];
    for( size_t i = bid * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)G * blockDim.x )
    {
        const float e = slot_a_rz < 0 ? sv.e[i] : fmaf( alpha, d[i], sv.e[i] );
        if( code[i] & BORA_CODE_FLUID )
        {
            const float2 x = sv.x[i];
            const DF y = df_add_f( DF{ x.x, x.y }, e );
            sv.x[i] = make_float2( y.hi, y.lo );
        }
        sv.e[i] = 0.f;
        sv.q[i] = 0.f;
    }
}

__global__ void k_refine_accumulate( size_t ncells, const uint16_t* __restrict__ code, BoraSolverDev sv, int dsel,
                                     const double* __restrict__ ring, int slot_a_rz, int slot_a_dq )
{
    refine_accumulate_body( ncells, code, sv, dsel, ring, slot_a_rz, slot_a_dq, blockIdx.x, gridDim.x );
}

__global__ void k_refine_accumulate_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    const BoraMemberSlots& q = L.sl[k];
    refine_accumulate_body( (size_t)m.ntiles * 512, m.code, m.sv, q.dsel, m.red.ring, q.a_rz, q.a_dq, bid,
                            (unsigned)m.grid[kGridCells] );
}

// r = b - A x in double-float arithmetic (A from the stencil code, x the double-float
// iterate); r stored in FP32, ||r||^2 and max|r| reduced. Streaming, one thread per cell.
// GB300's FP64 pipe is narrow: in FP64 this kernel and the accumulation were bound by it.
__device__ __forceinline__ void refine_residual_body( size_t ncells, const int32_t* __restrict__ nbr,
                                                      const float* __restrict__ b, const uint16_t* __restrict__ code,
                                                      const BoraSolverDev& sv, const BoraReduceDev& red, int slot_norm2,
                                                      int slot_max, unsigned bid, unsigned G )
{
    DF n2{ 0.f, 0.f };
    float mx = 0.f;
    for( size_t cell = bid * (size_t)blockDim.x + threadIdx.x; cell < ncells; cell += (size_t)G * blockDim.x )
    {
        const uint16_t cc = code[cell];
        if( !( cc & BORA_CODE_FLUID ) ) { sv.r[cell] = 0.f; continue; }
        const int s = (int)( cell >> 9 ), l = (int)( cell & 511 );
        DF acc{ 0.f, 0.f };
#pragma unroll
        for( int q = 0; q < 6; ++q )
        {
            if( !( cc & ( 1u << q ) ) ) continue;
            const size_t nc = face_nbr( nbr, cell, s, l, q );
            if( nc == (size_t)-1 ) { atomicOr( red.err, 2u ); continue; }
            const float2 xn = sv.x[nc];
            acc = df_add( acc, DF{ xn.x, xn.y } );
        }
        const float2 xc = sv.x[cell];
        const float dg = (float)code_diag( cc );
        const DF ax = df_add_f( df_prod( xc.x, dg ), xc.y * dg );  // diag * x (diag <= 12)
        const DF t = df_add( ax, DF{ -acc.hi, -acc.lo } );
        const DF rv = df_add_f( DF{ -t.hi, -t.lo }, b[cell] );
        const float rf = rv.hi + rv.lo;
        sv.r[cell] = rf;
        n2 = df_add( n2, df_prod( rf, rf ) );
        mx = fmaxf( mx, fabsf( rf ) );
    }
    reduce2_publish_dfmax( n2, mx, red, slot_norm2, slot_max, bid, G );
}

__global__ void __launch_bounds__( 256 ) k_refine_residual( size_t ncells, const int32_t* __restrict__ nbr,
                                                            const float* __restrict__ b, const uint16_t* __restrict__ code,
                                                            BoraSolverDev sv, BoraReduceDev red, int slot_norm2,
                                                            int slot_max )
{
    refine_residual_body( ncells, nbr, b, code, sv, red, slot_norm2, slot_max, blockIdx.x, gridDim.x );
}

__global__ void __launch_bounds__( 256 ) k_refine_residual_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    const BoraMemberSlots& q = L.sl[k];
    refine_residual_body( (size_t)m.ntiles * 512, m.nbr, m.b, m.code, m.sv, m.red, q.n2, q.mx, bid,
                          (unsigned)m.grid[kGridResidual] );
}

__global__ void k_write_pressure( size_t ncells, const uint16_t* __restrict__ code, const float2* __restrict__ x,
                                  float* __restrict__ pres )
{
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)gridDim.x * blockDim.x )
        pres[i] = ( code[i] & BORA_CODE_FLUID ) ? x[i].x + x[i].y : 0.f;
}

__global__ void k_write_pressure_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const BoraMemberSolve& m = L.ms[bora_batch_member( L, blockIdx.x, &bid )];
    const unsigned G = (unsigned)m.grid[kGridCells];
    const size_t ncells = (size_t)m.ntiles * 512;
    for( size_t i = bid * (size_t)blockDim.x + threadIdx.x; i < ncells; i += (size_t)G * blockDim.x )
        m.pres[i] = ( m.code[i] & BORA_CODE_FLUID ) ? m.sv.x[i].x + m.sv.x[i].y : 0.f;
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
    // the pressure is read with the flag, not after it (every active cell holds a pressure,
    // 0 off the fluid), so that a cell's two loads are in flight together
#pragma unroll 4
    for( int h = threadIdx.x; h < H2::N; h += blockDim.x )
    {
        const long long gi = halo_index<2>( g, nb, ti, tj, tk, h );
        if( gi < 0 ) { sf[h] = BORA_AIR; sp[h] = 0.f; }
        else
        {
            const uint8_t f = c.flag[gi];
            const float pr = c.pres[gi];
            sf[h] = f;
            sp[h] = f == BORA_FLUID ? pr : 0.f;
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

void bora_launch_rhs( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, uint32_t* nfluid, cudaStream_t st )
{
    if( ntiles > 0 ) k_rhs<<<ntiles, 512, 0, st>>>( g, t, c, nfluid );
}

void bora_launch_vel_update( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraCellsDev c, cudaStream_t st )
{
    if( ntiles > 0 ) k_vel_update<<<ntiles, 512, 0, st>>>( g, t, c );
}

void bora_launch_mic_factor( const BoraGridDev&, int ntiles, const uint16_t* code, float* minv, cudaStream_t st )
{
    ensure_tables();
    if( ntiles <= 0 ) return;
    const int nb = std::min( ( ntiles + kTilesPerCta - 1 ) / kTilesPerCta, num_sms() * 8 );
    k_mic_factor<<<nb, 32 * kTilesPerCta, 0, st>>>( ntiles, code, minv );
}

void bora_launch_solve_init( int ntiles, const float* b, const uint16_t*, BoraSolverDev s, BoraReduceDev red,
                             int slot_norm2, int slot_max, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    k_solve_init<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, b, s, red, slot_norm2, slot_max );
}

void bora_launch_pcg_update( int ntiles, const uint16_t* code, BoraSolverDev s, BoraReduceDev red, int slot_rz_in,
                             int slot_dq_in, int slot_rz_out, int slot_rr_out, cudaStream_t st )
{
    (void)code;
    static BoraPerDevice per_sm;
    const int bps = per_sm.get( [] {
        int v = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor( &v, k_pcg_update, 32 * kUpdWarps, 0 ) == cudaSuccess && v > 0 ? v : 1;
    } );
    // as many rounds of one tile per warp as the resident warps need, and the grid sized so
    // that every warp gets that many tiles (no warp waits in the reduction for a straggler)
    const int cap = std::max( 1, std::min( bps * num_sms(), kBoraMaxReduceBlocks ) ) * kUpdWarps;
    const int rounds = std::max( 1, ( ntiles + cap - 1 ) / cap );  // one block even for no tiles: it publishes the sums
    const int nb = std::max( 1, ( ntiles + kUpdWarps * rounds - 1 ) / ( kUpdWarps * rounds ) );
    bora_launch_pdl( k_pcg_update, nb, 32 * kUpdWarps, 0, st, ntiles, s, red, slot_rz_in, slot_dq_in, slot_rz_out,
                     slot_rr_out );
}

namespace {
// Grid of the direction kernel: every warp gets the same number of tiles; at most
// kBoraMaxReduceBlocks CTAs (partial sums capacity).
int direction_grid( int ntiles )
{
    if( ntiles <= 0 ) return 0;
    static BoraPerDevice per_sm;
    const int b = per_sm.get( [] {
        int v = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor( &v, k_pcg_direction, 32 * kDirWarps, 0 ) == cudaSuccess && v > 0 ? v : 1;
    } );
    const int cap = std::max( 1, std::min( b * num_sms(), kBoraMaxReduceBlocks ) ) * kDirWarps;
    const int rounds = ( ntiles + cap - 1 ) / cap;
    return std::max( 1, ( ntiles + kDirWarps * rounds - 1 ) / ( kDirWarps * rounds ) );
}
int residual_grid( size_t nc ) { return (int)std::max<size_t>( 1, std::min<size_t>( ( nc + 255 ) / 256, (size_t)num_sms() * 8 ) ); }
}  // namespace

void bora_projection_grids( int ntiles, int* grid )
{
    const size_t nc = (size_t)std::max( ntiles, 0 ) * 512;
    grid[kGridDir] = direction_grid( ntiles );
    grid[kGridCells] = grid_for( nc, 256 );
    grid[kGridResidual] = residual_grid( nc );
}

void bora_launch_solve_init_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks > 0 ) k_solve_init_batch<<<blocks, 256, 0, st>>>( L );
}

void bora_launch_pcg_direction_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks > 0 ) bora_launch_pdl( k_pcg_direction_batch, dim3( blocks ), dim3( 32 * kDirWarps ), 0, st, L );
}

void bora_launch_refine_accumulate_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks > 0 ) k_refine_accumulate_batch<<<blocks, 256, 0, st>>>( L );
}

void bora_launch_refine_residual_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks > 0 ) k_refine_residual_batch<<<blocks, 256, 0, st>>>( L );
}

void bora_launch_write_pressure_batch( const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks > 0 ) k_write_pressure_batch<<<blocks, 256, 0, st>>>( L );
}

int bora_pcg_persistent_grid()
{
    static BoraPerDevice per_sm;
    const int b = per_sm.get( [] {
        int v = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor( &v, k_pcg_persistent, 32 * kUpdWarps, 0 ) == cudaSuccess ? v : 0;
    } );
    return std::min( b * num_sms(), kBoraMaxReduceBlocks );
}

int bora_launch_pcg_persistent( int ntiles, const int32_t* nbr, const uint16_t* code, BoraSolverDev s, BoraReduceDev red,
                                int dsel, int slot_rz_prev, int max_inner, double target, int slot_a_rz, int slot_a_dq,
                                int slot_rr, uint32_t* iters, unsigned* bar, double* part, bool never_release,
                                cudaStream_t st )
{
    const int grid = bora_pcg_persistent_grid();
    if( grid <= 0 ) return -1;
    PcgPersistArgs a{};
    a.ntiles = ntiles; a.nbr = nbr; a.code = code; a.sv = s; a.red = red;
    a.dsel = dsel; a.slot_rz_prev = slot_rz_prev; a.max_inner = max_inner; a.target = target;
    a.slot_a_rz = slot_a_rz; a.slot_a_dq = slot_a_dq; a.slot_rr = slot_rr; a.iters = iters;
    a.bar = bar; a.part = part;
    // a barrier that waits for one block more than there are never releases: every wait runs
    // out (fault injection for tests), after a short limit
    a.expect = (unsigned)grid + ( never_release ? 1u : 0u );
    a.limit = never_release ? ( 1u << 12 ) : ( 1u << 22 );
    if( cudaMemsetAsync( bar, 0, 2 * sizeof( unsigned ), st ) != cudaSuccess ) return -1;
    void* args[] = { &a };
    return cudaLaunchCooperativeKernel( (const void*)k_pcg_persistent, dim3( grid ), dim3( 32 * kUpdWarps ), args, 0, st ) ==
                   cudaSuccess
               ? 0
               : -1;
}

void bora_launch_pcg_direction( const BoraGridDev&, int ntiles, BoraTilesDev t, const uint16_t* code, BoraSolverDev s,
                                int dsel_in, BoraReduceDev red, int slot_rz_new, int slot_rz_old, int slot_dq_out,
                                int slot_a_rz, int slot_a_dq, cudaStream_t st )
{
    if( ntiles <= 0 ) return;
    const int grid = direction_grid( ntiles );
    bora_launch_pdl( k_pcg_direction, grid, 32 * kDirWarps, 0, st, ntiles, (const int32_t*)t.nbr, code, s, dsel_in, red,
                     slot_rz_new, slot_rz_old, slot_dq_out, slot_a_rz, slot_a_dq );
}

void bora_launch_solve_warm( int ntiles, const uint16_t* code, const int32_t* tile_of, const int32_t* slot_prev,
                             const float* pres, BoraSolverDev s, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    if( nc ) k_solve_warm<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, code, tile_of, slot_prev, pres, s.x );
}

void bora_launch_refine_accumulate( int ntiles, const uint16_t* code, BoraSolverDev s, int dsel, const double* ring,
                                    int slot_a_rz, int slot_a_dq, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    if( nc ) k_refine_accumulate<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, code, s, dsel, ring, slot_a_rz, slot_a_dq );
}

void bora_launch_refine_residual( const BoraGridDev&, int ntiles, BoraTilesDev t, const float* b, const uint16_t* code,
                                  BoraSolverDev s, BoraReduceDev red, int slot_norm2, int slot_max, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    k_refine_residual<<<residual_grid( nc ), 256, 0, st>>>( nc, t.nbr, b, code, s, red, slot_norm2, slot_max );
}

void bora_launch_write_pressure( int ntiles, const uint16_t* code, const float2* x, float* pres, cudaStream_t st )
{
    const size_t nc = (size_t)ntiles * 512;
    if( nc ) k_write_pressure<<<grid_for( nc, 256 ), 256, 0, st>>>( nc, code, x, pres );
}
