// P2G on the sparse grid, fused with the particle-count field and the cell flags.
//
// Replaces Rasterization::PointsToVelField / PointsToCountField (sparse,
// base/source/Rasterization.cu:122-229), which scatter with 4 (+1) float atomics per
// stencil cell per particle, and the flags lambda of FLIPMethod::advanceOneStep
// (base/source/FLIPMethod.cu:242-281).
//
// Particles arrive sorted by dual cell (the base cell of the reference's 2x2x2 stencil,
// max(int(p-0.5),0) per axis), so the particles that touch cell c are exactly those of
// the 8 dual cells {c-1, c}^3. Each dual cell's particles are read once and summed per
// stencil corner, and each cell adds its 8 corner sums - no atomics, one store per field.
// Weights follow the reference (w = prod max(0, 1-|p-c|) + 1e-5); sums are FP32 in a
// fixed order (particles of a dual cell by source index, then a fixed tree over the 8
// dual cells), so the result is bit-reproducible.
#include "bora_internal.h"

namespace {

// Collider velocity at a cell centre (FLIPMethod.cu:248,260), out of line: rare, and its
// corner arrays would otherwise raise the register count of the whole kernel.
__device__ __noinline__ float3 col_velocity( const BoraGridDev* g, float x, float y, float z )
{
    float cv[3];
    bora_col_lerp( g->cols, g->nx, g->ny, g->nz, x, y, z, 2, cv );
    return make_float3( cv[0], cv[1], cv[2] );
}

// One CTA per tile. The threads take the tile's 512 dual cells, then the 217 of its low-side
// halo, one at a time; each reads its dual cell's particles once in bin order (fixed by
// k_order_bins) and keeps the 8 corner sums of m, m*v in registers. Every (cell, source dual cell) pair of
// the tile is produced by exactly one thread and parked in shared memory; each cell then
// adds its 8 sources with a fixed tree, so the result is reproducible. Halo dual cells
// are recomputed by every tile that needs them instead of being exchanged.
constexpr int kP2GThreads = 384;  // two CTAs per SM at 80 registers (the 729 dual cells in two rounds)
constexpr int kP2GHalo = 217;  // 9^3 - 8^3 dual cells with a -1 tile-local coordinate
constexpr size_t kP2GSmem = 8 * 4 * 512 * sizeof( float ) + 8 * 512 * sizeof( uint32_t );

__global__ void __launch_bounds__( kP2GThreads, 2 ) k_p2g( const __grid_constant__ BoraGridDev g, BoraTilesDev t,
                                                           BoraParticlesDev p, const uint32_t* __restrict__ idx,
                                                           const uint32_t* __restrict__ start, BoraCellsDev c )
{
    extern __shared__ float p2g_smem[];
    float* part = p2g_smem;                                         // [o][m, mx, my, mz][cell]
    uint32_t* pcnt = reinterpret_cast<uint32_t*>( p2g_smem + 8 * 4 * 512 );  // [o][cell]
    __shared__ int32_t nb[27];
    const int s = blockIdx.x, tid = threadIdx.x;
    if( tid < 27 ) nb[tid] = t.nbr[(size_t)s * 27 + tid];
    const int vt = t.tile_of[s];
    const int ti = vt % g.tx, tj = ( vt / g.tx ) % g.ty, tk = vt / ( g.tx * g.ty );
    __syncthreads();
    for( int item = tid; item < 512 + kP2GHalo; item += kP2GThreads )
    {
        int di, dj, dk;  // tile-local dual-cell coordinates in [-1, 7]
        if( item < 512 )
        {
            di = item & 7; dj = ( item >> 3 ) & 7; dk = item >> 6;
        }
        else
        {
            const int hh = item - 512;
            if( hh < 81 ) { di = hh % 9 - 1; dj = hh / 9 - 1; dk = -1; }
            else if( hh < 153 ) { const int u = hh - 81; di = u % 9 - 1; dj = -1; dk = u / 9; }
            else { const int u = hh - 153; di = -1; dj = u & 7; dk = u >> 3; }
        }
        const int ns = nb[bora_dir( di < 0 ? -1 : 0, dj < 0 ? -1 : 0, dk < 0 ? -1 : 0 )];
        uint32_t q0 = 0, q1 = 0;
        if( ns >= 0 )
        {
            const uint32_t key = (uint32_t)ns * BORA_TILE_CELLS + (uint32_t)bora_local( di, dj, dk );
            q0 = start[key];
            q1 = start[key + 1];
        }
        // centres of the two cells per axis that the dual cell's particles touch
        const int gi = ti * BORA_TILE + di, gj = tj * BORA_TILE + dj, gk = tk * BORA_TILE + dk;
        const float cx0 = (float)gi + .5f, cx1 = (float)( gi + 1 ) + .5f;
        const float cy0 = (float)gj + .5f, cy1 = (float)( gj + 1 ) + .5f;
        const float cz0 = (float)gk + .5f, cz1 = (float)( gk + 1 ) + .5f;
        float acc[8][4];
#pragma unroll
        for( int o = 0; o < 8; ++o ) acc[o][0] = acc[o][1] = acc[o][2] = acc[o][3] = 0.f;
        for( uint32_t q = q0; q < q1; ++q )
        {
            const uint32_t pi = idx[q];
            const float x = p.px[pi], y = p.py[pi], z = p.pz[pi];
            const float vx = p.vx[pi], vy = p.vy[pi], vz = p.vz[pi];
            const float wx[2] = { fmaxf( 0.f, 1.f - fabsf( x - cx0 ) ), fmaxf( 0.f, 1.f - fabsf( x - cx1 ) ) };
            const float wy[2] = { fmaxf( 0.f, 1.f - fabsf( y - cy0 ) ), fmaxf( 0.f, 1.f - fabsf( y - cy1 ) ) };
            const float wz[2] = { fmaxf( 0.f, 1.f - fabsf( z - cz0 ) ), fmaxf( 0.f, 1.f - fabsf( z - cz1 ) ) };
            // the weight rounds like the reference's; its products with the velocity are
            // accumulated with fused multiply-adds (the sums' order differs from the
            // reference's atomics in any case)
            const float wxy[4] = { wx[0] * wy[0], wx[1] * wy[0], wx[0] * wy[1], wx[1] * wy[1] };
#pragma unroll
            for( int cr = 0; cr < 8; ++cr )  // corner (a, b, c) = bits of cr
            {
                const float w = wxy[cr & 3] * wz[cr >> 2] + 1e-05f;
                acc[cr][0] += w;
                acc[cr][1] = fmaf( w, vx, acc[cr][1] );
                acc[cr][2] = fmaf( w, vy, acc[cr][2] );
                acc[cr][3] = fmaf( w, vz, acc[cr][3] );
            }
        }
        const uint32_t n = q1 - q0;
#pragma unroll
        for( int cr = 0; cr < 8; ++cr )
        {
            const int a = cr & 1, b = ( cr >> 1 ) & 1, cc = cr >> 2;
            const int li = di + a, lj = dj + b, lk = dk + cc;
            if( li < 0 || lj < 0 || lk < 0 || li > 7 || lj > 7 || lk > 7 ) continue;
            const int cell = li | ( lj << 3 ) | ( lk << 6 );
            const int o = 7 - cr;  // the dual cell is cell - 1 + bits(o)
            part[( o * 4 + 0 ) * 512 + cell] = acc[cr][0];
            part[( o * 4 + 1 ) * 512 + cell] = acc[cr][1];
            part[( o * 4 + 2 ) * 512 + cell] = acc[cr][2];
            part[( o * 4 + 3 ) * 512 + cell] = acc[cr][3];
            pcnt[o * 512 + cell] = n;
        }
    }
    __syncthreads();
    // per cell: fixed tree over the 8 source dual cells
    for( int l = tid; l < BORA_TILE_CELLS; l += kP2GThreads )
    {
        auto tree = [&]( int v ) {
            const float* q = part + v * 512 + l;
            return ( ( q[0 * 2048] + q[1 * 2048] ) + ( q[2 * 2048] + q[3 * 2048] ) ) +
                   ( ( q[4 * 2048] + q[5 * 2048] ) + ( q[6 * 2048] + q[7 * 2048] ) );
        };
        const float m = tree( 0 ), mx = tree( 1 ), my = tree( 2 ), mz = tree( 3 );
        uint32_t cnt = 0;
#pragma unroll
        for( int o = 0; o < 8; ++o ) cnt += pcnt[o * 512 + l];
        const size_t cell = (size_t)s * BORA_TILE_CELLS + l;
        const int i = ti * BORA_TILE + ( l & 7 ), j = tj * BORA_TILE + ( ( l >> 3 ) & 7 ), k = tk * BORA_TILE + ( l >> 6 );
        if( !( i < g.nx && j < g.ny && k < g.nz ) )
        {
            c.flag[cell] = BORA_MASKED;
            c.mass[cell] = 0.f; c.surf[cell] = 0.f;
            c.vx[cell] = 0.f; c.vy[cell] = 0.f; c.vz[cell] = 0.f;
            continue;
        }
        const float ccx = (float)i + .5f, ccy = (float)j + .5f, ccz = (float)k + .5f;
        float vx = 0.f, vy = 0.f, vz = 0.f, mass = 0.f;
        if( m > 0.f )
        {
            mass = m;
            vx = mx / m;
            vy = my / m;
            vz = mz / m;
        }
        // flags and collider velocity (FLIPMethod.cu:244-260)
        uint8_t f;
        const float phi = bora_col_phi( g, ccx, ccy, ccz );
        if( m > 0.f ) f = BORA_FLUID;
        else f = phi < 0.f ? BORA_SOLID : BORA_AIR;
        if( phi < 0.f )
        {
            const float3 cv = col_velocity( &g, ccx, ccy, ccz );
            vx += cv.x * g.col_vel_scale;
            vy += cv.y * g.col_vel_scale;
            vz += cv.z * g.col_vel_scale;
        }
        c.flag[cell] = f;
        c.mass[cell] = mass;
        c.surf[cell] = (float)cnt;
        c.vx[cell] = vx;
        c.vy[cell] = vy;
        c.vz[cell] = vz;
    }
}

}  // namespace

void bora_launch_p2g( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraParticlesDev p, const uint32_t* idx,
                      const uint32_t* start, BoraCellsDev c, cudaStream_t st )
{
    if( ntiles <= 0 ) return;
    static BoraPerDevice attr_set;
    attr_set.get( [] {
        cudaFuncSetAttribute( k_p2g, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP2GSmem );
        return 1;
    } );
    k_p2g<<<ntiles, kP2GThreads, kP2GSmem, st>>>( g, t, p, idx, start, c );
}
