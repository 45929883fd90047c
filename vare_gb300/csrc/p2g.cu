// P2G on the sparse grid, fused with the particle-count field and the cell flags.
//
// Replaces Rasterization::PointsToVelField / PointsToCountField (sparse,
// base/source/Rasterization.cu:122-229), which scatter with 4 (+1) float atomics per
// stencil cell per particle, and the flags lambda of FLIPMethod::advanceOneStep
// (base/source/FLIPMethod.cu:242-281).
//
// Particles arrive sorted by dual cell (the base cell of the reference's 2x2x2 stencil,
// max(int(p-0.5),0) per axis), so the particles that touch cell c are exactly those of
// the 8 dual cells {c-1, c}^3. One CTA handles one 8^3 tile, one thread one cell, and
// each thread gathers its 8 dual cells: no atomics, one coalesced store per field.
// Weights follow the reference (w = prod max(0, 1-|p-c|) + 1e-5); sums are accumulated
// in 64-bit fixed point (2^-32) so the result does not depend on the order of the
// particles inside a dual cell.
#include "bora_internal.h"

namespace {

constexpr float kFix = 4294967296.0f;     // 2^32
constexpr double kUnfix = 1.0 / 4294967296.0;

__global__ void __launch_bounds__( 512 ) k_p2g( BoraGridDev g, BoraTilesDev t, BoraParticlesDev p,
                                                const uint32_t* __restrict__ idx, const uint32_t* __restrict__ start,
                                                BoraCellsDev c )
{
    __shared__ int32_t nb[27];
    const int s = blockIdx.x;
    if( threadIdx.x < 27 ) nb[threadIdx.x] = t.nbr[(size_t)s * 27 + threadIdx.x];
    __syncthreads();
    const int vt = t.tile_of[s];
    const int ti = vt % g.tx, tj = ( vt / g.tx ) % g.ty, tk = vt / ( g.tx * g.ty );
    const int l = threadIdx.x;
    const int i = ti * BORA_TILE + ( l & 7 ), j = tj * BORA_TILE + ( ( l >> 3 ) & 7 ), k = tk * BORA_TILE + ( l >> 6 );
    const size_t cell = (size_t)s * BORA_TILE_CELLS + l;
    if( i >= g.nx || j >= g.ny || k >= g.nz )
    {
        c.flag[cell] = BORA_MASKED;
        c.mass[cell] = 0.f; c.surf[cell] = 0.f;
        c.vx[cell] = 0.f; c.vy[cell] = 0.f; c.vz[cell] = 0.f;
        return;
    }
    const float ccx = (float)i + .5f, ccy = (float)j + .5f, ccz = (float)k + .5f;
    long long m = 0, mx = 0, my = 0, mz = 0;
    uint32_t cnt = 0;
#pragma unroll 1
    for( int o = 0; o < 8; ++o )
    {
        const int di = i - 1 + ( o & 1 ), dj = j - 1 + ( ( o >> 1 ) & 1 ), dk = k - 1 + ( o >> 2 );
        if( di < 0 || dj < 0 || dk < 0 ) continue;
        const int ns = nb[bora_dir( ( di >> 3 ) - ti, ( dj >> 3 ) - tj, ( dk >> 3 ) - tk )];
        if( ns < 0 ) continue;
        const uint32_t key = (uint32_t)ns * BORA_TILE_CELLS + (uint32_t)bora_local( di, dj, dk );
        const uint32_t q0 = start[key], q1 = start[key + 1];
        cnt += q1 - q0;
        for( uint32_t q = q0; q < q1; ++q )
        {
            const uint32_t pi = idx[q];
            const float x = p.px[pi], y = p.py[pi], z = p.pz[pi];
            const float dx = x - ccx, dy = y - ccy, dz = z - ccz;
            const float xw = fmaxf( 0.f, 1.f - fabsf( dx ) );
            const float yw = fmaxf( 0.f, 1.f - fabsf( dy ) );
            const float zw = fmaxf( 0.f, 1.f - fabsf( dz ) );
            const float w = xw * yw * zw + 1e-05f;
            m += __float2ll_rn( w * kFix );
            mx += __float2ll_rn( ( w * p.vx[pi] ) * kFix );
            my += __float2ll_rn( ( w * p.vy[pi] ) * kFix );
            mz += __float2ll_rn( ( w * p.vz[pi] ) * kFix );
        }
    }
    float vx = 0.f, vy = 0.f, vz = 0.f, mass = 0.f;
    if( m > 0 )
    {
        mass = (float)( (double)m * kUnfix );
        const double dm = (double)m;
        vx = (float)( (double)mx / dm );
        vy = (float)( (double)my / dm );
        vz = (float)( (double)mz / dm );
    }
    // flags and collider velocity (FLIPMethod.cu:244-260)
    uint8_t f;
    const float phi = bora_col_phi( g, ccx, ccy, ccz );
    if( m > 0 ) f = BORA_FLUID;
    else f = phi < 0.f ? BORA_SOLID : BORA_AIR;
    if( phi < 0.f )
    {
        float cv[3];
        bora_col_lerp( g.cols, g.nx, g.ny, g.nz, ccx, ccy, ccz, 2, cv );
        vx += cv[0] * g.col_vel_scale;
        vy += cv[1] * g.col_vel_scale;
        vz += cv[2] * g.col_vel_scale;
    }
    c.flag[cell] = f;
    c.mass[cell] = mass;
    c.surf[cell] = (float)cnt;
    c.vx[cell] = vx;
    c.vy[cell] = vy;
    c.vz[cell] = vz;
}

}  // namespace

void bora_launch_p2g( const BoraGridDev& g, int ntiles, BoraTilesDev t, BoraParticlesDev p, const uint32_t* idx,
                      const uint32_t* start, BoraCellsDev c, cudaStream_t st )
{
    if( ntiles <= 0 ) return;
    k_p2g<<<ntiles, BORA_TILE_CELLS, 0, st>>>( g, t, p, idx, start, c );
}
