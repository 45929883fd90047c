// P2G on the sparse grid, fused with the particle-count field and the cell flags.
//
// Replaces Rasterization::PointsToVelField / PointsToCountField (sparse,
// base/source/Rasterization.cu:122-229), which scatter with 4 (+1) float atomics per
// stencil cell per particle, and the flags lambda of FLIPMethod::advanceOneStep
// (base/source/FLIPMethod.cu:242-281).
//
// Particles arrive sorted by dual cell (the base cell of the reference's 2x2x2 stencil,
// max(int(p-0.5),0) per axis), so the particles that touch cell c are exactly those of
// the 8 dual cells {c-1, c}^3: each cell gathers from its 8 dual cells (one thread per
// dual cell, combined by shuffles) - no atomics, one store per field.
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

// One thread per (cell, dual cell): 8 consecutive lanes own the 8 dual cells {c-1, c}^3
// of one cell, each sums its particles in bin order (fixed by k_order_bins), and the lanes
// combine their sums with a fixed shuffle tree, so the result is reproducible.
__global__ void __launch_bounds__( 256, 5 ) k_p2g( const __grid_constant__ BoraGridDev g, BoraTilesDev t, BoraParticlesDev p,
                                                const uint32_t* __restrict__ idx, const uint32_t* __restrict__ start,
                                                BoraCellsDev c, size_t ncells )
{
    const size_t total = ncells * 8;  // a multiple of 32: every lane of a warp runs the same iterations
    for( size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x; tid < total; tid += (size_t)gridDim.x * blockDim.x )
    {
        const size_t cell = tid >> 3;
        const int o = (int)( tid & 7 );
        const int s = (int)( cell >> 9 ), l = (int)( cell & 511 );
        const int vt = t.tile_of[s];
        const int ti = vt % g.tx, tj = ( vt / g.tx ) % g.ty, tk = vt / ( g.tx * g.ty );
        const int i = ti * BORA_TILE + ( l & 7 ), j = tj * BORA_TILE + ( ( l >> 3 ) & 7 ), k = tk * BORA_TILE + ( l >> 6 );
        const bool real = i < g.nx && j < g.ny && k < g.nz;
        const float ccx = (float)i + .5f, ccy = (float)j + .5f, ccz = (float)k + .5f;
        float m = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
        uint32_t cnt = 0;
        const int di = i - 1 + ( o & 1 ), dj = j - 1 + ( ( o >> 1 ) & 1 ), dk = k - 1 + ( o >> 2 );
        if( real && di >= 0 && dj >= 0 && dk >= 0 )
        {
            const int ns = t.nbr[(size_t)s * 27 + bora_dir( ( di >> 3 ) - ti, ( dj >> 3 ) - tj, ( dk >> 3 ) - tk )];
            if( ns >= 0 )
            {
                const uint32_t key = (uint32_t)ns * BORA_TILE_CELLS + (uint32_t)bora_local( di, dj, dk );
                const uint32_t q0 = start[key], q1 = start[key + 1];
                cnt = q1 - q0;
                for( uint32_t q = q0; q < q1; ++q )
                {
                    const uint32_t pi = idx[q];
                    const float x = p.px[pi], y = p.py[pi], z = p.pz[pi];
                    const float dx = x - ccx, dy = y - ccy, dz = z - ccz;
                    const float xw = fmaxf( 0.f, 1.f - fabsf( dx ) );
                    const float yw = fmaxf( 0.f, 1.f - fabsf( dy ) );
                    const float zw = fmaxf( 0.f, 1.f - fabsf( dz ) );
                    const float w = xw * yw * zw + 1e-05f;
                    m += w;
                    mx += w * p.vx[pi];
                    my += w * p.vy[pi];
                    mz += w * p.vz[pi];
                }
            }
        }
        // fixed butterfly over the 8 dual cells (float addition is commutative, so every
        // lane ends with the same, order-independent value)
#pragma unroll
        for( int sh = 1; sh < 8; sh <<= 1 )
        {
            m += __shfl_xor_sync( 0xffffffffu, m, sh );
            mx += __shfl_xor_sync( 0xffffffffu, mx, sh );
            my += __shfl_xor_sync( 0xffffffffu, my, sh );
            mz += __shfl_xor_sync( 0xffffffffu, mz, sh );
            cnt += __shfl_xor_sync( 0xffffffffu, cnt, sh );
        }
        if( o != 0 ) continue;
        if( !real )
        {
            c.flag[cell] = BORA_MASKED;
            c.mass[cell] = 0.f; c.surf[cell] = 0.f;
            c.vx[cell] = 0.f; c.vy[cell] = 0.f; c.vz[cell] = 0.f;
            continue;
        }
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
    const size_t ncells = (size_t)ntiles * BORA_TILE_CELLS;
    int dev = 0, sms = 0;
    cudaGetDevice( &dev );
    cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
    const size_t want = ( ncells * 8 + 255 ) / 256, cap = (size_t)( sms > 0 ? sms : 152 ) * 16;
    k_p2g<<<(int)( want < cap ? want : cap ), 256, 0, st>>>( g, t, p, idx, start, c, ncells );
}
