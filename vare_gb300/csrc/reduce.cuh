// FP64-accurate, deterministic reductions shared by the solver kernels.
#pragma once

#include "bora_internal.h"

namespace bora_reduce {

// ---------------------------------------------------------------------------------
// Double-float accumulation: GB300's FP64 pipe is ~1/64 of its FP32 rate, so per-cell
// dot-product terms are accumulated as unevaluated float pairs (hi + lo) with the
// error-free TwoProd (fmaf) and TwoSum transformations (Dekker 1971, Knuth TAOCP 4.2.2),
// giving ~48 significant bits from FP32 instructions; each warp converts its pair to
// FP64 once. The product is formed with __fmul_rn, which the compiler never fuses into a
// following addition, so the transformations stay error-free under -fmad=true as well
// (TwoSum has no multiplication to contract).
struct DF
{
    float hi, lo;
};
__device__ __forceinline__ DF df_prod( float a, float b )
{
    const float p = __fmul_rn( a, b );
    return DF{ p, fmaf( a, b, -p ) };
}
__device__ __forceinline__ DF df_add( DF a, DF b )
{
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float err = ( a.hi - ( s - bb ) ) + ( b.hi - bb );
    err += a.lo + b.lo;
    const float h = s + err;
    return DF{ h, err - ( h - s ) };
}
// DF + float (TwoSum with a zero low part).
__device__ __forceinline__ DF df_add_f( DF a, float b )
{
    const float s = a.hi + b;
    const float bb = s - a.hi;
    const float err = ( ( a.hi - ( s - bb ) ) + ( b - bb ) ) + a.lo;
    const float h = s + err;
    return DF{ h, err - ( h - s ) };
}
// FP32 dot product of two float4 (fused multiply-adds). Short FP32 partial sums like this
// one (4 terms, relative error ~2^-22) feed the double-float accumulators: that keeps the
// totals accurate to ~1e-7 relative, far more than the FP32 alpha and beta of PCG need,
// at a quarter of the double-float operations.
__device__ __forceinline__ float dot4( float4 a, float4 b )
{
    return fmaf( a.w, b.w, fmaf( a.z, b.z, fmaf( a.y, b.y, a.x * b.x ) ) );
}
__device__ __forceinline__ double df_warp_sum( DF v )
{
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 )
    {
        DF w;
        w.hi = __shfl_xor_sync( 0xffffffffu, v.hi, o );
        w.lo = __shfl_xor_sync( 0xffffffffu, v.lo, o );
        v = df_add( v, w );
    }
    return (double)v.hi + (double)v.lo;
}
__device__ __forceinline__ float warp_maxf( float v )
{
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) v = fmaxf( v, __shfl_xor_sync( 0xffffffffu, v, o ) );
    return v;
}

// ---------------------------------------------------------------------------------
// Deterministic FP64 block reduction published through a ring slot: every block writes
// its partial, the last block to arrive sums the partials in block order.
__device__ __forceinline__ double warp_sum( double v )
{
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) v += __shfl_xor_sync( 0xffffffffu, v, o );
    return v;
}
__device__ __forceinline__ double warp_max( double v )
{
#pragma unroll
    for( int o = 16; o > 0; o >>= 1 ) v = fmax( v, __shfl_xor_sync( 0xffffffffu, v, o ) );
    return v;
}

// op1: 0 = sum, 1 = max for the second value. Slots < 0 are skipped. Inputs are the
// per-warp totals (already reduced across the warp, valid in every lane). The block takes
// part as block `bid` of `nblocks` (blockIdx.x of gridDim.x unless a batched launch runs
// several simulations' blocks side by side in y).
__device__ __forceinline__ void reduce2_publish_warp( double v0, double v1, int op1, BoraReduceDev red, int slot0, int slot1,
                                                      unsigned bid, unsigned nblocks )
{
    __shared__ double w0[32], w1[32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = ( blockDim.x + 31 ) >> 5;
    if( lane == 0 ) { w0[wid] = v0; w1[wid] = v1; }
    __syncthreads();
    if( threadIdx.x == 0 )
    {
        double a = 0.0, b = 0.0;
        for( int q = 0; q < nw; ++q ) { a += w0[q]; b = op1 ? fmax( b, w1[q] ) : b + w1[q]; }
        red.partials[2 * (size_t)bid] = a;
        red.partials[2 * (size_t)bid + 1] = b;
        __threadfence();
        const int key = slot0 >= 0 ? slot0 : slot1;
        const unsigned prev = atomicAdd( &red.done[key % BORA_RING], 1u );
        last = ( prev == nblocks - 1 );
    }
    __syncthreads();
    if( !last ) return;
    __threadfence();
    // All threads of the last block: thread-strided partial sums in a fixed order
    // (independent loads, unrolled so that many are in flight), then a fixed-shape tree.
    double a = 0.0, b = 0.0;
    const unsigned nb = nblocks, stride = blockDim.x;
#pragma unroll 4
    for( unsigned q = threadIdx.x; q < nb; q += stride )
    {
        const double2 pq = __ldcg( reinterpret_cast<const double2*>( red.partials ) + q );
        a += pq.x;
        b = op1 ? fmax( b, pq.y ) : b + pq.y;
    }
    a = warp_sum( a );
    b = op1 ? warp_max( b ) : warp_sum( b );
    if( lane == 0 ) { w0[wid] = a; w1[wid] = b; }
    __syncthreads();
    if( threadIdx.x == 0 )
    {
        double ta = 0.0, tb = 0.0;
        for( int q = 0; q < nw; ++q ) { ta += w0[q]; tb = op1 ? fmax( tb, w1[q] ) : tb + w1[q]; }
        if( slot0 >= 0 ) red.ring[slot0] = ta;
        if( slot1 >= 0 ) red.ring[slot1] = tb;
        if( red.mirror )  // host-visible once the kernel has completed
        {
            if( slot0 >= 0 ) red.mirror[slot0] = ta;
            if( slot1 >= 0 ) red.mirror[slot1] = tb;
        }
        const int key = slot0 >= 0 ? slot0 : slot1;
        red.done[key % BORA_RING] = 0;
        __threadfence();
    }
}

__device__ __forceinline__ void reduce2_publish_warp( double v0, double v1, int op1, BoraReduceDev red, int slot0, int slot1 )
{
    reduce2_publish_warp( v0, v1, op1, red, slot0, slot1, blockIdx.x, gridDim.x );
}

// Per-thread double-float sums (op1 = 0) or a float max in v1 (op1 = 1).
__device__ __forceinline__ void reduce2_publish_df( DF v0, DF v1, BoraReduceDev red, int slot0, int slot1,
                                                    unsigned bid, unsigned nblocks )
{
    const double a = df_warp_sum( v0 );
    const double b = df_warp_sum( v1 );
    reduce2_publish_warp( a, b, 0, red, slot0, slot1, bid, nblocks );
}
__device__ __forceinline__ void reduce2_publish_df( DF v0, DF v1, BoraReduceDev red, int slot0, int slot1 )
{
    reduce2_publish_df( v0, v1, red, slot0, slot1, blockIdx.x, gridDim.x );
}
__device__ __forceinline__ void reduce2_publish_dfmax( DF v0, float vmax, BoraReduceDev red, int slot0, int slot1,
                                                       unsigned bid, unsigned nblocks )
{
    const double a = df_warp_sum( v0 );
    const double b = (double)warp_maxf( vmax );
    reduce2_publish_warp( a, b, 1, red, slot0, slot1, bid, nblocks );
}
__device__ __forceinline__ void reduce2_publish_dfmax( DF v0, float vmax, BoraReduceDev red, int slot0, int slot1 )
{
    reduce2_publish_dfmax( v0, vmax, red, slot0, slot1, blockIdx.x, gridDim.x );
}


}  // namespace bora_reduce

using namespace bora_reduce;
