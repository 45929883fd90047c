// The tiled levels of the multigrid V-cycle (levels 0, 1, 2: 8^3, 4^3 and 2^3 cells per
// tile) as stencil passes over each level's own cells.
//
// A level is pre-smoothed and restricted in two passes and prolonged and post-smoothed in
// two more; every pass is a 7-point stencil that reads its neighbours' values of one field:
//   down 1  z2 = S_B(S_A(0)). The first sweep from zero is pointwise, z1 = w_A r' / d, so
//           the second reads its neighbours' r' and codes.                      z2 -> scratch
//   down 2  res = r' - A z2 (the neighbours' z2); z0 = FP16(z2); the coarser level's
//           r = FP16(0.5 * sum of the 8 children's res)
//   up 1    za = z0 + e(parent) (injection of the coarser correction), zb = S_B(za) (the
//           neighbours' za).                                                    zb -> scratch
//   up 2    z = S_A(zb) (the neighbours' zb); level 0 unscales into the FP32 z of the PCG and
//           sums r.z, the other levels store FP16 z1 for the finer level's up 1
// where r' = r * sc on level 0 (sc = 1 / ||r|| of the latest residual whose norm is known: it
// keeps the FP16 levels' values O(1), and the V-cycle is linear in r, so any scale serves) and r
// on the others,
// S_w(v) = v + (w / d) (r' - (d v - sum of the neighbours' v)) on fluid cells and 0 elsewhere,
// neighbour sums in the order ((x- + x+) + (y- + y+)) + (z- + z+), and the 8 children summed as
// ((x pairs) + (y pairs)) + (z pairs). Every cell is computed once per pass; the scratch is
// the FP32 cell vector that the plain form keeps its preconditioner pivots in (the mixed form
// has none), used by one pass pair at a time: level 0 stores its z2 and zb there in FP16 (half
// the bytes of the pass pair's store and reads; the residual of down 2 is then formed from the
// same FP16 values that z0 keeps), levels 1 and 2 in FP32.
//
// Level 0's down passes also apply the PCG's residual update r -= alpha q (alpha = rz / dq of the
// last direction): down 1 forms the updated residual of its cells and of the face cells it reads,
// without storing it, and sums r.r over the grid (the convergence check); down 2, which reads no
// neighbour's r, stores it. This takes the update kernel out of every iteration.
//
// Level 0 runs one warp per tile: a lane owns the x-rows (j, k) and (j, k + 4) of the tile as
// 16-byte vectors (lane = j + 8 k), its x neighbours are in its registers, the y and z
// neighbours come from other lanes by shuffles, and the lanes of the tile's faces load the face
// rows of the six neighbour tiles. Levels 1 and 2 run one thread per cell.
#include <algorithm>
#include <type_traits>

#include "bora_internal.h"
#include "reduce.cuh"

namespace {

constexpr float kOmegaA = 0.5687f;  // the Chebyshev pair of the smoothers (multigrid.cu)
constexpr float kOmegaB = 1.6902f;
// launch shapes (the autotuner picks one per size class; the results do not depend on it):
// level 0 tiles (warps) per block, levels 1 and 2 threads (cells) per block
constexpr int kPassWarpsOf[3] = { 2, 4, 8 };
constexpr int kFlatThreadsOf[4] = { 64, 128, 256, 512 };
constexpr int kReduceWarps = 4;  // level 0's up 2 sums r.z over its blocks: its shape is fixed
constexpr unsigned kAll = 0xffffffffu;

__device__ __forceinline__ int cdiag( uint16_t c ) { return ( c >> 8 ) & 15; }
__device__ __forceinline__ bool cfluid( uint16_t c ) { return ( c & BORA_CODE_FLUID ) != 0; }

// w / d for d = 0..15 (0 for d = 0): w_A in [0, 16), w_B in [16, 32)
__device__ __forceinline__ void init_weights( float* w )
{
    const int t = threadIdx.x;
    if( t < 32 )
    {
        const int d = t & 15;
        w[t] = d ? ( t < 16 ? kOmegaA : kOmegaB ) / (float)d : 0.f;
    }
}

// one damped Jacobi update of cell value v from its neighbour sum (w = w_A or w_B table)
__device__ __forceinline__ float sweep( float v, float r, uint16_t c, float sum, const float* w )
{
    return cfluid( c ) ? v + w[cdiag( c )] * ( r - ( (float)cdiag( c ) * v - sum ) ) : 0.f;
}

__device__ __forceinline__ float scale_from( const double* ring, int slot )
{
    const double rr = ring[slot];
    return rr > 0.0 ? (float)( 1.0 / sqrt( rr ) ) : 1.f;
}

// ---- level 0: one warp per tile ---------------------------------------------------------

__device__ __forceinline__ void codes8( const uint16_t* __restrict__ code, size_t g, uint16_t* c )
{
    const uint4 w = *reinterpret_cast<const uint4*>( code + g );
    const uint32_t a[4] = { w.x, w.y, w.z, w.w };
#pragma unroll
    for( int i = 0; i < 4; ++i )
    {
        c[2 * i] = (uint16_t)( a[i] & 0xffffu );
        c[2 * i + 1] = (uint16_t)( a[i] >> 16 );
    }
}

__device__ __forceinline__ void f32x8( const float* __restrict__ p, size_t g, float* v )
{
    const float4 a = *reinterpret_cast<const float4*>( p + g ), b = *reinterpret_cast<const float4*>( p + g + 4 );
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

__device__ __forceinline__ void st_f32x8( float* __restrict__ p, size_t g, const float* v )
{
    reinterpret_cast<float4*>( p + g )[0] = make_float4( v[0], v[1], v[2], v[3] );
    reinterpret_cast<float4*>( p + g )[1] = make_float4( v[4], v[5], v[6], v[7] );
}

__device__ __forceinline__ float hbits( uint32_t w, int q ) { return __half2float( __ushort_as_half( (unsigned short)( w >> ( 16 * q ) ) ) ); }

__device__ __forceinline__ void f16x8( const __half* __restrict__ p, size_t g, float* v )
{
    const uint4 w = *reinterpret_cast<const uint4*>( p + g );
    const uint32_t a[4] = { w.x, w.y, w.z, w.w };
#pragma unroll
    for( int i = 0; i < 4; ++i ) { v[2 * i] = hbits( a[i], 0 ); v[2 * i + 1] = hbits( a[i], 1 ); }
}

__device__ __forceinline__ uint32_t pack2( float a, float b )
{
    return (uint32_t)__half_as_ushort( __float2half_rn( a ) ) | ( (uint32_t)__half_as_ushort( __float2half_rn( b ) ) << 16 );
}

// the fields a pass reads at its neighbours, for 8 cells of a row or one cell of tile slot t
// (cell index c in the tile; t < 0 gives zeros)
struct FieldZ1  // down 1: the first sweep's z1 = w_A r' / d of the updated residual r - alpha q
{
    const uint16_t* code;
    const float* r0;
    const float* q;  // null: no update
    float alpha;
    float sc;
    const float* w;
    __device__ void row( int t, int c, float* v ) const
    {
        if( t < 0 ) { for( int i = 0; i < 8; ++i ) v[i] = 0.f; return; }
        const size_t g = (size_t)t * 512 + c;
        uint16_t cc[8];
        float rr[8];
        codes8( code, g, cc );
        f32x8( r0, g, rr );
        if( q )
        {
            float qq[8];
            f32x8( q, g, qq );
#pragma unroll
            for( int i = 0; i < 8; ++i ) rr[i] = fmaf( -alpha, qq[i], rr[i] );
        }
#pragma unroll
        for( int i = 0; i < 8; ++i ) v[i] = cfluid( cc[i] ) ? ( rr[i] * sc ) * w[cdiag( cc[i] )] : 0.f;
    }
    __device__ float one( int t, int c ) const
    {
        if( t < 0 ) return 0.f;
        const size_t g = (size_t)t * 512 + c;
        const uint16_t cc = code[g];
        const float r = q ? fmaf( -alpha, q[g], r0[g] ) : r0[g];
        return cfluid( cc ) ? ( r * sc ) * w[cdiag( cc )] : 0.f;
    }
};

struct FieldF32  // down 2 and up 2: a scratch value
{
    const float* v;
    __device__ void row( int t, int c, float* o ) const
    {
        if( t < 0 ) { for( int i = 0; i < 8; ++i ) o[i] = 0.f; return; }
        f32x8( v, (size_t)t * 512 + c, o );
    }
    __device__ float one( int t, int c ) const { return t < 0 ? 0.f : v[(size_t)t * 512 + c]; }
};

struct FieldF16  // down 2 and up 2 (level 0): a scratch value stored in FP16
{
    const __half* v;
    __device__ void row( int t, int c, float* o ) const
    {
        if( t < 0 ) { for( int i = 0; i < 8; ++i ) o[i] = 0.f; return; }
        f16x8( v, (size_t)t * 512 + c, o );
    }
    __device__ float one( int t, int c ) const { return t < 0 ? 0.f : __half2float( v[(size_t)t * 512 + c] ); }
};

__device__ __forceinline__ void st_f16x8( __half* __restrict__ p, size_t g, const float* v )
{
    *reinterpret_cast<uint4*>( p + g ) = make_uint4( pack2( v[0], v[1] ), pack2( v[2], v[3] ), pack2( v[4], v[5] ), pack2( v[6], v[7] ) );
}

struct FieldZa  // up 1: za = z0 + e(parent) on fluid cells
{
    const uint16_t* code;
    const __half* z0;
    const __half* ec;  // level 1's correction, 64 cells per tile
    __device__ void row( int t, int c, float* v ) const
    {
        if( t < 0 ) { for( int i = 0; i < 8; ++i ) v[i] = 0.f; return; }
        const size_t g = (size_t)t * 512 + c;
        uint16_t cc[8];
        float zz[8];
        codes8( code, g, cc );
        f16x8( z0, g, zz );
        const int jj = ( c >> 3 ) & 7, kk = c >> 6;
        const uint2 e = *reinterpret_cast<const uint2*>( ec + (size_t)t * 64 + 4 * ( ( jj >> 1 ) + 4 * ( kk >> 1 ) ) );
#pragma unroll
        for( int i = 0; i < 8; ++i )
        {
            const float ev = hbits( ( i >> 2 ) ? e.y : e.x, ( i >> 1 ) & 1 );
            v[i] = cfluid( cc[i] ) ? zz[i] + ev : 0.f;
        }
    }
    __device__ float one( int t, int c ) const
    {
        if( t < 0 ) return 0.f;
        const size_t g = (size_t)t * 512 + c;
        const uint16_t cc = code[g];
        const int x = c & 7, jj = ( c >> 3 ) & 7, kk = c >> 6;
        const float ev = __half2float( ec[(size_t)t * 64 + ( x >> 1 ) + 4 * ( ( jj >> 1 ) + 4 * ( kk >> 1 ) )] );
        return cfluid( cc ) ? __half2float( z0[g] ) + ev : 0.f;
    }
};

// The neighbour sums of a lane's rows A = (j, kq) and B = (j, kq + 4) of tile s from their own
// values vA, vB (every lane of the warp calls this for the same tile).
// nf: the face-neighbour slots -x +x -y +y -z +z.
template <class F>
__device__ __forceinline__ void row_sums( const F& f, const int* nf, int lane, const float* vA, const float* vB, float* sA,
                                          float* sB )
{
    const int j = lane & 7, kq = lane >> 3;
    const int smx = nf[0], spx = nf[1], smy = nf[2], spy = nf[3], smz = nf[4], spz = nf[5];
    // the x ends of both rows, the y face row of lanes j = 0 / 7 (both rows), the z face row
    // of row A at k = 0 (-z) and of row B at k = 7 (+z)
    const float xmA = f.one( smx, 8 * lane + 7 ), xpA = f.one( spx, 8 * lane );
    const float xmB = f.one( smx, 256 + 8 * lane + 7 ), xpB = f.one( spx, 256 + 8 * lane );
    float yhA[8], yhB[8], zh[8];
    {
        const int yt = j == 0 ? smy : ( j == 7 ? spy : -1 );
        const int yc = 8 * ( lane - j ) + ( j == 0 ? 56 : 0 );
        f.row( yt, yc, yhA );
        f.row( yt, yc + 256, yhB );
        const int zt = kq == 0 ? smz : ( kq == 3 ? spz : -1 );
        f.row( zt, 8 * j + ( kq == 0 ? 448 : 0 ), zh );
    }
#pragma unroll
    for( int i = 0; i < 8; ++i )
    {
        float ymA = __shfl_up_sync( kAll, vA[i], 1 ), ypA = __shfl_down_sync( kAll, vA[i], 1 );
        float ymB = __shfl_up_sync( kAll, vB[i], 1 ), ypB = __shfl_down_sync( kAll, vB[i], 1 );
        if( j == 0 ) { ymA = yhA[i]; ymB = yhB[i]; }
        if( j == 7 ) { ypA = yhA[i]; ypB = yhB[i]; }
        float zmA = __shfl_up_sync( kAll, vA[i], 8 );
        if( kq == 0 ) zmA = zh[i];
        // the source lane picks the row: lane + 8 wraps from kq = 3 to row B of kq = 0, lane - 8
        // from kq = 0 to row A of kq = 3
        const float zpA = __shfl_sync( kAll, kq == 0 ? vB[i] : vA[i], ( lane + 8 ) & 31 );
        const float zmB = __shfl_sync( kAll, kq == 3 ? vA[i] : vB[i], ( lane + 24 ) & 31 );
        float zpB = __shfl_down_sync( kAll, vB[i], 8 );
        if( kq == 3 ) zpB = zh[i];
        const float xmA_ = i > 0 ? vA[i > 0 ? i - 1 : 0] : xmA, xpA_ = i < 7 ? vA[i < 7 ? i + 1 : 7] : xpA;
        const float xmB_ = i > 0 ? vB[i > 0 ? i - 1 : 0] : xmB, xpB_ = i < 7 ? vB[i < 7 ? i + 1 : 7] : xpB;
        sA[i] = ( ( xmA_ + xpA_ ) + ( ymA + ypA ) ) + ( zmA + zpA );
        sB[i] = ( ( xmB_ + xpB_ ) + ( ymB + ypB ) ) + ( zmB + zpB );
    }
}

struct Pass0Args
{
    int ntiles;
    const int32_t* nbr;
    BoraLevelDev F;       // level 0
    BoraLevelDev C;       // level 1 (down 2 writes its r; up 1 reads its z1)
    float* r0;            // the PCG residual (down 2 stores its update)
    const float* q;       // the PCG's A d (the update's direction term)
    float* scratch;       // FP32 per cell
    float* zout;          // up 2: the PCG's z
    BoraReduceDev red;
    int slot_rr;          // the scale's r.r
    int slot_rz;          // up 2: r.z out
    int slot_rz_in, slot_dq_in;  // down 1, 2: alpha = rz_in / dq_in (slot_rz_in < 0: no update)
    int slot_rr_out;      // down 1: r.r of the updated residual out
};

// pass P of level 0: 0 = down 1, 1 = down 2, 2 = up 1, 3 = up 2; W tiles (warps) per block
template <int W, int P>
__device__ __forceinline__ void pass0_body( const Pass0Args& a, unsigned bid, unsigned G )
{
    __shared__ float w[32];
    __shared__ float s_sc;
    bora_pdl_trigger();
    init_weights( w );
    const int lane = threadIdx.x & 31, j = lane & 7, kq = lane >> 3;
    const int stride = (int)G * W;
    // what no kernel of the solve writes - the tile's face neighbours and the rows' codes - is
    // read a tile ahead, the first tile's before the dependency wait
    int nfn[6] = { -1, -1, -1, -1, -1, -1 };
    uint4 cwA = make_uint4( 0u, 0u, 0u, 0u ), cwB = cwA;
    auto fetch = [&]( int t ) {
        if( t >= a.ntiles ) return;
        const int32_t* __restrict__ nb = a.nbr + (size_t)t * 27;
        nfn[0] = nb[bora_dir( -1, 0, 0 )]; nfn[1] = nb[bora_dir( 1, 0, 0 )];
        nfn[2] = nb[bora_dir( 0, -1, 0 )]; nfn[3] = nb[bora_dir( 0, 1, 0 )];
        nfn[4] = nb[bora_dir( 0, 0, -1 )]; nfn[5] = nb[bora_dir( 0, 0, 1 )];
        cwA = *reinterpret_cast<const uint4*>( a.F.code + (size_t)t * 512 + 8 * lane );
        cwB = *reinterpret_cast<const uint4*>( a.F.code + (size_t)t * 512 + 256 + 8 * lane );
    };
    int s = (int)bid * W + ( threadIdx.x >> 5 );
    fetch( s );
    __shared__ float s_alpha;
    bora_pdl_wait();  // the previous kernel's results are complete from here
    if( threadIdx.x == 0 )
    {
        s_sc = scale_from( a.red.ring, a.slot_rr );
        s_alpha = a.slot_rz_in < 0 ? 0.f : (float)( a.red.ring[a.slot_rz_in] / a.red.ring[a.slot_dq_in] );
    }
    __syncthreads();
    const float sc = s_sc, alpha = s_alpha;
    const bool upd = ( P == 0 || P == 1 ) && a.slot_rz_in >= 0;  // down 1, 2 apply r -= alpha q
    DF acc{ 0.f, 0.f };  // down 1: r.r of the updated residual; up 2: r.z
    for( ; s < a.ntiles; s += stride )
    {
        int nf[6];
#pragma unroll
        for( int q = 0; q < 6; ++q ) nf[q] = nfn[q];
        const size_t gA = (size_t)s * 512 + 8 * lane, gB = gA + 256;
        uint16_t cA[8], cB[8];
        {
            const uint32_t wa[4] = { cwA.x, cwA.y, cwA.z, cwA.w }, wb[4] = { cwB.x, cwB.y, cwB.z, cwB.w };
#pragma unroll
            for( int i = 0; i < 4; ++i )
            {
                cA[2 * i] = (uint16_t)( wa[i] & 0xffffu ); cA[2 * i + 1] = (uint16_t)( wa[i] >> 16 );
                cB[2 * i] = (uint16_t)( wb[i] & 0xffffu ); cB[2 * i + 1] = (uint16_t)( wb[i] >> 16 );
            }
        }
        fetch( s + stride );
        float rA[8], rB[8];  // r' on fluid cells
        f32x8( a.r0, gA, rA );
        f32x8( a.r0, gB, rB );
        if( upd )
        {
            float qA[8], qB[8];
            f32x8( a.q, gA, qA );
            f32x8( a.q, gB, qB );
#pragma unroll
            for( int i = 0; i < 8; ++i )
            {
                rA[i] = fmaf( -alpha, qA[i], rA[i] );
                rB[i] = fmaf( -alpha, qB[i], rB[i] );
            }
            if constexpr( P == 1 )
            {
                st_f32x8( a.r0, gA, rA );
                st_f32x8( a.r0, gB, rB );
            }
        }
        if constexpr( P == 0 )
        {
            float t = 0.f;
#pragma unroll
            for( int i = 0; i < 8; ++i ) { t = fmaf( rA[i], rA[i], t ); t = fmaf( rB[i], rB[i], t ); }
            acc = df_add_f( acc, t );
        }
#pragma unroll
        for( int i = 0; i < 8; ++i )
        {
            rA[i] = cfluid( cA[i] ) ? rA[i] * sc : 0.f;
            rB[i] = cfluid( cB[i] ) ? rB[i] * sc : 0.f;
        }
        float vA[8], vB[8], sA[8], sB[8];
        if constexpr( P == 0 )
        {
#pragma unroll
            for( int i = 0; i < 8; ++i )
            {
                vA[i] = cfluid( cA[i] ) ? rA[i] * w[cdiag( cA[i] )] : 0.f;
                vB[i] = cfluid( cB[i] ) ? rB[i] * w[cdiag( cB[i] )] : 0.f;
            }
            row_sums( FieldZ1{ a.F.code, a.r0, upd ? a.q : nullptr, alpha, sc, w }, nf, lane, vA, vB, sA, sB );
#pragma unroll
            for( int i = 0; i < 8; ++i )
            {
                vA[i] = sweep( vA[i], rA[i], cA[i], sA[i], w + 16 );
                vB[i] = sweep( vB[i], rB[i], cB[i], sB[i], w + 16 );
            }
            st_f16x8( reinterpret_cast<__half*>( a.scratch ), gA, vA );
            st_f16x8( reinterpret_cast<__half*>( a.scratch ), gB, vB );
        }
        else if constexpr( P == 1 )
        {
            f16x8( reinterpret_cast<const __half*>( a.scratch ), gA, vA );
            f16x8( reinterpret_cast<const __half*>( a.scratch ), gB, vB );
            row_sums( FieldF16{ reinterpret_cast<const __half*>( a.scratch ) }, nf, lane, vA, vB, sA, sB );
            float qA[8], qB[8];  // residuals
#pragma unroll
            for( int i = 0; i < 8; ++i )
            {
                qA[i] = cfluid( cA[i] ) ? rA[i] - ( (float)cdiag( cA[i] ) * vA[i] - sA[i] ) : 0.f;
                qB[i] = cfluid( cB[i] ) ? rB[i] - ( (float)cdiag( cB[i] ) * vB[i] - sB[i] ) : 0.f;
            }
            *reinterpret_cast<uint4*>( a.F.z0 + gA ) =
                make_uint4( pack2( vA[0], vA[1] ), pack2( vA[2], vA[3] ), pack2( vA[4], vA[5] ), pack2( vA[6], vA[7] ) );
            *reinterpret_cast<uint4*>( a.F.z0 + gB ) =
                make_uint4( pack2( vB[0], vB[1] ), pack2( vB[2], vB[3] ), pack2( vB[4], vB[5] ), pack2( vB[6], vB[7] ) );
            // restriction: x pairs in the row, y pairs from lane j + 1, z pairs from lane + 8
            float pA[4], pB[4];
#pragma unroll
            for( int q = 0; q < 4; ++q )
            {
                pA[q] = qA[2 * q] + qA[2 * q + 1];
                pB[q] = qB[2 * q] + qB[2 * q + 1];
                pA[q] = pA[q] + __shfl_down_sync( kAll, pA[q], 1 );
                pB[q] = pB[q] + __shfl_down_sync( kAll, pB[q], 1 );
                pA[q] = pA[q] + __shfl_down_sync( kAll, pA[q], 8 );
                pB[q] = pB[q] + __shfl_down_sync( kAll, pB[q], 8 );
            }
            if( !( j & 1 ) && !( kq & 1 ) )
            {
                __half* cr = a.C.r + (size_t)s * 64 + 4 * ( j >> 1 );
                *reinterpret_cast<uint2*>( cr + 16 * ( kq >> 1 ) ) =
                    make_uint2( pack2( 0.5f * pA[0], 0.5f * pA[1] ), pack2( 0.5f * pA[2], 0.5f * pA[3] ) );
                *reinterpret_cast<uint2*>( cr + 16 * ( 2 + ( kq >> 1 ) ) ) =
                    make_uint2( pack2( 0.5f * pB[0], 0.5f * pB[1] ), pack2( 0.5f * pB[2], 0.5f * pB[3] ) );
            }
        }
        else if constexpr( P == 2 )
        {
            const FieldZa f{ a.F.code, a.F.z0, a.C.z1 };
            f.row( s, 8 * lane, vA );
            f.row( s, 256 + 8 * lane, vB );
            row_sums( f, nf, lane, vA, vB, sA, sB );
#pragma unroll
            for( int i = 0; i < 8; ++i )
            {
                vA[i] = sweep( vA[i], rA[i], cA[i], sA[i], w + 16 );
                vB[i] = sweep( vB[i], rB[i], cB[i], sB[i], w + 16 );
            }
            st_f16x8( reinterpret_cast<__half*>( a.scratch ), gA, vA );
            st_f16x8( reinterpret_cast<__half*>( a.scratch ), gB, vB );
        }
        else
        {
            f16x8( reinterpret_cast<const __half*>( a.scratch ), gA, vA );
            f16x8( reinterpret_cast<const __half*>( a.scratch ), gB, vB );
            row_sums( FieldF16{ reinterpret_cast<const __half*>( a.scratch ) }, nf, lane, vA, vB, sA, sB );
            float rawA[8], rawB[8];
            f32x8( a.r0, gA, rawA );
            f32x8( a.r0, gB, rawB );
            float trz = 0.f;
#pragma unroll
            for( int i = 0; i < 8; ++i )
            {
                // undo the FP16 scaling of the residual
                vA[i] = sweep( vA[i], rA[i], cA[i], sA[i], w ) / sc;
                vB[i] = sweep( vB[i], rB[i], cB[i], sB[i], w ) / sc;
                if( cfluid( cA[i] ) ) trz = fmaf( rawA[i], vA[i], trz );
                if( cfluid( cB[i] ) ) trz = fmaf( rawB[i], vB[i], trz );
            }
            st_f32x8( a.zout, gA, vA );
            st_f32x8( a.zout, gB, vB );
            acc = df_add_f( acc, trz );
        }
    }
    if constexpr( P == 3 ) reduce2_publish_warp( df_warp_sum( acc ), 0.0, 0, a.red, a.slot_rz, -1, bid, G );
    if constexpr( P == 0 ) reduce2_publish_warp( df_warp_sum( acc ), 0.0, 0, a.red, a.slot_rr_out, -1, bid, G );
}

template <int W, int P>
__global__ void __launch_bounds__( 32 * W, 16 / W ) k_mg_pass0( const __grid_constant__ Pass0Args a )
{
    pass0_body<W, P>( a, blockIdx.x, gridDim.x );
}

template <int W, int P>
__global__ void __launch_bounds__( 32 * W, 16 / W ) k_mg_pass0_batch( const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    const BoraMemberSlots& q = L.sl[k];
    Pass0Args a;
    a.ntiles = m.ntiles;
    a.nbr = m.nbr;
    a.F = m.L[0];
    a.C = m.L[1];
    a.r0 = m.sv.r;
    a.q = m.sv.q;
    a.scratch = m.sv.minv;
    a.zout = m.sv.z;
    a.red = m.red;
    a.slot_rr = q.rr;
    a.slot_rz = q.rz;
    a.slot_rz_in = q.rz_in;
    a.slot_dq_in = q.dq_in;
    a.slot_rr_out = q.rr_out;
    pass0_body<W, P>( a, bid, (unsigned)m.grid[P == 0 || P == 3 ? kGridPass0R : kGridPass0] );
}

// ---- levels 1 and 2: one thread per cell --------------------------------------------------

struct PassFArgs
{
    int ntiles;
    const int32_t* nbr;
    BoraLevelDev F;     // this level (E = 4 or 2)
    BoraLevelDev C;     // the coarser one (down 2 writes its r)
    const __half* ec;   // up 1: the coarser level's correction
    float* scratch;
};

// pass P (0 = down 1, 1 = down 2, 2 = up 1, 3 = up 2) of a level with E = 4 or 2, one cell
// per thread (the grid covers every cell once; a block holds whole tiles). What no kernel of
// the solve writes - the cell's code, its neighbours' indices and codes - is read before the
// dependency wait, so that it overlaps the previous kernel.
template <int E, int P, int T>
__device__ __forceinline__ void passf_body( const PassFArgs& a, unsigned bid )
{
    constexpr int E3 = E * E * E, H = E / 2, H3 = H * H * H;
    constexpr bool kCodes = P == 0 || P == 2;  // the neighbours' values need their codes
    __shared__ float w[32];
    __shared__ float res[T];
    bora_pdl_trigger();
    init_weights( w );
    const size_t ncells = (size_t)a.ntiles * E3;
    const size_t base = (size_t)bid * T, g = base + threadIdx.x;
    const bool live = g < ncells;
    const BoraLevelDev& F = a.F;
    int s = 0, x = 0, y = 0, z = 0;
    uint16_t cc = 0;
    int64_t gn[6];     // neighbour cells -x +x -y +y -z +z (-1: none)
    uint16_t cn[6];
    int pn[6];         // up 1: the neighbours' parents on the coarser level
    if( live )
    {
        s = (int)( g / E3 );
        const int l = (int)( g % E3 );
        x = l % E; y = ( l / E ) % E; z = l / ( E * E );
        cc = F.code[g];
        const int32_t* __restrict__ nb = a.nbr + (size_t)s * 27;
#pragma unroll
        for( int q = 0; q < 6; ++q )
        {
            const int dx = q == 0 ? -1 : ( q == 1 ? 1 : 0 ), dy = q == 2 ? -1 : ( q == 3 ? 1 : 0 ),
                      dz = q == 4 ? -1 : ( q == 5 ? 1 : 0 );
            int xx = x + dx, yy = y + dy, zz = z + dz, t = s;
            if( xx < 0 || xx >= E || yy < 0 || yy >= E || zz < 0 || zz >= E )
            {
                t = nb[bora_dir( dx, dy, dz )];
                xx &= E - 1; yy &= E - 1; zz &= E - 1;
            }
            gn[q] = t < 0 ? -1 : (int64_t)t * E3 + xx + E * ( yy + E * zz );
            pn[q] = t < 0 ? 0 : t * H3 + ( xx >> 1 ) + H * ( ( yy >> 1 ) + H * ( zz >> 1 ) );
            cn[q] = kCodes && t >= 0 ? F.code[gn[q]] : 0;
        }
    }
    bora_pdl_wait();  // the previous kernel's results are complete from here
    __syncthreads();
    // the field value the pass reads at cell gi (code ci, parent pi)
    auto value = [&]( int64_t gi, uint16_t ci, int pi ) -> float {
        if( gi < 0 ) return 0.f;
        if constexpr( P == 0 ) return cfluid( ci ) ? __half2float( F.r[gi] ) * w[cdiag( ci )] : 0.f;
        else if constexpr( P == 2 ) return cfluid( ci ) ? __half2float( F.z0[gi] ) + __half2float( a.ec[pi] ) : 0.f;
        else return a.scratch[gi];
    };
    float out = 0.f;
    if( live )
    {
        const float rp = cfluid( cc ) ? __half2float( F.r[g] ) : 0.f;
        const int pg = s * H3 + ( x >> 1 ) + H * ( ( y >> 1 ) + H * ( z >> 1 ) );
        const float v = value( (int64_t)g, cc, pg );
        const float sum = ( ( value( gn[0], cn[0], pn[0] ) + value( gn[1], cn[1], pn[1] ) ) +
                            ( value( gn[2], cn[2], pn[2] ) + value( gn[3], cn[3], pn[3] ) ) ) +
                          ( value( gn[4], cn[4], pn[4] ) + value( gn[5], cn[5], pn[5] ) );
        if constexpr( P == 0 ) out = sweep( v, rp, cc, sum, w + 16 );
        else if constexpr( P == 1 ) out = cfluid( cc ) ? rp - ( (float)cdiag( cc ) * v - sum ) : 0.f;
        else if constexpr( P == 2 ) out = sweep( v, rp, cc, sum, w + 16 );
        else out = sweep( v, rp, cc, sum, w );
        if constexpr( P == 0 || P == 2 ) a.scratch[g] = out;
        else if constexpr( P == 1 ) F.z0[g] = __float2half_rn( v );
        else F.z1[g] = __float2half_rn( out );
    }
    if constexpr( P == 1 )
    {
        // restriction of the block's tiles
        res[threadIdx.x] = out;
        __syncthreads();
        constexpr int kParents = T / 8;
        if( threadIdx.x < kParents )
        {
            const int p = threadIdx.x, tl = p / H3, pl = p % H3;
            const size_t tile = base / E3 + tl;
            if( tile < (size_t)a.ntiles )
            {
                const int pa = pl % H, pb = ( pl / H ) % H, pc = pl / ( H * H );
                const int l = tl * E3 + 2 * pa + E * ( 2 * pb + E * 2 * pc );
                const float sum = ( ( res[l] + res[l + 1] ) + ( res[l + E] + res[l + E + 1] ) ) +
                                  ( ( res[l + E * E] + res[l + E * E + 1] ) + ( res[l + E * E + E] + res[l + E * E + E + 1] ) );
                a.C.r[tile * H3 + pl] = __float2half_rn( 0.5f * sum );
            }
        }
    }
}

template <int E, int P, int T>
__global__ void __launch_bounds__( T ) k_mg_passf( const __grid_constant__ PassFArgs a )
{
    passf_body<E, P, T>( a, blockIdx.x );
}

template <int E, int P, int T>
__global__ void __launch_bounds__( T ) k_mg_passf_batch( const __grid_constant__ BoraBatchLaunch L )
{
    constexpr int l = E == 4 ? 1 : 2;
    unsigned bid;
    const int k = bora_batch_member( L, blockIdx.x, &bid );
    const BoraMemberSolve& m = L.ms[k];
    PassFArgs a;
    a.ntiles = m.ntiles;
    a.nbr = m.nbr;
    a.F = m.L[l];
    a.C = m.L[l + 1];
    a.ec = l == 1 ? m.L[2].z1 : m.z3;
    a.scratch = m.sv.minv;
    passf_body<E, P, T>( a, bid );
}

int num_sms_pass()
{
    static BoraPerDevice sms;
    return sms.get( [] {
        int dev = 0, n = 0;
        cudaGetDevice( &dev );
        cudaDeviceGetAttribute( &n, cudaDevAttrMultiProcessorCount, dev );
        return n > 0 ? n : 152;
    } );
}

template <int E, int P>
void launch_passf( const PassFArgs& a, int v, cudaStream_t st )
{
    const int g = bora_mg_pass_grid( E, a.ntiles, v );
    if( g <= 0 ) return;
    switch( v )
    {
    case 0: bora_launch_pdl( k_mg_passf<E, P, 64>, dim3( g ), dim3( 64 ), 0, st, a ); break;
    case 1: bora_launch_pdl( k_mg_passf<E, P, 128>, dim3( g ), dim3( 128 ), 0, st, a ); break;
    case 2: bora_launch_pdl( k_mg_passf<E, P, 256>, dim3( g ), dim3( 256 ), 0, st, a ); break;
    default: bora_launch_pdl( k_mg_passf<E, P, 512>, dim3( g ), dim3( 512 ), 0, st, a ); break;
    }
}

template <int P>
void launch_pass0( const Pass0Args& a, int v, cudaStream_t st )
{
    const int g = bora_mg_pass_grid( 8, a.ntiles, v );
    if( g <= 0 ) return;
    switch( v )
    {
    case 0: bora_launch_pdl( k_mg_pass0<2, P>, dim3( g ), dim3( 64 ), 0, st, a ); break;
    case 1: bora_launch_pdl( k_mg_pass0<4, P>, dim3( g ), dim3( 128 ), 0, st, a ); break;
    default: bora_launch_pdl( k_mg_pass0<8, P>, dim3( g ), dim3( 256 ), 0, st, a ); break;
    }
}

}  // namespace

// Grid of the passes of a level with E cells per tile edge in launch shape v: level 0 as many
// blocks as make equal rounds of warps over the tiles with up to 16 warps per SM (the up 2 pass,
// shape kReduceWarps, reduces over them: at most kBoraMaxReduceBlocks); levels 1 and 2 one
// thread per cell.
int bora_mg_pass_grid( int E, int ntiles, int v )
{
    if( ntiles <= 0 ) return 0;
    const int sms = num_sms_pass();
    if( E == 8 )
    {
        const int W = v < 0 ? kReduceWarps : kPassWarpsOf[std::min( v, 2 )];
        const int cap = std::max( 1, std::min( 32 / W * sms, kBoraMaxReduceBlocks ) ) * W;
        const int rounds = ( ntiles + cap - 1 ) / cap;
        return std::max( 1, ( ntiles + W * rounds - 1 ) / ( W * rounds ) );
    }
    const int T = kFlatThreadsOf[std::min( std::max( v, 0 ), 3 )];
    const size_t n = (size_t)ntiles * E * E * E;
    return (int)( ( n + T - 1 ) / T );
}

void bora_mg_pass_down( const BoraLevelDev* levels, int l, const BoraTilesDev& t, int ntiles, float* r0, const float* q,
                        float* scratch, const BoraReduceDev& red, int slot_rr, int slot_rz_in, int slot_dq_in,
                        int slot_rr_out, cudaStream_t st )
{
    const int group = l == 0 ? kBoraTuneL0 : ( l == 1 ? kBoraTuneL1 : kBoraTuneL2 );
    const BoraTunePick pick = bora_tune_pick( group, ntiles );
    BoraTuneTimer timer( pick, group, ntiles, st );  // times the level's two down passes
    const int v = pick.variant;
    if( levels[l].E == 8 )
    {
        Pass0Args a{};
        a.ntiles = ntiles; a.nbr = t.nbr; a.F = levels[0]; a.C = levels[1]; a.r0 = r0; a.q = q; a.scratch = scratch;
        a.red = red; a.slot_rr = slot_rr; a.slot_rz = -1;
        a.slot_rz_in = slot_rz_in; a.slot_dq_in = slot_dq_in; a.slot_rr_out = slot_rr_out;
        // down 1 sums r.r over its blocks: the fixed shape
        const int g = bora_mg_pass_grid( 8, ntiles, -1 );
        if( g > 0 ) bora_launch_pdl( k_mg_pass0<kReduceWarps, 0>, dim3( g ), dim3( 32 * kReduceWarps ), 0, st, a );
        launch_pass0<1>( a, v, st );
        return;
    }
    PassFArgs a{};
    a.ntiles = ntiles; a.nbr = t.nbr; a.F = levels[l]; a.C = levels[l + 1]; a.scratch = scratch;
    if( levels[l].E == 4 ) { launch_passf<4, 0>( a, v, st ); launch_passf<4, 1>( a, v, st ); }
    else { launch_passf<2, 0>( a, v, st ); launch_passf<2, 1>( a, v, st ); }
}

void bora_mg_pass_up( const BoraLevelDev* levels, int l, const __half* ec, const BoraTilesDev& t, int ntiles,
                      const float* r0, float* scratch, const BoraReduceDev& red, int slot_rr, float* z, int slot_rz,
                      cudaStream_t st )
{
    const int group = l == 0 ? kBoraTuneL0 : ( l == 1 ? kBoraTuneL1 : kBoraTuneL2 );
    const int v = bora_tune_pick( group, ntiles ).variant;
    if( levels[l].E == 8 )
    {
        Pass0Args a{};
        a.ntiles = ntiles; a.nbr = t.nbr; a.F = levels[0]; a.C = levels[1]; a.C.z1 = const_cast<__half*>( ec );
        a.r0 = const_cast<float*>( r0 ); a.scratch = scratch; a.zout = z; a.red = red; a.slot_rr = slot_rr; a.slot_rz = slot_rz;
        a.slot_rz_in = -1; a.slot_dq_in = -1; a.slot_rr_out = -1;
        launch_pass0<2>( a, v, st );
        // r.z: the fixed shape
        const int g = bora_mg_pass_grid( 8, ntiles, -1 );
        if( g > 0 ) bora_launch_pdl( k_mg_pass0<kReduceWarps, 3>, dim3( g ), dim3( 32 * kReduceWarps ), 0, st, a );
        return;
    }
    PassFArgs a{};
    a.ntiles = ntiles; a.nbr = t.nbr; a.F = levels[l]; a.C = levels[l + 1]; a.ec = ec; a.scratch = scratch;
    if( levels[l].E == 4 ) { launch_passf<4, 2>( a, v, st ); launch_passf<4, 3>( a, v, st ); }
    else { launch_passf<2, 2>( a, v, st ); launch_passf<2, 3>( a, v, st ); }
}

void bora_launch_mg_pass_batch( int l, int pass, int v, const BoraBatchLaunch& L, int blocks, cudaStream_t st )
{
    if( blocks <= 0 ) return;
    const dim3 grid( blocks );
    if( l == 0 )
    {
        // down 1 and up 2 reduce over their blocks: the fixed shape
        if( pass == 0 || pass == 3 )
        {
            if( pass == 0 ) bora_launch_pdl( k_mg_pass0_batch<kReduceWarps, 0>, grid, dim3( 32 * kReduceWarps ), 0, st, L );
            else bora_launch_pdl( k_mg_pass0_batch<kReduceWarps, 3>, grid, dim3( 32 * kReduceWarps ), 0, st, L );
            return;
        }
        const int W = kPassWarpsOf[std::min( std::max( v, 0 ), 2 )];
        const dim3 blk( 32 * W );
        auto go = [&]( auto k0, auto k1, auto k2 ) {
            if( pass == 0 ) bora_launch_pdl( k0, grid, blk, 0, st, L );
            else if( pass == 1 ) bora_launch_pdl( k1, grid, blk, 0, st, L );
            else bora_launch_pdl( k2, grid, blk, 0, st, L );
        };
        if( W == 2 ) go( k_mg_pass0_batch<2, 0>, k_mg_pass0_batch<2, 1>, k_mg_pass0_batch<2, 2> );
        else if( W == 4 ) go( k_mg_pass0_batch<4, 0>, k_mg_pass0_batch<4, 1>, k_mg_pass0_batch<4, 2> );
        else go( k_mg_pass0_batch<8, 0>, k_mg_pass0_batch<8, 1>, k_mg_pass0_batch<8, 2> );
        return;
    }
    const int T = kFlatThreadsOf[std::min( std::max( v, 0 ), 3 )];
    auto flat = [&]( auto tag ) {
        constexpr int E = decltype( tag )::value;
        auto go = [&]( auto k0, auto k1, auto k2, auto k3 ) {
            const dim3 blk( T );
            if( pass == 0 ) bora_launch_pdl( k0, grid, blk, 0, st, L );
            else if( pass == 1 ) bora_launch_pdl( k1, grid, blk, 0, st, L );
            else if( pass == 2 ) bora_launch_pdl( k2, grid, blk, 0, st, L );
            else bora_launch_pdl( k3, grid, blk, 0, st, L );
        };
        if( T == 64 ) go( k_mg_passf_batch<E, 0, 64>, k_mg_passf_batch<E, 1, 64>, k_mg_passf_batch<E, 2, 64>, k_mg_passf_batch<E, 3, 64> );
        else if( T == 128 ) go( k_mg_passf_batch<E, 0, 128>, k_mg_passf_batch<E, 1, 128>, k_mg_passf_batch<E, 2, 128>, k_mg_passf_batch<E, 3, 128> );
        else if( T == 256 ) go( k_mg_passf_batch<E, 0, 256>, k_mg_passf_batch<E, 1, 256>, k_mg_passf_batch<E, 2, 256>, k_mg_passf_batch<E, 3, 256> );
        else go( k_mg_passf_batch<E, 0, 512>, k_mg_passf_batch<E, 1, 512>, k_mg_passf_batch<E, 2, 512>, k_mg_passf_batch<E, 3, 512> );
    };
    if( l == 1 ) flat( std::integral_constant<int, 4>{} );
    else flat( std::integral_constant<int, 2>{} );
}
