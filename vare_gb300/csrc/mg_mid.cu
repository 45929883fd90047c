// The coarse tail of the multigrid V-cycle (level 3, one cell per 8^3 tile, down to the
// coarsest level and back) in one thread-block cluster whose CTAs keep every value in
// distributed shared memory.
//
// Levels 0-2 are large and run as grid-wide fused tile kernels (multigrid.cu). Below them
// the hierarchy is tiny (level 3 has one cell per active tile, then dense grids halved per
// level down to <= 512 cells). Run from global memory every operation of these levels is a
// chain of dependent global loads (tile tables, codes, neighbours' values) followed by a
// cluster barrier: 3-7 us per operation, 43 us per V-cycle at 256^3 for 12.5 K cells. Here
// the cluster's CTAs split every level by ownership (contiguous slot ranges of level 3,
// contiguous index ranges of the dense levels, the coarsest level in CTA 0). Everything
// that is static during a solve - stencil codes and, per owned cell, packed references
// (owning CTA, local index) of its six face neighbours, its parent and its eight children -
// is laid out once per step by k_mg_mid_image as one block per CTA in global memory, in the
// CTA's shared-memory layout, and each V-cycle copies its block in with asynchronous
// 16-byte copies before waiting for the previous kernel. The operations then run out of
// shared memory: a CTA reads other cells' values from the owning CTA's shared memory
// through the cluster window and writes only its own.
//
// The arithmetic is the V-cycle of multigrid.cu: per level two Jacobi sweeps before
// (kOmegaA from zero, then kOmegaB) and after (kOmegaB, then kOmegaA), the residual
// restricted as 0.5 * sum of the 8 children, injection as prolongation, and damped Jacobi
// sweeps from zero on the coarsest level; values stay FP32 inside the kernel (the grid-
// wide kernels store FP16 between launches). Operations of a level, each followed by a
// cluster barrier:
//   down:  B = z after the second pre-smoothing sweep (A holds the first, pointwise sweep)
//          A = residual r - S B
//          r, A of the coarser level = 0.5 * sum of the children's A, its pointwise sweep
//   up:    A = B + Z(parent)      (Z: the coarser level's final correction)
//          B = A + wB (r - S A)
//          A = B + wA (r - S B)   (the level's final correction)
// Non-fluid cells hold 0 in A and B and are never summed (the stencil code's neighbour
// bits select the fluid neighbours).
#include <algorithm>
#include <cooperative_groups.h>
#include <cstring>

#include <cuda_fp16.h>

#include "bora_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr float kOmega = 0.9f;      // coarsest level: damped Jacobi
constexpr float kOmegaA = 0.5687f;  // Chebyshev pair of the smoothers (multigrid.cu)
constexpr float kOmegaB = 1.6902f;

constexpr int kMidThreads = 512;
constexpr int kMidMaxLevels = 8;
constexpr int kMidCtasMax = 16;  // non-portable cluster size where the device allows it
constexpr size_t kMidSmemMax = 200 * 1024;

// A packed reference to a cell: owning CTA in bits 24-31, local index in bits 0-23; -1 none.
__device__ inline int32_t pack_ref( int owner, int local ) { return ( owner << 24 ) | local; }

struct MidLevel
{
    int tiled;       // 1: one cell per active tile (level 3); 0: dense
    int n;           // cells
    int chunk;       // cells per CTA (the coarsest level: all, in CTA 0)
    int dx, dy, dz;  // dense extent
    const uint16_t* code;                          // global stencil codes (static during a solve)
    int o_code, o_nb, o_par, o_ch;                 // static block: byte offsets (-1: none)
    int o_r, o_a, o_b;                             // values: byte offsets after the static block
};

struct MidDesc
{
    MidLevel L[kMidMaxLevels];
    int n;  // levels; L[0] is level 3 of the hierarchy, then dense; the last is the coarsest
    const int32_t* nbr;
    const int32_t* tile_of;
    const int32_t* slot_of;
    int tx, ty, tz;
    const __half* r_in;  // level-3 residual (written by the level-2 down kernel)
    __half* z_out;       // level-3 correction (read by the level-2 up kernel)
    int sweeps;
    int ctas;
    int static_bytes;    // bytes of a CTA's static block (a multiple of 16)
    char* image;         // ctas static blocks, built by k_mg_mid_image
    uint32_t* err;       // inconsistent stencil codes are recorded here
};

extern __shared__ __align__( 16 ) char g_mid_smem[];

__device__ inline int code_diag( uint16_t c ) { return ( c >> 8 ) & 15; }

// face directions in the 27-entry tile neighbour table: -x +x -y +y -z +z
__device__ __constant__ int kFaceDir[6] = { 12, 14, 10, 16, 4, 22 };

struct Mid
{
    const MidDesc& d;
    cg::cluster_group cl;
    unsigned me;

    template <class T> __device__ T* arr( int off ) const { return reinterpret_cast<T*>( g_mid_smem + off ); }
    __device__ int owned( const MidLevel& L ) const
    {
        const int lo = (int)me * L.chunk;
        return L.n > lo ? min( L.chunk, L.n - lo ) : 0;
    }
    __device__ int32_t ref( const MidLevel& L, int c ) const  // packed reference of cell c of L
    {
        if( c < 0 ) return -1;
        const int o = c / L.chunk;
        return pack_ref( o, c - o * L.chunk );
    }
    // the value at a packed reference in array `off`: a shared-memory load when this CTA owns
    // the cell, else a load from the owning CTA's shared memory through the cluster window
    __device__ float ld( int off, int32_t rf ) const
    {
        const unsigned o = (unsigned)rf >> 24;
        const int i = rf & 0xFFFFFF;
        if( o == me ) return arr<float>( off )[i];
        const uint32_t sa = (uint32_t)__cvta_generic_to_shared( arr<float>( off ) + i );
        uint32_t ra;
        float v;
        asm volatile( "mapa.shared::cluster.u32 %0, %1, %2;" : "=r"( ra ) : "r"( sa ), "r"( o ) );
        asm volatile( "ld.shared::cluster.f32 %0, [%1];" : "=f"( v ) : "r"( ra ) : "memory" );
        return v;
    }
    __device__ void barrier() const { cl.sync(); }

    // static data of level t for the owned cells (codes, neighbours, parent, children),
    // written into the block at `blk` (the CTA's slice of the image)
    __device__ void stage( int t, char* blk ) const
    {
        const MidLevel& L = d.L[t];
        const int n = owned( L ), base = (int)me * L.chunk;
        uint16_t* code = reinterpret_cast<uint16_t*>( blk + L.o_code );
        int32_t* nb = reinterpret_cast<int32_t*>( blk + L.o_nb );
        for( int i = threadIdx.x; i < n; i += kMidThreads ) code[i] = L.code[base + i];
        for( int i = threadIdx.x; i < n * 6; i += kMidThreads )
        {
            const int c = base + i / 6, q = i % 6;
            int nc;
            if( L.tiled ) nc = d.nbr[(size_t)c * 27 + kFaceDir[q]];
            else
            {
                const int x = c % L.dx, y = ( c / L.dx ) % L.dy, z = c / ( L.dx * L.dy );
                switch( q )
                {
                    case 0: nc = x > 0 ? c - 1 : -1; break;
                    case 1: nc = x < L.dx - 1 ? c + 1 : -1; break;
                    case 2: nc = y > 0 ? c - L.dx : -1; break;
                    case 3: nc = y < L.dy - 1 ? c + L.dx : -1; break;
                    case 4: nc = z > 0 ? c - L.dx * L.dy : -1; break;
                    default: nc = z < L.dz - 1 ? c + L.dx * L.dy : -1; break;
                }
            }
            nb[i] = ref( L, nc );
        }
        if( L.o_par >= 0 )
        {
            const MidLevel& P = d.L[t + 1];
            int32_t* par = reinterpret_cast<int32_t*>( blk + L.o_par );
            for( int i = threadIdx.x; i < n; i += kMidThreads )
            {
                const int c = base + i;
                int x, y, z;
                if( L.tiled )
                {
                    const int vt = d.tile_of[c];
                    x = vt % d.tx; y = ( vt / d.tx ) % d.ty; z = vt / ( d.tx * d.ty );
                }
                else
                {
                    x = c % L.dx; y = ( c / L.dx ) % L.dy; z = c / ( L.dx * L.dy );
                }
                par[i] = ref( P, ( x >> 1 ) + P.dx * ( ( y >> 1 ) + P.dy * ( z >> 1 ) ) );
            }
        }
        if( L.o_ch >= 0 )
        {
            const MidLevel& F = d.L[t - 1];
            int32_t* ch = reinterpret_cast<int32_t*>( blk + L.o_ch );
            for( int i = threadIdx.x; i < n * 8; i += kMidThreads )
            {
                const int c = base + i / 8, o = i % 8;
                const int x = c % L.dx, y = ( c / L.dx ) % L.dy, z = c / ( L.dx * L.dy );
                const int a = 2 * x + ( o & 1 ), b = 2 * y + ( ( o >> 1 ) & 1 ), e = 2 * z + ( o >> 2 );
                int fc = -1;
                if( F.tiled )
                {
                    if( a < d.tx && b < d.ty && e < d.tz ) fc = d.slot_of[( (size_t)e * d.ty + b ) * d.tx + a];
                }
                else if( a < F.dx && b < F.dy && e < F.dz )
                {
                    fc = a + F.dx * ( b + F.dy * e );
                }
                ch[i] = ref( F, fc );
            }
        }
    }

    // out = in + w[d] (r - (d in - sum of fluid neighbours' in)) on the owned fluid cells, 0 elsewhere
    __device__ void sweep( int t, int in, int out, const float* w, uint32_t* err ) const
    {
        const MidLevel& L = d.L[t];
        const int n = owned( L );
        const uint16_t* code = arr<uint16_t>( L.o_code );
        const int32_t* nb = arr<int32_t>( L.o_nb );
        const float* r = arr<float>( L.o_r );
        const float* zi = arr<float>( in );
        float* zo = arr<float>( out );
        for( int lc = threadIdx.x; lc < n; lc += kMidThreads )
        {
            const uint16_t cc = code[lc];
            const int dg = code_diag( cc );
            float v = 0.f;
            if( ( cc & BORA_CODE_FLUID ) && dg > 0 )
            {
                float sum = 0.f;
#pragma unroll
                for( int q = 0; q < 6; ++q )
                {
                    if( !( cc & ( 1u << q ) ) ) continue;
                    const int32_t rf = nb[lc * 6 + q];
                    if( rf < 0 ) { atomicOr( err, 4u ); continue; }
                    sum += ld( in, rf );
                }
                const float z = zi[lc];
                v = z + w[dg] * ( r[lc] - ( (float)dg * z - sum ) );
            }
            zo[lc] = v;
        }
    }
    // A = r - S B on the owned cells (0 on non-fluid cells)
    __device__ void residual( int t, uint32_t* err ) const
    {
        const MidLevel& L = d.L[t];
        const int n = owned( L );
        const uint16_t* code = arr<uint16_t>( L.o_code );
        const int32_t* nb = arr<int32_t>( L.o_nb );
        const float* r = arr<float>( L.o_r );
        const float* zb = arr<float>( L.o_b );
        float* res = arr<float>( L.o_a );
        for( int lc = threadIdx.x; lc < n; lc += kMidThreads )
        {
            const uint16_t cc = code[lc];
            float v = 0.f;
            if( cc & BORA_CODE_FLUID )
            {
                float sum = 0.f;
#pragma unroll
                for( int q = 0; q < 6; ++q )
                {
                    if( !( cc & ( 1u << q ) ) ) continue;
                    const int32_t rf = nb[lc * 6 + q];
                    if( rf < 0 ) { atomicOr( err, 8u ); continue; }
                    sum += ld( L.o_b, rf );
                }
                v = r[lc] - ( (float)code_diag( cc ) * zb[lc] - sum );
            }
            res[lc] = v;
        }
    }
    // level t (>= 1): r = 0.5 * sum of the children's residuals (A of level t - 1), and the
    // first pre-smoothing sweep from zero, A = w[d] r
    __device__ void gather( int t, const float* w ) const
    {
        const MidLevel& L = d.L[t];
        const MidLevel& F = d.L[t - 1];
        const int n = owned( L );
        const uint16_t* code = arr<uint16_t>( L.o_code );
        const int32_t* ch = arr<int32_t>( L.o_ch );
        float* r = arr<float>( L.o_r );
        float* a = arr<float>( L.o_a );
        for( int lc = threadIdx.x; lc < n; lc += kMidThreads )
        {
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for( int o = 0; o < 8; o += 2 )
            {
                const int32_t c0 = ch[lc * 8 + o], c1 = ch[lc * 8 + o + 1];
                if( c0 >= 0 ) s0 += ld( F.o_a, c0 );
                if( c1 >= 0 ) s1 += ld( F.o_a, c1 );
            }
            const float rv = 0.5f * ( s0 + s1 );
            const uint16_t cc = code[lc];
            const int dg = code_diag( cc );
            r[lc] = rv;
            a[lc] = ( ( cc & BORA_CODE_FLUID ) && dg > 0 ) ? w[dg] * rv : 0.f;
        }
    }
    // A = B + Z(parent) on the owned fluid cells (Z = array zoff of level t + 1)
    __device__ void inject( int t, int zoff ) const
    {
        const MidLevel& L = d.L[t];
        const int n = owned( L );
        const uint16_t* code = arr<uint16_t>( L.o_code );
        const int32_t* par = arr<int32_t>( L.o_par );
        const float* zb = arr<float>( L.o_b );
        float* a = arr<float>( L.o_a );
        for( int lc = threadIdx.x; lc < n; lc += kMidThreads )
        {
            const uint16_t cc = code[lc];
            float v = 0.f;
            if( ( cc & BORA_CODE_FLUID ) && code_diag( cc ) > 0 ) v = zb[lc] + ld( zoff, par[lc] );
            a[lc] = v;
        }
    }
};

// One CTA per cluster CTA: lay out that CTA's static block of the image (once per step).
__global__ void __launch_bounds__( kMidThreads ) k_mg_mid_image( const __grid_constant__ MidDesc d )
{
    Mid m{ d, cg::this_cluster(), blockIdx.x };
    char* blk = d.image + (size_t)blockIdx.x * d.static_bytes;
    for( int t = 0; t < d.n; ++t ) m.stage( t, blk );
}

__device__ __forceinline__ void mg_mid_body( const MidDesc& d )
{
    __shared__ float wA[16], wB[16], wC[16];
    uint32_t* err = d.err;
    Mid m{ d, cg::this_cluster(), 0u };
    m.me = m.cl.block_rank();
    const int tid = threadIdx.x;
    bora_pdl_trigger();
    if( tid < 16 )
    {
        wA[tid] = tid ? kOmegaA / (float)tid : 0.f;
        wB[tid] = tid ? kOmegaB / (float)tid : 0.f;
        wC[tid] = tid ? kOmega / (float)tid : 0.f;
    }
    // the static block (no kernel of the solve writes it) before the dependency wait:
    // asynchronous 16-byte copies, all in flight at once
    {
        const char* src = d.image + (size_t)m.me * d.static_bytes;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared( g_mid_smem );
        for( int i = tid * 16; i < d.static_bytes; i += kMidThreads * 16 )
            asm volatile( "cp.async.cg.shared.global [%0], [%1], 16;" ::"r"( dst + i ), "l"( src + i ) : "memory" );
        asm volatile( "cp.async.commit_group;\n\tcp.async.wait_all;" ::: "memory" );
    }
    bora_pdl_wait();  // the level-2 down kernel's restricted residual is complete from here
    __syncthreads();
    {
        const MidLevel& L = d.L[0];
        const int n = m.owned( L );
        const uint16_t* code = m.arr<uint16_t>( L.o_code );
        float* r = m.arr<float>( L.o_r );
        float* a = m.arr<float>( L.o_a );
        const __half* g = d.r_in + (size_t)m.me * L.chunk;
        for( int i = tid; i < n; i += kMidThreads )
        {
            const uint16_t cc = code[i];
            const int dg = code_diag( cc );
            const float rv = ( cc & BORA_CODE_FLUID ) ? __half2float( g[i] ) : 0.f;
            r[i] = rv;
            a[i] = ( ( cc & BORA_CODE_FLUID ) && dg > 0 ) ? wA[dg] * rv : 0.f;
        }
    }
    m.barrier();
    // ---- down ----
    const int last = d.n - 1;
    for( int t = 0; t < last; ++t )
    {
        const MidLevel& L = d.L[t];
        m.sweep( t, L.o_a, L.o_b, wB, err );         // B = second pre-smoothing sweep
        m.barrier();
        m.residual( t, err );                        // A = r - S B
        m.barrier();
        m.gather( t + 1, t + 1 == last ? wC : wA );  // coarser r and its pointwise first sweep
        m.barrier();
    }
    // ---- coarsest level: damped Jacobi from zero in CTA 0 (the first sweep, pointwise,
    // came with the gather). Each thread keeps its cell's code, weight, residual and
    // neighbours in registers across the sweeps; the values ping-pong between A and B. ----
    const MidLevel& Lc = d.L[last];
    const int zc = ( d.sweeps - 1 ) % 2 == 0 ? Lc.o_a : Lc.o_b;  // the coarsest correction's array
    if( m.me == 0 && d.sweeps > 1 )
    {
        float* za = m.arr<float>( Lc.o_a );
        float* zb = m.arr<float>( Lc.o_b );
        const bool mine = tid < Lc.n;
        const uint16_t cc = mine ? m.arr<uint16_t>( Lc.o_code )[tid] : 0;
        const int dg = code_diag( cc );
        const bool act = mine && ( cc & BORA_CODE_FLUID ) && dg > 0;
        const float w = wC[dg], rc = mine ? m.arr<float>( Lc.o_r )[tid] : 0.f, fd = (float)dg;
        int nbl[6];
#pragma unroll
        for( int q = 0; q < 6; ++q )
        {
            nbl[q] = -1;
            if( act && ( cc & ( 1u << q ) ) )
            {
                const int32_t rf = m.arr<int32_t>( Lc.o_nb )[tid * 6 + q];  // owner 0: the index is local
                if( rf < 0 ) atomicOr( err, 4u );
                else nbl[q] = rf & 0xFFFFFF;
            }
        }
        for( int it = 1; it < d.sweeps; ++it )
        {
            const float* zi = ( it & 1 ) ? za : zb;
            float* zo = ( it & 1 ) ? zb : za;
            if( mine )
            {
                float v = 0.f;
                if( act )
                {
                    float sum = 0.f;
#pragma unroll
                    for( int q = 0; q < 6; ++q )
                        if( nbl[q] >= 0 ) sum += zi[nbl[q]];
                    const float z = zi[tid];
                    v = z + w * ( rc - ( fd * z - sum ) );
                }
                zo[tid] = v;
            }
            __syncthreads();
        }
    }
    m.barrier();
    // ---- up ----
    for( int t = last - 1; t >= 0; --t )
    {
        const MidLevel& L = d.L[t];
        m.inject( t, t + 1 == last ? zc : d.L[t + 1].o_a );  // A = B + Z(parent)
        m.barrier();
        m.sweep( t, L.o_a, L.o_b, wB, err );                   // B = A + wB (r - S A)
        m.barrier();
        m.sweep( t, L.o_b, L.o_a, wA, err );                   // A = final correction
        if( t > 0 ) m.barrier();
    }
    {
        const MidLevel& L = d.L[0];
        const int n = m.owned( L );
        const float* a = m.arr<float>( L.o_a );
        __half* g = d.z_out + (size_t)m.me * L.chunk;
        for( int i = tid; i < n; i += kMidThreads ) g[i] = __float2half_rn( a[i] );
    }
    m.barrier();  // no CTA leaves while another may still read its shared memory
}

__global__ void __launch_bounds__( kMidThreads, 1 ) k_mg_mid( const __grid_constant__ MidDesc d ) { mg_mid_body( d ); }

// Batched: one cluster per simulation taking part (all clusters of the same size; a
// simulation's offset in the launch is a multiple of it, so a cluster is one simulation's).
__global__ void __launch_bounds__( kMidThreads, 1 ) k_mg_mid_batch( const MidDesc* __restrict__ descs,
                                                                    const __grid_constant__ BoraBatchLaunch L )
{
    unsigned bid;
    mg_mid_body( descs[bora_batch_member( L, blockIdx.x, &bid )] );
}

// Cluster size: 16 CTAs where the device co-schedules such a cluster of this kernel with
// the largest shared memory it may ask for, else 8; 0 when neither fits (the caller then
// runs these levels itself). Queried once per device.
int mid_cluster_size()
{
    static BoraPerDevice size;  // 16, 8, or 1 for "none"
    const int v = size.get( [] {
        cudaFuncSetAttribute( k_mg_mid, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 );
        cudaFuncSetAttribute( k_mg_mid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMidSmemMax );
        cudaFuncSetAttribute( k_mg_mid_batch, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 );
        cudaFuncSetAttribute( k_mg_mid_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMidSmemMax );
        cudaGetLastError();
        auto fits = []( int ctas ) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3( ctas );
            cfg.blockDim = dim3( kMidThreads );
            cfg.dynamicSmemBytes = kMidSmemMax;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = ctas;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            const bool ok = cudaOccupancyMaxActiveClusters( &clusters, k_mg_mid, &cfg ) == cudaSuccess && clusters > 0;
            cudaGetLastError();  // a refused query leaves no error behind
            return ok;
        };
        return fits( kMidCtasMax ) ? kMidCtasMax : ( fits( 8 ) ? 8 : 1 );
    } );
    return v > 1 ? v : 0;
}

// Shared-memory layout of the levels for `ctas` CTAs: the static block (codes, neighbour,
// parent and child references of every level) first, then the values. Returns the bytes
// per CTA.
size_t mid_layout( MidDesc& d, int ctas )
{
    size_t off = 0;
    auto take = [&]( size_t bytes ) {
        const int o = (int)off;
        off += ( bytes + 15 ) & ~(size_t)15;
        return o;
    };
    d.ctas = ctas;
    for( int t = 0; t < d.n; ++t )
    {
        MidLevel& L = d.L[t];
        L.chunk = t == d.n - 1 ? L.n : ( L.n + ctas - 1 ) / ctas;
        const size_t c = (size_t)L.chunk;
        L.o_code = take( c * 2 );
        L.o_nb = take( c * 6 * 4 );
        L.o_par = t < d.n - 1 ? take( c * 4 ) : -1;
        L.o_ch = t > 0 ? take( c * 8 * 4 ) : -1;
    }
    d.static_bytes = (int)off;
    for( int t = 0; t < d.n; ++t )
    {
        MidLevel& L = d.L[t];
        const size_t c = (size_t)L.chunk;
        L.o_r = take( c * 4 );
        L.o_a = take( c * 4 );
        L.o_b = take( c * 4 );
    }
    return off;
}

// The cluster layout of level 3 .. coarsest, or false when the hierarchy does not have the
// shape this kernel handles (level 3 with one cell per tile, then dense grids ending at
// <= 512 cells) or a level does not fit the cluster's shared memory.
bool mid_describe( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles, int sweeps,
                   MidDesc& d, size_t& smem )
{
    constexpr int first = 3;
    if( nlevels < first + 2 || nlevels - first > kMidMaxLevels || ntiles <= 0 || sweeps < 1 ) return false;
    if( levels[first].kind != 0 || levels[first].E != 1 || (int)levels[first].ncells != ntiles ) return false;
    for( int l = first + 1; l < nlevels; ++l )
        if( levels[l].kind != 1 ) return false;
    if( levels[nlevels - 1].ncells > 512 || ntiles >= ( 1 << 24 ) ) return false;
    d = MidDesc{};
    d.n = nlevels - first;
    for( int q = 0; q < d.n; ++q )
    {
        const BoraLevelDev& B = levels[first + q];
        MidLevel& L = d.L[q];
        L.tiled = q == 0;
        L.n = (int)B.ncells;
        L.dx = B.dx; L.dy = B.dy; L.dz = B.dz;
        L.code = B.code;
    }
    d.nbr = t.nbr; d.tile_of = t.tile_of; d.slot_of = t.slot_of;
    d.tx = g.tx; d.ty = g.ty; d.tz = g.tz;
    d.r_in = levels[first].r;
    d.z_out = levels[first].z0;
    d.sweeps = sweeps;
    const int ctas = mid_cluster_size();
    if( ctas == 0 ) return false;
    smem = mid_layout( d, ctas );
    return smem <= kMidSmemMax;
}

}  // namespace

size_t bora_mg_mid_image_bytes( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles )
{
    MidDesc d;
    size_t smem = 0;
    if( !mid_describe( g, levels, nlevels, t, ntiles, 16, d, smem ) ) return 0;
    return (size_t)d.ctas * d.static_bytes;
}

void bora_mg_mid_setup( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles,
                        void* image, cudaStream_t st )
{
    MidDesc d;
    size_t smem = 0;
    if( !image || !mid_describe( g, levels, nlevels, t, ntiles, 16, d, smem ) ) return;
    d.image = static_cast<char*>( image );
    k_mg_mid_image<<<d.ctas, kMidThreads, 0, st>>>( d );
}

int bora_mg_mid_vcycle( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles,
                        const void* image, uint32_t* err, int sweeps, cudaStream_t st, bool launch )
{
    MidDesc d;
    size_t smem = 0;
    if( !image || !mid_describe( g, levels, nlevels, t, ntiles, sweeps, d, smem ) ) return 0;
    if( !launch ) return 1;
    d.image = static_cast<char*>( const_cast<void*>( image ) );
    d.err = err;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3( d.ctas );
    cfg.blockDim = dim3( kMidThreads );
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = d.ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    cudaLaunchKernelEx( &cfg, k_mg_mid, d );
    return 1;
}

size_t bora_mg_mid_desc_bytes() { return sizeof( MidDesc ); }

int bora_mg_mid_describe( const BoraGridDev& g, const BoraLevelDev* levels, int nlevels, BoraTilesDev t, int ntiles,
                          const void* image, uint32_t* err, int sweeps, void* desc, size_t* smem, int* ctas )
{
    MidDesc d;
    size_t sm = 0;
    if( !image || !mid_describe( g, levels, nlevels, t, ntiles, sweeps, d, sm ) ) return 0;
    d.image = static_cast<char*>( const_cast<void*>( image ) );
    d.err = err;
    std::memcpy( desc, &d, sizeof( d ) );
    *smem = sm;
    *ctas = d.ctas;
    return 1;
}

void bora_mg_mid_launch_batch( const void* descs, const BoraBatchLaunch& L, int blocks, int ctas, size_t smem,
                               cudaStream_t st )
{
    if( blocks <= 0 || ctas <= 0 || blocks % ctas ) return;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3( blocks );
    cfg.blockDim = dim3( kMidThreads );
    cfg.dynamicSmemBytes = smem;
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
    cudaLaunchKernelEx( &cfg, k_mg_mid_batch, static_cast<const MidDesc*>( descs ), L );
}
