// Device exclusive prefix sum of uint32 counts (tile activation flags, per-dual-cell
// particle counts). Three passes: per-block sums, one-block scan of the block sums,
// per-block scan with the block's offset. Each pass reads its input with 128-bit
// loads; the block-sum scratch array (2048 elements per block) is owned by the caller.
#include "bora_internal.h"

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;  // per thread -> 2048 elements per block
constexpr int kScanChunk = kScanThreads * kScanItems;

__device__ inline uint32_t warp_incl_scan( uint32_t v )
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for( int o = 1; o < 32; o <<= 1 )
    {
        const uint32_t t = __shfl_up_sync( 0xffffffffu, v, o );
        if( lane >= o ) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and
// the block total in *total.
__device__ inline uint32_t block_excl_scan( uint32_t v, uint32_t* total )
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan( v );
    if( lane == 31 ) warp_sums[wid] = inc;
    __syncthreads();
    if( wid == 0 )
    {
        uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        s = warp_incl_scan( s );
        if( lane < kScanThreads / 32 ) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t base = wid > 0 ? warp_sums[wid - 1] : 0u;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return base + inc - v;
}

__device__ inline void load_items( const uint32_t* __restrict__ in, size_t n, size_t base, uint32_t v[kScanItems] )
{
    const size_t i0 = base + (size_t)threadIdx.x * kScanItems;
    if( i0 + kScanItems <= n && ( ( reinterpret_cast<uintptr_t>( in + i0 ) & 15 ) == 0 ) )
    {
        const uint4 a = *reinterpret_cast<const uint4*>( in + i0 );
        const uint4 b = *reinterpret_cast<const uint4*>( in + i0 + 4 );
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
    else
    {
#pragma unroll
        for( int q = 0; q < kScanItems; ++q ) v[q] = ( i0 + q < n ) ? in[i0 + q] : 0u;
    }
}

__global__ void k_scan_reduce( const uint32_t* __restrict__ in, size_t n, uint32_t* __restrict__ block_sums )
{
    uint32_t v[kScanItems];
    load_items( in, n, (size_t)blockIdx.x * kScanChunk, v );
    uint32_t s = 0;
#pragma unroll
    for( int q = 0; q < kScanItems; ++q ) s += v[q];
    uint32_t total;
    block_excl_scan( s, &total );
    if( threadIdx.x == 0 ) block_sums[blockIdx.x] = total;
}

// One block scans the nb block sums in place (exclusive) and writes the grand total.
__global__ void k_scan_blocks( uint32_t* __restrict__ block_sums, int nb, uint32_t* __restrict__ grand_total )
{
    uint32_t carry = 0;
    for( int base = 0; base < nb; base += kScanThreads )
    {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nb ? block_sums[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_excl_scan( v, &total );
        if( i < nb ) block_sums[i] = carry + ex;
        carry += total;
    }
    if( threadIdx.x == 0 && grand_total ) *grand_total = carry;
}

__global__ void k_scan_down( const uint32_t* __restrict__ in, size_t n, const uint32_t* __restrict__ block_sums,
                             uint32_t* __restrict__ out )
{
    uint32_t v[kScanItems];
    const size_t base = (size_t)blockIdx.x * kScanChunk;
    load_items( in, n, base, v );
    uint32_t s = 0;
#pragma unroll
    for( int q = 0; q < kScanItems; ++q ) s += v[q];
    uint32_t total;
    uint32_t run = block_excl_scan( s, &total ) + block_sums[blockIdx.x];
    const size_t i0 = base + (size_t)threadIdx.x * kScanItems;
    uint32_t o[kScanItems];
#pragma unroll
    for( int q = 0; q < kScanItems; ++q ) { o[q] = run; run += v[q]; }
    if( i0 + kScanItems <= n && ( ( reinterpret_cast<uintptr_t>( out + i0 ) & 15 ) == 0 ) )
    {
        *reinterpret_cast<uint4*>( out + i0 ) = make_uint4( o[0], o[1], o[2], o[3] );
        *reinterpret_cast<uint4*>( out + i0 + 4 ) = make_uint4( o[4], o[5], o[6], o[7] );
    }
    else
    {
#pragma unroll
        for( int q = 0; q < kScanItems; ++q )
            if( i0 + q < n ) out[i0 + q] = o[q];
    }
}

}  // namespace

size_t bora_scan_scratch_elems( size_t n ) { return ( n + kScanChunk - 1 ) / kScanChunk + 1; }

// out[i] = sum_{j<i} in[i]; *total = sum of all (device pointer, may be null).
// in and out may alias. scratch holds bora_scan_scratch_elems(n) uint32.
void bora_device_scan( const uint32_t* in, uint32_t* out, size_t n, uint32_t* scratch, uint32_t* total, cudaStream_t st )
{
    if( n == 0 )
    {
        if( total ) cudaMemsetAsync( total, 0, sizeof( uint32_t ), st );
        return;
    }
    const int nb = (int)( ( n + kScanChunk - 1 ) / kScanChunk );
    k_scan_reduce<<<nb, kScanThreads, 0, st>>>( in, n, scratch );
    k_scan_blocks<<<1, kScanThreads, 0, st>>>( scratch, nb, total );
    k_scan_down<<<nb, kScanThreads, 0, st>>>( in, n, scratch, out );
}

// ---- public C ABI: device exclusive prefix sum -------------------------------------
#include "../../include/bora_flip.h"

extern "C" int bora_scan_u32( const uint32_t* d_in, uint32_t* d_out, size_t n, uint32_t* d_total, void* stream )
{
    if( n > 0 && ( !d_in || !d_out ) ) return BORA_ERR_INVALID_ARG;
    if( n > (size_t)0xFFFFFFFFu ) return BORA_ERR_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* scratch = nullptr;
    if( n > 0 )
    {
        // stream-ordered scratch for the per-block sums, released on the same stream
        const cudaError_t e = cudaMallocAsync( (void**)&scratch, bora_scan_scratch_elems( n ) * sizeof( uint32_t ), st );
        if( e != cudaSuccess ) return e == cudaErrorMemoryAllocation ? BORA_ERR_OUT_OF_MEMORY : BORA_ERR_CUDA;
    }
    bora_device_scan( d_in, d_out, n, scratch, d_total, st );
    cudaError_t e = cudaGetLastError();
    if( scratch )
    {
        const cudaError_t f = cudaFreeAsync( scratch, st );
        if( e == cudaSuccess ) e = f;
    }
    return e == cudaSuccess ? BORA_OK : BORA_ERR_CUDA;
}

// ---- no-allocation variant ---------------------------------------------------------
// For callers that must not allocate device memory (see bora_scan_u32_noalloc in
// include/bora_flip.h). The per-block sums live in this file-scope array: 2048 input
// counts per block, so 2^28 counts need 131,073 sums (512 KiB + 4 B). Every device that
// loads the library holds the array until the process exits.
#include <mutex>

#define BORA_SCAN_NOALLOC_MAX ( (size_t)1 << 28 )
static __device__ __align__( 256 ) uint32_t g_noalloc_block_sums[BORA_SCAN_NOALLOC_MAX / kScanChunk + 1];

namespace {
std::mutex g_noalloc_mutex;
uint32_t* g_noalloc_addr[64] = {};  // device address of g_noalloc_block_sums, per device ordinal
}  // namespace

extern "C" int bora_scan_u32_noalloc( const uint32_t* d_in, uint32_t* d_out, size_t n, uint32_t* d_total, void* stream )
{
    if( n > 0 && ( !d_in || !d_out ) ) return BORA_ERR_INVALID_ARG;
    if( n > BORA_SCAN_NOALLOC_MAX ) return BORA_ERR_CAPACITY;
    int dev = -1;
    if( cudaGetDevice( &dev ) != cudaSuccess || dev < 0 || dev >= 64 ) return BORA_ERR_CUDA;
    uint32_t* scratch = nullptr;
    {
        // First call on this device: the host-side name of the array is not a device
        // address, so ask the runtime for the address on the current device.
        std::lock_guard<std::mutex> lock( g_noalloc_mutex );
        if( !g_noalloc_addr[dev] )
        {
            void* p = nullptr;
            if( cudaGetSymbolAddress( &p, g_noalloc_block_sums ) != cudaSuccess || !p ) return BORA_ERR_CUDA;
            g_noalloc_addr[dev] = static_cast<uint32_t*>( p );
        }
        scratch = g_noalloc_addr[dev];
    }
    // Each call writes every block sum before reading it, so the array's previous
    // contents never matter and nothing needs clearing.
    bora_device_scan( d_in, d_out, n, scratch, d_total, (cudaStream_t)stream );
    return cudaGetLastError() == cudaSuccess ? BORA_OK : BORA_ERR_CUDA;
}
