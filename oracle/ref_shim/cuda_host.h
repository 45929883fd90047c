// ORACLE INFRASTRUCTURE: host stand-ins for the CUDA runtime calls that the reference's
// FLIP sources make (managed allocation in base/header/Array.h:1194-1235 and
// base/source/SparseFrame.cu:12-26, atomicAdd in SparseFrame.cu:112 and
// Rasterization.cu:165-168,224).
#pragma once

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <cstddef>

typedef int cudaError_t;
enum cudaMemcpyKind
{
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

// Every "device" allocation carries a zero-filled guard region in front of it.
// The reference's tile-marking kernel (SparseFrame.cu:105-113) adds 1 at negative
// tile indices for particles in the first tile row/column; the guard absorbs
// those writes instead of corrupting the heap. Zero fill also matches what
// SparseFrame::create relies on when it assigns an object into fresh managed
// memory (SparseFrame.cu:15-16).
static const size_t kShimGuardBytes = (size_t)4 << 20;

inline cudaError_t shimAlloc( void** p, size_t bytes )
{
    char* raw = (char*)std::calloc( 1, bytes + kShimGuardBytes );
    if( !raw ) { *p = nullptr; return 2; }
    *p = raw + kShimGuardBytes;
    return 0;
}

template <class T> inline cudaError_t cudaMallocManaged( T** p, size_t bytes ) { return shimAlloc( (void**)p, bytes ); }
template <class T> inline cudaError_t cudaMalloc( T** p, size_t bytes ) { return shimAlloc( (void**)p, bytes ); }

inline cudaError_t cudaFree( void* p )
{
    if( p ) std::free( (char*)p - kShimGuardBytes );
    return 0;
}

inline cudaError_t cudaMemcpy( void* dst, const void* src, size_t n, cudaMemcpyKind ) { std::memmove( dst, src, n ); return 0; }
inline cudaError_t cudaMemset( void* dst, int v, size_t n ) { std::memset( dst, v, n ); return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }

template <class T>
inline T atomicAdd( T* addr, T v )
{
    return std::atomic_ref<T>( *addr ).fetch_add( v, std::memory_order_relaxed );
}
