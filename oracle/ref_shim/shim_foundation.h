// ORACLE INFRASTRUCTURE: host stand-ins for what the reference's Foundation.h pulls in
// (base/header/Foundation.h). Used only to compile the reference's FLIP sources for the
// CPU; see Bora.h in this directory.
#pragma once

#include <map>
#include <set>
#include <list>
#include <stack>
#include <queue>
#include <cmath>
#include <cfloat>
#include <cstring>
#include <bitset>
#include <vector>
#include <string>
#include <atomic>
#include <cstdarg>
#include <fstream>
#include <iomanip>
#include <climits>
#include <cstdlib>
#include <cstdint>
#include <iostream>
#include <sstream>
#include <iterator>
#include <numeric>
#include <algorithm>
#include <chrono>
#include <unordered_set>
#include <unordered_map>
#include <sys/stat.h>
#include <sys/time.h>

// ---- qualifiers and namespace macros (base/header/Foundation.h:11-21) -------------
#define __device__
#define __host__
#define BORA_FUNC_QUAL
#define BORA_UNIFIED
#define BORA_DEVICE
#define BORA_HOST
#define BORA_NAMESPACE_BEGIN namespace Bora {
#define BORA_NAMESPACE_END }
#define BORA_HOST_KERNEL [&] ( const size_t ix )
#define BORA_DEVICE_KERNEL [=] ( const size_t ix )

// ---- CUDA runtime stand-ins -------------------------------------------------------
#include "cuda_host.h"

// ---- launch substrate (base/header/LauncherCuda.h:13-29) --------------------------
// The reference runs every per-element lambda through thrust::for_each on the device.
// On the host the same lambdas run as an OpenMP parallel loop (the reference has no
// multithreaded CPU path of its own; its LaunchCudaHost is serial).
template <class KERNEL>
inline void LaunchCudaDevice( KERNEL& kernel, const size_t& P, const size_t& N )
{
    const long long lo = (long long)P, hi = (long long)(P + N);
#pragma omp parallel for schedule(static)
    for( long long n = lo; n < hi; ++n ) kernel( (size_t)n );
}

template <class KERNEL>
inline void LaunchCudaHost( KERNEL& kernel, const size_t& P, const size_t& N )
{
    for( size_t n = P; n < P + N; ++n ) kernel( n );
}

inline void SyncCuda() {}

// ---- thrust names used by BLAS::dot (base/source/BLAS.cu:98-104) -----------------
namespace thrust
{
    template <class T> using device_ptr = T*;
    template <class I1, class I2, class T>
    inline T inner_product( I1 a0, I1 a1, I2 b0, T init ) { return std::inner_product( a0, a1, b0, init ); }
}

// ---- glm: only the type names that appear in conversion operators ---------------
namespace glm
{
    template <class T> struct tvec2 { T x, y; tvec2( T a=0, T b=0 ) : x(a), y(b) {} };
    template <class T> struct tvec3 { T x, y, z; tvec3( T a=0, T b=0, T c=0 ) : x(a), y(b), z(c) {} };
    template <class T> struct tvec4 { T x, y, z, w; tvec4( T a=0, T b=0, T c=0, T d=0 ) : x(a), y(b), z(c), w(d) {} };
    template <class T> struct tmat2x2 { tvec2<T> c[2]; tmat2x2() {} template <class V> tmat2x2( const V&, const V& ) {} tvec2<T>& operator[]( int i ) { return c[i]; } const tvec2<T>& operator[]( int i ) const { return c[i]; } };
    template <class T> struct tmat3x3 { tvec3<T> c[3]; tmat3x3() {} template <class V> tmat3x3( const V&, const V&, const V& ) {} tvec3<T>& operator[]( int i ) { return c[i]; } const tvec3<T>& operator[]( int i ) const { return c[i]; } };
    template <class T> struct tmat4x4 { tvec4<T> c[4]; tmat4x4() {} template <class V> tmat4x4( const V&, const V&, const V&, const V& ) {} tvec4<T>& operator[]( int i ) { return c[i]; } const tvec4<T>& operator[]( int i ) const { return c[i]; } };
    template <class T> struct tquat
    {
        T w, x, y, z;
        tquat( T a=1, T b=0, T c=0, T d=0 ) : w(a), x(b), y(c), z(d) {}
        template <class U> tquat( const tquat<U>& q ) : w((T)q.w), x((T)q.x), y((T)q.y), z((T)q.z) {}
    };
    typedef tvec4<float> vec4;
    typedef tquat<float> fquat;
    typedef tquat<double> dquat;
    // Curl noise is disabled on the FLIP path (FLIPMethod.h:58 enableCurl=false).
    inline float perlin( const vec4& ) { return 0.f; }
    inline float simplex( const vec4& ) { return 0.f; }
}

// ---- OpenGL: no-op declarations so that the viewport-drawing members of Grid and
// ---- Particles parse. They are never called on the FLIP path and draw nothing.
#define GL_LINES 1
#define GL_POINTS 0
#define GL_FLOAT 0x1406
#define GL_VERTEX_ARRAY 0x8074
#define GL_COLOR_ARRAY 0x8076
inline void glBegin( int ) {}
inline void glEnd() {}
inline void glVertex3f( float, float, float ) {}
inline void glPushMatrix() {}
inline void glPopMatrix() {}
inline void glMultMatrixf( const float* ) {}
inline void glScalef( float, float, float ) {}
inline void glScale( float, float, float ) {}
inline void glTranslatef( float, float, float ) {}
inline void glEnableClientState( int ) {}
inline void glDisableClientState( int ) {}
inline void glVertexPointer( int, int, int, const void* ) {}
inline void glColorPointer( int, int, int, const void* ) {}
inline void glDrawArrays( int, int, size_t ) {}
inline void glColor3f( float, float, float ) {}
inline void glPointSize( float ) {}

// ---- OpenVDB: the two grid handle types named in FLIPMethod's signature ----------
namespace openvdb
{
    struct FloatGrid { typedef const FloatGrid* ConstPtr; };
    struct Vec3fGrid { typedef const Vec3fGrid* ConstPtr; };
}
