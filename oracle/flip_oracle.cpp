// ORACLE (test infrastructure only): a CPU restatement of the reference's sparse-grid
// FLIP substep, FLIPMethod::advanceOneStep (base/source/FLIPMethod.cu:208-298).
//
// Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library, and only as the test oracle or the timed CPU baseline; the product path never
// calls it.
//
// Each stage follows the reference's arithmetic in the same operation order, so that
// with one thread and the reference's own tile size (4^3), tile-index wrap and CG stop
// rule ("compat" mode) it reproduces the reference bit for bit. With the build's tile
// size (8^3), the wrap-free activation rule and an FP64 CG solve it is the oracle that
// the device path is checked against. Compile with -ffp-contract=off: a fused
// multiply-add changes the rounding that this file restates.
#include <cmath>
#include <cstdint>
#include <climits>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <atomic>
#include <algorithm>
#include <omp.h>

#include "collider_math.h"

namespace {

// Cell types of FluidProjection::CELLTYPE (base/header/FluidProjection.h:32-39).
enum : int64_t { kAir = 0, kSolid = 1, kWall = 2, kMark = 3, kFluid = 4 };
const int64_t kNull = -1;  // NULL_MAX / MAX_SIZE_T (base/header/Definitions.h:22-23)

struct V3 { float x, y, z; };

inline float fminr( float a, float b ) { return a < b ? a : b; }  // MathUtils.h:174 Min
inline float fmaxr( float a, float b ) { return a > b ? a : b; }  // MathUtils.h:194 Max
inline int imin( int a, int b ) { return a < b ? a : b; }
inline int imax( int a, int b ) { return a > b ? a : b; }
inline float absr( float x ) { return x < 0 ? -x : x; }          // MathUtils.h:129 Abs
inline float clampf( float x, float lo, float hi ) { if( x < lo ) return lo; if( x > hi ) return hi; return x; }  // MathUtils.h:286
inline int clampi( int x, int lo, int hi ) { if( x < lo ) return lo; if( x > hi ) return hi; return x; }

template <class T> inline void atomic_add( T* a, T v ) { std::atomic_ref<T>( *a ).fetch_add( v, std::memory_order_relaxed ); }

}  // namespace

extern "C" {

typedef struct OracleConfig
{
    int nx, ny, nz;        // requested grid resolution (Grid::initialize)
    float bmin[3], bmax[3];
    int block;             // tile edge in cells: 4 (reference) or 8 (build)
    int compat_wrap;       // 1: reproduce the reference's unclamped tile-neighbour loop
    int solver;            // 0: reference CG rule (LinearSystemSolver.cpp:12-50), 1: FP64 CG to tol,
                           // 2: the reference's FP32 recurrence with FP64 dots to a relative tol
    double tol;            // relative tolerance of solvers 1 and 2
    int max_iter;          // projIteration (solver 0) / iteration cap (solver 1)
    float gravity[3];      // world units (FLIPMethod::Params::extForce)
    float wall_level;      // world units (FLIPMethod::Params::wallLevel)
    int maxsubsteps;
    float col_vel_scale;
    int enable_tank;
    float damping_band;    // world units
    float voxel_size;      // FLIPMethod::Params::voxelSize
    int advection;         // 0: the reference's Euler substeps; 1: RK2 midpoint in the grid velocity
} OracleConfig;

}

struct Oracle
{
    OracleConfig cfg;
    // frame (SparseFrame::initialize, base/source/SparseFrame.cu:28-73)
    int B = 4;
    int fx = 0, fy = 0, fz = 0;   // tile counts
    int nx = 0, ny = 0, nz = 0;   // frame grid (padded to a multiple of 4)
    float translate[3] = { 0, 0, 0 }, scale[3] = { 1, 1, 1 };
    float voxelWall = 0.f;
    V3 voxelForce = { 0, 0, 0 };
    std::vector<int64_t> pointers;   // per tile: storage offset or kNull
    std::vector<int32_t> markers;    // per tile: activation count
    std::vector<int64_t> coords;     // active tiles, 3 per tile
    // fields (SparseField storage: active tiles x B^3, x fastest inside the tile)
    std::vector<int64_t> mark;
    std::vector<float> mass, surf, pres;
    std::vector<V3> velo, comp;
    float surfBackground = 10.f;
    // projection
    std::vector<int64_t> fluidCells;
    std::vector<float> Avals;   // 7 per row
    std::vector<int64_t> Acols; // 7 per row
    std::vector<float> x, b;
    int lastIters = 0;
    double lastRel = 0.0;
    // particles
    std::vector<V3> pos, vel;
    std::vector<float> adj;
    std::vector<int32_t> pid;
    std::vector<uint8_t> removed;
    // colliders
    BoraColliderSet cols;
    std::vector<int> col_tslot;        // sparse collider (ora_set_collider_voxels)
    std::vector<float> col_tphi, col_tvel;

    size_t ncells() const { return coords.size() / 3 * (size_t)B * B * B; }

    // SparseField::operator() / findIndex (base/header/SparseField.h:57-95)
    inline int64_t findIndex( int i, int j, int k ) const
    {
        const int64_t p = pointers[(size_t)( k / B ) * fx * fy + (size_t)( j / B ) * fx + (size_t)( i / B )];
        if( p == kNull ) return kNull;
        return p + (int64_t)( k % B ) * B * B + (int64_t)( j % B ) * B + ( i % B );
    }
    // SparseField::findIndices (SparseField.h:104-112)
    inline void findIndices( size_t n, int& i, int& j, int& k ) const
    {
        const size_t bb = (size_t)B * B * B;
        const size_t t = n / bb, r = n % bb;
        i = (int)coords[3 * t] * B + (int)( r % B );
        j = (int)coords[3 * t + 1] * B + (int)( ( r / B ) % B );
        k = (int)coords[3 * t + 2] * B + (int)( ( r / ( B * B ) ) % B );
    }
    inline bool real( int i, int j, int k ) const { return i < nx && j < ny && k < nz; }

    template <class T> inline T at( const std::vector<T>& f, int i, int j, int k, T bg ) const
    {
        const int64_t n = findIndex( i, j, k );
        return n == kNull ? bg : f[(size_t)n];
    }

    // Collider queries (CollisionSource.h:128-150, restated in collider_math.h)
    inline float colPhi( float px, float py, float pz ) const
    {
        if( !bora_collider_active( &cols ) ) return 5.f;
        float v[3];
        bora_collider_lerp( &cols, nx, ny, nz, px, py, pz, BORA_COLLIDER_PHI, v );
        return v[0];
    }
    inline V3 colVec( float px, float py, float pz, int which ) const
    {
        if( !bora_collider_active( &cols ) ) return V3{ 0.f, 0.f, 0.f };
        float v[3];
        bora_collider_lerp( &cols, nx, ny, nz, px, py, pz, which, v );
        return V3{ v[0], v[1], v[2] };
    }

    // SparseField::lerp over a scalar field (SparseField.h:150-173)
    inline float lerpS( const std::vector<float>& f, float bg, float px, float py, float pz ) const
    {
        const int i = clampi( (int)( px - 0.5f ), 0, nx - 2 );
        const int j = clampi( (int)( py - 0.5f ), 0, ny - 2 );
        const int k = clampi( (int)( pz - 0.5f ), 0, nz - 2 );
        const float x = clampf( px - ( (float)i + .5f ), 0.f, 1.f );
        const float y = clampf( py - ( (float)j + .5f ), 0.f, 1.f );
        const float z = clampf( pz - ( (float)k + .5f ), 0.f, 1.f );
        const float c00 = at( f, i, j, k, bg ) * ( 1.f - x ) + at( f, i + 1, j, k, bg ) * x;
        const float c01 = at( f, i, j, k + 1, bg ) * ( 1.f - x ) + at( f, i + 1, j, k + 1, bg ) * x;
        const float c10 = at( f, i, j + 1, k, bg ) * ( 1.f - x ) + at( f, i + 1, j + 1, k, bg ) * x;
        const float c11 = at( f, i, j + 1, k + 1, bg ) * ( 1.f - x ) + at( f, i + 1, j + 1, k + 1, bg ) * x;
        const float c0 = c00 * ( 1.f - y ) + c10 * y;
        const float c1 = c01 * ( 1.f - y ) + c11 * y;
        return c0 * ( 1.f - z ) + c1 * z;
    }
    inline V3 lerpV( const std::vector<V3>& f, float px, float py, float pz ) const
    {
        const int i = clampi( (int)( px - 0.5f ), 0, nx - 2 );
        const int j = clampi( (int)( py - 0.5f ), 0, ny - 2 );
        const int k = clampi( (int)( pz - 0.5f ), 0, nz - 2 );
        const float x = clampf( px - ( (float)i + .5f ), 0.f, 1.f );
        const float y = clampf( py - ( (float)j + .5f ), 0.f, 1.f );
        const float z = clampf( pz - ( (float)k + .5f ), 0.f, 1.f );
        const V3 z0{ 0.f, 0.f, 0.f };
        const V3 a = at( f, i, j, k, z0 ), bb = at( f, i + 1, j, k, z0 );
        const V3 c = at( f, i, j, k + 1, z0 ), d = at( f, i + 1, j, k + 1, z0 );
        const V3 e = at( f, i, j + 1, k, z0 ), g = at( f, i + 1, j + 1, k, z0 );
        const V3 h = at( f, i, j + 1, k + 1, z0 ), q = at( f, i + 1, j + 1, k + 1, z0 );
        V3 out;
        float* o = &out.x;
        const float *A = &a.x, *Bv = &bb.x, *C = &c.x, *D = &d.x, *E = &e.x, *G = &g.x, *H = &h.x, *Q = &q.x;
        for( int m = 0; m < 3; ++m )
        {
            const float c00 = A[m] * ( 1.f - x ) + Bv[m] * x;
            const float c01 = C[m] * ( 1.f - x ) + D[m] * x;
            const float c10 = E[m] * ( 1.f - x ) + G[m] * x;
            const float c11 = H[m] * ( 1.f - x ) + Q[m] * x;
            const float c0 = c00 * ( 1.f - y ) + c10 * y;
            const float c1 = c01 * ( 1.f - y ) + c11 * y;
            o[m] = c0 * ( 1.f - z ) + c1 * z;
        }
        return out;
    }
    // SparseField::lerpMin (SparseField.h:176-196)
    inline float lerpMinS( const std::vector<float>& f, float bg, float px, float py, float pz ) const
    {
        const int i = clampi( (int)( px - 0.5f ), 0, nx - 2 );
        const int j = clampi( (int)( py - 0.5f ), 0, ny - 2 );
        const int k = clampi( (int)( pz - 0.5f ), 0, nz - 2 );
        float v = fminr( at( f, i, j, k, bg ), at( f, i + 1, j, k, bg ) );
        v = fminr( v, fminr( at( f, i, j, k + 1, bg ), at( f, i + 1, j, k + 1, bg ) ) );
        v = fminr( v, fminr( at( f, i, j + 1, k, bg ), at( f, i + 1, j + 1, k, bg ) ) );
        v = fminr( v, fminr( at( f, i, j + 1, k + 1, bg ), at( f, i + 1, j + 1, k + 1, bg ) ) );
        return v;
    }

    // ---------------------------------------------------------------------------------
    // SparseFrame::initialize (SparseFrame.cu:28-73) and FLIPMethod::initialize
    // (FLIPMethod.cu:16-47): pad the grid to a multiple of 4 cells per axis, re-centre
    // the box with a uniform spacing h = min(dx,dy,dz), convert gravity and the wall
    // level to voxel units.
    void initialize( const OracleConfig& c )
    {
        cfg = c;
        B = c.block;
        // Grid::initialize(Nx,Ny,Nz,min,max) (base/header/Grid.h:124-141)
        float gT[3] = { c.bmin[0], c.bmin[1], c.bmin[2] };
        float gS[3] = { ( c.bmax[0] - c.bmin[0] ) / (float)c.nx, ( c.bmax[1] - c.bmin[1] ) / (float)c.ny,
                        ( c.bmax[2] - c.bmin[2] ) / (float)c.nz };
        const int gn[3] = { c.nx, c.ny, c.nz };
        int f4[3];
        for( int a = 0; a < 3; ++a ) f4[a] = gn[a] / 4 + ( ( gn[a] % 4 ) ? 1 : 0 );
        nx = f4[0] * 4; ny = f4[1] * 4; nz = f4[2] * 4;
        // boundingBox() of the input grid (Grid.h:253-262)
        float minP[3], maxP[3], cen[3], d[3];
        for( int a = 0; a < 3; ++a )
        {
            const float e = gT[a] + (float)gn[a] * gS[a];
            minP[a] = gT[a] < e ? gT[a] : e;
            maxP[a] = gT[a] < e ? e : gT[a];
        }
        for( int a = 0; a < 3; ++a ) cen[a] = ( minP[a] + maxP[a] ) * 0.5f;
        for( int a = 0; a < 3; ++a ) d[a] = ( maxP[a] - minP[a] ) / (float)gn[a];
        const float h = fminr( fminr( d[0], d[1] ), d[2] );
        const float L[3] = { (float)nx * h, (float)ny * h, (float)nz * h };
        float nmin[3], nmax[3];
        for( int a = 0; a < 3; ++a ) nmin[a] = cen[a] - L[a] * 0.5f;
        for( int a = 0; a < 3; ++a ) nmax[a] = nmin[a] + L[a];
        const int fn[3] = { nx, ny, nz };
        for( int a = 0; a < 3; ++a )
        {
            translate[a] = nmin[a];
            scale[a] = ( nmax[a] - nmin[a] ) / (float)fn[a];
        }
        fx = ( nx + B - 1 ) / B; fy = ( ny + B - 1 ) / B; fz = ( nz + B - 1 ) / B;
        pointers.assign( (size_t)fx * fy * fz, kNull );
        markers.assign( (size_t)fx * fy * fz, 0 );
        coords.clear();
        // Grid::voxelVector / voxelPoint (Grid.h:446-458)
        voxelForce = V3{ c.gravity[0] / scale[0], c.gravity[1] / scale[1], c.gravity[2] / scale[2] };
        voxelWall = ( c.wall_level - translate[1] ) / scale[1];
        std::memset( &cols, 0, sizeof( cols ) );
        cols.band = 5.f;
    }

    // ---------------------------------------------------------------------------------
    // SparseFrame::buildFromPoints (SparseFrame.cu:83-155) + SparseFrame::build
    // (SparseFrame.cu:75-81, SparseField::build SparseField.h:221-226).
    void rebuild()
    {
        const int br = B;
        std::fill( markers.begin(), markers.end(), 0 );
        const int64_t ntiles = (int64_t)markers.size();
        const long long np = (long long)pos.size();
        const bool wrap = cfg.compat_wrap != 0;
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < np; ++n )
        {
            const V3& p = pos[(size_t)n];
            const int ci = imax( (int)( p.x ) / br, 0 );
            const int cj = imax( (int)( p.y ) / br, 0 );
            const int ck = imax( (int)( p.z ) / br, 0 );
            if( wrap )
            {
                // Reference loop (SparseFrame.cu:101-114): lower bounds are not clamped,
                // so index -1 wraps into the previous row/slab; writes outside the
                // table land in memory the reference does not own and are dropped here.
                for( int k = ck - 1; k <= imin( ck + 1, fz - 1 ); ++k )
                    for( int j = cj - 1; j <= imin( cj + 1, fy - 1 ); ++j )
                        for( int i = ci - 1; i <= imin( ci + 1, fx - 1 ); ++i )
                        {
                            const int64_t t = (int64_t)k * fx * fy + (int64_t)j * fx + i;
                            if( t >= 0 && t < ntiles ) atomic_add( &markers[(size_t)t], 1 );
                        }
            }
            else
            {
                // Build rule: the particle's tile (clamped to the table) dilated by one
                // tile, clamped on both sides, no wrap.
                const int ti = imin( ci, fx - 1 ), tj = imin( cj, fy - 1 ), tk = imin( ck, fz - 1 );
                for( int k = imax( tk - 1, 0 ); k <= imin( tk + 1, fz - 1 ); ++k )
                    for( int j = imax( tj - 1, 0 ); j <= imin( tj + 1, fy - 1 ); ++j )
                        for( int i = imax( ti - 1, 0 ); i <= imin( ti + 1, fx - 1 ); ++i )
                            atomic_add( &markers[(size_t)k * fx * fy + (size_t)j * fx + i], 1 );
            }
        }
        if( cfg.enable_tank )
        {
            // SparseFrame.cu:119-129
            const int tall = clampi( (int)( voxelWall ) / br, 0, fy );
            for( int k = 0; k < fz; ++k )
                for( int j = 0; j < tall; ++j )
                    for( int i = 0; i < fx; ++i ) markers[(size_t)k * fx * fy + (size_t)j * fx + i] = 1;
        }
        coords.clear();
        int64_t count = 0;
        const int64_t bs = (int64_t)br * br * br;
        for( size_t n = 0; n < markers.size(); ++n )
        {
            if( markers[n] > 0 )
            {
                pointers[n] = count;
                coords.push_back( (int64_t)( n % fx ) );
                coords.push_back( (int64_t)( ( n / fx ) % fy ) );
                coords.push_back( (int64_t)( ( n / ( (size_t)fx * fy ) ) % fz ) );
                count += bs;
            }
            else
            {
                pointers[n] = kNull;
            }
        }
        const size_t nc = ncells();
        // SparseField::build: every registered field re-filled with its background
        // (FLIPMethod.cu:28-33: mark 0, mass 0, surf 10, pres 0, velo 0, comp 0).
        mark.assign( nc, 0 );
        mass.assign( nc, 0.f );
        surf.assign( nc, surfBackground );
        pres.assign( nc, 0.f );
        velo.assign( nc, V3{ 0.f, 0.f, 0.f } );
        comp.assign( nc, V3{ 0.f, 0.f, 0.f } );
    }

    // ---------------------------------------------------------------------------------
    // Rasterization::PointsToVelField, sparse (base/source/Rasterization.cu:122-190) and
    // Rasterization::PointsToCountField, sparse (Rasterization.cu:199-229).
    void p2g()
    {
        std::fill( mass.begin(), mass.end(), 0.f );
        std::fill( velo.begin(), velo.end(), V3{ 0.f, 0.f, 0.f } );
        const int EI = nx - 1, EJ = ny - 1, EK = nz - 1;
        const long long np = (long long)pos.size();
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < np; ++n )
        {
            const V3 p = pos[(size_t)n];
            const V3 v = vel[(size_t)n];
            if( !inside( p ) ) continue;
            const int ci = imax( (int)( p.x - 0.5f ), 0 );
            const int cj = imax( (int)( p.y - 0.5f ), 0 );
            const int ck = imax( (int)( p.z - 0.5f ), 0 );
            for( int k = ck; k <= imin( ck + 1, EK ); ++k )
                for( int j = cj; j <= imin( cj + 1, EJ ); ++j )
                    for( int i = ci; i <= imin( ci + 1, EI ); ++i )
                    {
                        const int64_t idx = findIndex( i, j, k );
                        if( idx == kNull ) continue;
                        const float dx = p.x - ( (float)i + .5f );
                        const float dy = p.y - ( (float)j + .5f );
                        const float dz = p.z - ( (float)k + .5f );
                        const float xw = fmaxr( 0.f, 1.f - absr( dx ) );
                        const float yw = fmaxr( 0.f, 1.f - absr( dy ) );
                        const float zw = fmaxr( 0.f, 1.f - absr( dz ) );
                        const float w = xw * yw * zw + 1e-05f;
                        atomic_add( &mass[(size_t)idx], w );
                        atomic_add( &velo[(size_t)idx].x, w * v.x );
                        atomic_add( &velo[(size_t)idx].y, w * v.y );
                        atomic_add( &velo[(size_t)idx].z, w * v.z );
                    }
        }
        const long long nc = (long long)mass.size();
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < nc; ++n )
        {
            if( mass[(size_t)n] > 0.f )
            {
                const float m = mass[(size_t)n];
                velo[(size_t)n].x /= m;
                velo[(size_t)n].y /= m;
                velo[(size_t)n].z /= m;
            }
            else
            {
                mass[(size_t)n] = 0.f;
                velo[(size_t)n] = V3{ 0.f, 0.f, 0.f };
            }
        }
        // count field
        std::fill( surf.begin(), surf.end(), 0.f );
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < np; ++n )
        {
            const V3 p = pos[(size_t)n];
            if( !inside( p ) ) continue;
            const int ci = imax( (int)( p.x - 0.5f ), 0 );
            const int cj = imax( (int)( p.y - 0.5f ), 0 );
            const int ck = imax( (int)( p.z - 0.5f ), 0 );
            for( int k = ck; k <= imin( ck + 1, EK ); ++k )
                for( int j = cj; j <= imin( cj + 1, EJ ); ++j )
                    for( int i = ci; i <= imin( ci + 1, EI ); ++i )
                    {
                        const int64_t idx = findIndex( i, j, k );
                        if( idx == kNull ) continue;
                        atomic_add( &surf[(size_t)idx], 1.f );
                    }
        }
    }

    // Grid::inside (base/header/Grid.h:408-417)
    inline bool inside( const V3& p ) const
    {
        if( p.x < 0.f ) return false;
        if( p.x > (float)nx ) return false;
        if( p.y < 0.f ) return false;
        if( p.y > (float)ny ) return false;
        if( p.z < 0.f ) return false;
        if( p.z > (float)nz ) return false;
        return true;
    }

    // ---------------------------------------------------------------------------------
    // Cell flags and collider velocity, the lambda in FLIPMethod::advanceOneStep
    // (FLIPMethod.cu:242-281); curl noise is off (enableCurl=false). Cells of an 8^3
    // tile that lie beyond the grid are left at their background values.
    void markCells()
    {
        const long long nc = (long long)mark.size();
        const float cvs = cfg.col_vel_scale;
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < nc; ++n )
        {
            int i, j, k;
            findIndices( (size_t)n, i, j, k );
            if( !real( i, j, k ) ) continue;
            const float cx = (float)i + .5f, cy = (float)j + .5f, cz = (float)k + .5f;
            const float phi = colPhi( cx, cy, cz );
            const V3 v = colVec( cx, cy, cz, BORA_COLLIDER_VELOCITY );
            if( mass[(size_t)n] > 0.f ) mark[(size_t)n] = kFluid;
            else mark[(size_t)n] = phi < 0.f ? kSolid : kAir;
            if( phi < 0.f )
            {
                velo[(size_t)n].x += v.x * cvs;
                velo[(size_t)n].y += v.y * cvs;
                velo[(size_t)n].z += v.z * cvs;
            }
            comp[(size_t)n] = velo[(size_t)n];
        }
    }

    // ---------------------------------------------------------------------------------
    // FluidProjection::buildLinearSystem, sparse (base/source/FluidProjection.cu:165-274)
    void buildSystem()
    {
        fluidCells.clear();
        int64_t count = 0;
        for( size_t n = 0; n < mark.size(); ++n )
        {
            if( mark[n] >= kFluid )
            {
                mark[n] = count + kFluid;
                fluidCells.push_back( (int64_t)n );
                count++;
            }
        }
        const int EI = nx - 1, EJ = ny - 1, EK = nz - 1;
        Avals.assign( (size_t)count * 7, 0.f );
        Acols.assign( (size_t)count * 7, kNull );
        x.assign( (size_t)count, 0.f );
        b.assign( (size_t)count, 0.f );
        const float wallLv = voxelWall;
        const V3 z0{ 0.f, 0.f, 0.f };
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < (long long)count; ++n )
        {
            int i, j, k;
            findIndices( (size_t)fluidCells[(size_t)n], i, j, k );
            const int64_t wall = (float)j + 0.5f <= wallLv + 1.f ? kWall : kAir;
            const int64_t t_cc = at( mark, i, j, k, (int64_t)0 );
            const int64_t t_i0 = i == 0 ? wall : at( mark, i - 1, j, k, (int64_t)0 );
            const int64_t t_i1 = i == EI ? wall : at( mark, i + 1, j, k, (int64_t)0 );
            const int64_t t_j0 = j == 0 ? wall : at( mark, i, j - 1, k, (int64_t)0 );
            const int64_t t_j1 = j == EJ ? wall : at( mark, i, j + 1, k, (int64_t)0 );
            const int64_t t_k0 = k == 0 ? wall : at( mark, i, j, k - 1, (int64_t)0 );
            const int64_t t_k1 = k == EK ? wall : at( mark, i, j, k + 1, (int64_t)0 );
            const V3 v = at( comp, i, j, k, z0 );
            const float i0_j_k = i == 0 ? 2.f * v.x - at( comp, i + 1, j, k, z0 ).x : at( comp, i - 1, j, k, z0 ).x;
            const float i1_j_k = i == EI ? 2.f * v.x - at( comp, i - 1, j, k, z0 ).x : at( comp, i + 1, j, k, z0 ).x;
            const float i_j0_k = j == 0 ? 2.f * v.y - at( comp, i, j + 1, k, z0 ).y : at( comp, i, j - 1, k, z0 ).y;
            const float i_j1_k = j == EJ ? 2.f * v.y - at( comp, i, j - 1, k, z0 ).y : at( comp, i, j + 1, k, z0 ).y;
            const float i_j_k0 = k == 0 ? 2.f * v.z - at( comp, i, j, k + 1, z0 ).z : at( comp, i, j, k - 1, z0 ).z;
            const float i_j_k1 = k == EK ? 2.f * v.z - at( comp, i, j, k - 1, z0 ).z : at( comp, i, j, k + 1, z0 ).z;
            const float v_i0 = t_i0 == kAir ? 2.f * v.x - i1_j_k : t_i0 == kWall ? absr( v.x ) : i0_j_k;
            const float v_i1 = t_i1 == kAir ? 2.f * v.x - i0_j_k : t_i1 == kWall ? -absr( v.x ) : i1_j_k;
            const float v_j0 = t_j0 == kAir ? 2.f * v.y - i_j1_k : t_j0 == kWall ? absr( v.y ) : i_j0_k;
            const float v_j1 = t_j1 == kAir ? 2.f * v.y - i_j0_k : t_j1 == kWall ? -absr( v.y ) : i_j1_k;
            const float v_k0 = t_k0 == kAir ? 2.f * v.z - i_j_k1 : t_k0 == kWall ? absr( v.z ) : i_j_k0;
            const float v_k1 = t_k1 == kAir ? 2.f * v.z - i_j_k0 : t_k1 == kWall ? -absr( v.z ) : i_j_k1;
            float p = 6.f, p_i0 = 0.f, p_i1 = 0.f, p_j0 = 0.f, p_j1 = 0.f, p_k0 = 0.f, p_k1 = 0.f;
            const float d = -( ( v_i1 - v_i0 ) * 0.5f + ( v_j1 - v_j0 ) * 0.5f + ( v_k1 - v_k0 ) * 0.5f );
            auto rule = [&]( int64_t t, float& off ) {
                if( t == kAir ) p += 1.f;
                else if( t == kSolid || t == kWall ) p -= 1.f;
                else if( t >= kFluid ) off -= 1.f;
            };
            rule( t_i0, p_i0 ); rule( t_i1, p_i1 ); rule( t_j0, p_j0 ); rule( t_j1, p_j1 ); rule( t_k0, p_k0 ); rule( t_k1, p_k1 );
            float* vals = &Avals[(size_t)n * 7];
            int64_t* inds = &Acols[(size_t)n * 7];
            vals[0] = p; vals[1] = p_i0; vals[2] = p_i1; vals[3] = p_j0; vals[4] = p_j1; vals[5] = p_k0; vals[6] = p_k1;
            inds[0] = t_cc - kFluid;
            inds[1] = t_i0 >= kFluid ? t_i0 - kFluid : kNull;
            inds[2] = t_i1 >= kFluid ? t_i1 - kFluid : kNull;
            inds[3] = t_j0 >= kFluid ? t_j0 - kFluid : kNull;
            inds[4] = t_j1 >= kFluid ? t_j1 - kFluid : kNull;
            inds[5] = t_k0 >= kFluid ? t_k0 - kFluid : kNull;
            inds[6] = t_k1 >= kFluid ? t_k1 - kFluid : kNull;
            x[(size_t)n] = at( pres, i, j, k, 0.f );
            b[(size_t)n] = d;
        }
    }

    // ---------------------------------------------------------------------------------
    // Linear solve.
    // solver 0: LinearSystemSolver::cg (base/source/LinearSystemSolver.cpp:12-50) with the
    //           BLAS kernels it calls (base/source/BLAS.cu:12-209) in float, sequential
    //           float dot products (thrust::inner_product, BLAS.cu:98-104).
    // solver 1: the same system solved by CG in double to ||r||/||b|| < tol.
    void spmvF( const std::vector<float>& p, std::vector<float>& out, const std::vector<float>* a, bool sub ) const
    {
        const long long rows = (long long)b.size();
#pragma omp parallel for schedule(static)
        for( long long r = 0; r < rows; ++r )
        {
            const float* vals = &Avals[(size_t)r * 7];
            const int64_t* inds = &Acols[(size_t)r * 7];
            float acc = 0.f;
            for( int c = 0; c < 7; ++c )
            {
                const int64_t n = inds[c];
                if( n != kNull ) acc += vals[c] * p[(size_t)n];
            }
            out[(size_t)r] = a ? ( sub ? ( *a )[(size_t)r] - acc : ( *a )[(size_t)r] + acc ) : acc;
        }
    }
    static float dotF( const std::vector<float>& a, const std::vector<float>& c )
    {
        float s = 0.f;
        for( size_t i = 0; i < a.size(); ++i ) s = s + a[i] * c[i];
        return s;
    }
    int solveRef( int max )
    {
        const size_t N = b.size();
        std::vector<float> r( N ), p( N ), Ap( N );
        spmvF( x, r, &b, true );  // submul(b, A, x, r)
        p = r;                    // equ(r, p)
        float rsold = dotF( r, r );
        if( std::sqrt( rsold ) < 1e-30f ) return 0;
        const int iter = (int)N;
        int count = 0;
        for( int i = 0; i < iter + 5; ++i, ++count )
        {
            spmvF( p, Ap, nullptr, false );
            const float alpha = rsold / dotF( p, Ap );
            axpyF( x, alpha, p, x );   // BLAS::axpy (BLAS.cu:142-150) as a parallel loop, like
            axpyF( r, -alpha, Ap, r ); // the reference's LaunchCudaDevice; element-wise, so the
            const float rsnew = dotF( r, r );  // result does not depend on the thread count
            if( std::sqrt( rsnew ) < 1e-3f ) break;
            const float beta = rsnew / rsold;
            axpyF( r, beta, p, p );
            rsold = rsnew;
            if( count > max ) break;
        }
        return count;
    }
    // out = a + s * c element-wise in float (r - alpha*Ap is written a + (-alpha)*c: IEEE
    // negation is exact, so it rounds like a - alpha*c)
    static void axpyF( const std::vector<float>& a, float s_, const std::vector<float>& c, std::vector<float>& out )
    {
        const long long n = (long long)a.size();
#pragma omp parallel for schedule(static)
        for( long long i = 0; i < n; ++i ) out[(size_t)i] = a[(size_t)i] + ( s_ * c[(size_t)i] );
    }
    static double dotFD( const std::vector<float>& a, const std::vector<float>& c )
    {
        double s_ = 0.0;
        const long long n = (long long)a.size();
#pragma omp parallel for reduction(+ : s_) schedule(static)
        for( long long i = 0; i < n; ++i ) s_ += (double)a[(size_t)i] * (double)c[(size_t)i];
        return s_;
    }
    // The like-for-like CPU baseline of a converged solve: LinearSystemSolver::cg's FP32
    // recurrence (LinearSystemSolver.cpp:12-50) with its dots in FP64 and its stop rule
    // replaced by ||r||/||b|| < tol on the recursive residual, no 201-iteration cap.
    int solveTol( double tol, int maxit )
    {
        const size_t N = b.size();
        std::vector<float> r( N ), p( N ), Ap( N );
        spmvF( x, r, &b, true );
        p = r;
        const double bn = std::sqrt( dotFD( b, b ) );
        double rsold = dotFD( r, r );
        int it = 0;
        if( bn > 0.0 )
        {
            while( std::sqrt( rsold ) > tol * bn && it < maxit )
            {
                spmvF( p, Ap, nullptr, false );
                const float alpha = (float)( rsold / dotFD( p, Ap ) );
                axpyF( x, alpha, p, x );
                axpyF( r, -alpha, Ap, r );
                const double rsnew = dotFD( r, r );
                const float beta = (float)( rsnew / rsold );
                axpyF( r, beta, p, p );
                rsold = rsnew;
                ++it;
            }
        }
        lastRel = bn > 0.0 ? std::sqrt( rsold ) / bn : 0.0;
        return it;
    }
    void spmvD( const std::vector<double>& p, std::vector<double>& out ) const
    {
        const long long rows = (long long)b.size();
#pragma omp parallel for schedule(static)
        for( long long r = 0; r < rows; ++r )
        {
            const float* vals = &Avals[(size_t)r * 7];
            const int64_t* inds = &Acols[(size_t)r * 7];
            double acc = 0.0;
            for( int c = 0; c < 7; ++c )
            {
                const int64_t n = inds[c];
                if( n != kNull ) acc += (double)vals[c] * p[(size_t)n];
            }
            out[(size_t)r] = acc;
        }
    }
    static double dotD( const std::vector<double>& a, const std::vector<double>& c )
    {
        double s = 0.0;
        const long long n = (long long)a.size();
#pragma omp parallel for reduction(+ : s) schedule(static)
        for( long long i = 0; i < n; ++i ) s += a[(size_t)i] * c[(size_t)i];
        return s;
    }
    int solve64( double tol, int maxit )
    {
        const size_t N = b.size();
        std::vector<double> X( N ), Bv( N ), R( N ), P( N ), Q( N );
        for( size_t i = 0; i < N; ++i ) { X[i] = x[i]; Bv[i] = b[i]; }
        spmvD( X, Q );
        for( size_t i = 0; i < N; ++i ) { R[i] = Bv[i] - Q[i]; P[i] = R[i]; }
        const double bn = std::sqrt( dotD( Bv, Bv ) );
        double rs = dotD( R, R );
        int it = 0;
        if( bn > 0.0 )
        {
            while( std::sqrt( rs ) > tol * bn && it < maxit )
            {
                spmvD( P, Q );
                const double alpha = rs / dotD( P, Q );
                const long long n = (long long)N;
#pragma omp parallel for schedule(static)
                for( long long i = 0; i < n; ++i ) { X[(size_t)i] += alpha * P[(size_t)i]; R[(size_t)i] -= alpha * Q[(size_t)i]; }
                const double rn = dotD( R, R );
                const double beta = rn / rs;
#pragma omp parallel for schedule(static)
                for( long long i = 0; i < n; ++i ) P[(size_t)i] = R[(size_t)i] + beta * P[(size_t)i];
                rs = rn;
                ++it;
            }
        }
        for( size_t i = 0; i < N; ++i ) x[i] = (float)X[i];
        lastRel = bn > 0.0 ? std::sqrt( rs ) / bn : 0.0;
        return it;
    }
    int solve()
    {
        if( cfg.solver == 0 ) lastIters = solveRef( cfg.max_iter );
        else if( cfg.solver == 2 ) lastIters = solveTol( cfg.tol, cfg.max_iter );
        else lastIters = solve64( cfg.tol, cfg.max_iter );
        return lastIters;
    }

    // ---------------------------------------------------------------------------------
    // FluidProjection::solve after the solver (FluidProjection.cu:291-378): scatter the
    // pressure, give air cells next to fluid the mean of their fluid neighbours, then
    // subtract the central-difference pressure gradient with the ghost rules.
    void updateVelocity()
    {
        const long long nu = (long long)fluidCells.size();
        for( long long n = 0; n < nu; ++n )
        {
            const size_t idx = (size_t)fluidCells[(size_t)n];
            pres[idx] = x[(size_t)( mark[idx] - kFluid )];
        }
        const int EI = nx - 1, EJ = ny - 1, EK = nz - 1;
        const long long nc = (long long)mark.size();
        auto isF = [&]( int i, int j, int k ) { return at( mark, i, j, k, (int64_t)0 ) >= kFluid; };
        auto P = [&]( int i, int j, int k ) { return at( pres, i, j, k, 0.f ); };
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < nc; ++n )
        {
            if( mark[(size_t)n] != kAir ) continue;
            int i, j, k;
            findIndices( (size_t)n, i, j, k );
            if( !real( i, j, k ) ) continue;
            float press = 0.f;
            int count = 0;
            if( i > 0 && isF( i - 1, j, k ) ) { press += P( i - 1, j, k ); count++; }
            if( i < EI && isF( i + 1, j, k ) ) { press += P( i + 1, j, k ); count++; }
            if( j > 0 && isF( i, j - 1, k ) ) { press += P( i, j - 1, k ); count++; }
            if( j < EJ && isF( i, j + 1, k ) ) { press += P( i, j + 1, k ); count++; }
            if( k > 0 && isF( i, j, k - 1 ) ) { press += P( i, j, k - 1 ); count++; }
            if( k < EK && isF( i, j, k + 1 ) ) { press += P( i, j, k + 1 ); count++; }
            if( count > 0 ) pres[(size_t)n] = press / (float)count;
        }
        const float wallLv = voxelWall;
#pragma omp parallel for schedule(static)
        for( long long t = 0; t < nu; ++t )
        {
            const size_t n = (size_t)fluidCells[(size_t)t];
            int i, j, k;
            findIndices( n, i, j, k );
            const int64_t wall = (float)j + 0.5f <= wallLv + 1.f ? kSolid : kAir;
            const float p = pres[n];
            const int64_t t_i0 = i == 0 ? wall : at( mark, i - 1, j, k, (int64_t)0 );
            const int64_t t_i1 = i == EI ? wall : at( mark, i + 1, j, k, (int64_t)0 );
            const int64_t t_j0 = j == 0 ? wall : at( mark, i, j - 1, k, (int64_t)0 );
            const int64_t t_j1 = j == EJ ? wall : at( mark, i, j + 1, k, (int64_t)0 );
            const int64_t t_k0 = k == 0 ? wall : at( mark, i, j, k - 1, (int64_t)0 );
            const int64_t t_k1 = k == EK ? wall : at( mark, i, j, k + 1, (int64_t)0 );
            const float i0_j_k = i == 0 ? 2.f * p - P( i + 1, j, k ) : P( i - 1, j, k );
            const float i1_j_k = i == EI ? 2.f * p - P( i - 1, j, k ) : P( i + 1, j, k );
            const float i_j0_k = j == 0 ? 2.f * p - P( i, j + 1, k ) : P( i, j - 1, k );
            const float i_j1_k = j == EJ ? 2.f * p - P( i, j - 1, k ) : P( i, j + 1, k );
            const float i_j_k0 = k == 0 ? 2.f * p - P( i, j, k + 1 ) : P( i, j, k - 1 );
            const float i_j_k1 = k == EK ? 2.f * p - P( i, j, k - 1 ) : P( i, j, k + 1 );
            const float p_i0 = t_i0 == kSolid ? 2.f * p - i1_j_k : t_i0 == kAir ? -i0_j_k : i0_j_k;
            const float p_i1 = t_i1 == kSolid ? 2.f * p - i0_j_k : t_i1 == kAir ? -i1_j_k : i1_j_k;
            const float p_j0 = t_j0 == kSolid ? 2.f * p - i_j1_k : t_j0 == kAir ? -i_j0_k : i_j0_k;
            const float p_j1 = t_j1 == kSolid ? 2.f * p - i_j0_k : t_j1 == kAir ? -i_j1_k : i_j1_k;
            const float p_k0 = t_k0 == kSolid ? 2.f * p - i_j_k1 : t_k0 == kAir ? -i_j_k0 : i_j_k0;
            const float p_k1 = t_k1 == kSolid ? 2.f * p - i_j_k0 : t_k1 == kAir ? -i_j_k1 : i_j_k1;
            comp[n].x -= ( p_i1 - p_i0 ) * 0.5f;
            comp[n].y -= ( p_j1 - p_j0 ) * 0.5f;
            comp[n].z -= ( p_k1 - p_k0 ) * 0.5f;
        }
    }

    // ---------------------------------------------------------------------------------
    // FLIPMethod::updateParticles (base/source/FLIPMethod.cu:54-175): G2P with the
    // FLIP/PIC blend, tank damping, collider carry, Euler advection substeps with the
    // box clamp and collider push-out, kill flags, then gravity.
    void updateParticles( float dt )
    {
        const float lx = (float)nx + 0.5f, lz = (float)nz + 0.5f;
        const bool enableTank = cfg.enable_tank != 0;
        const float band = cfg.damping_band / cfg.voxel_size;
        const float wall = voxelWall;
        const V3 ef = voxelForce;
        const int maxsub = cfg.maxsubsteps;
        const long long np = (long long)pos.size();
        removed.assign( (size_t)np, 0 );
        adj.resize( (size_t)np );
#pragma omp parallel for schedule(static)
        for( long long ix = 0; ix < np; ++ix )
        {
            V3 p = pos[(size_t)ix];
            V3 v = vel[(size_t)ix];
            adj[(size_t)ix] = lerpMinS( surf, surfBackground, p.x, p.y, p.z );
            {
                const V3 g = lerpV( comp, p.x, p.y, p.z );
                const V3 o = lerpV( velo, p.x, p.y, p.z );
                const V3 f{ g.x - o.x, g.y - o.y, g.z - o.z };
                v.x += f.x; v.y += f.y; v.z += f.z;
                v = V3{ v.x * 0.95f + g.x * 0.05f, v.y * 0.95f + g.y * 0.05f, v.z * 0.95f + g.z * 0.05f };
            }
            if( enableTank && p.y <= wall )
            {
                float w = 1.f;
                if( p.x < band ) w = fminr( w, clampf( ( p.x - 0.f ) / band, 0.f, 1.f ) );
                if( p.x > lx - band ) w = fminr( w, clampf( ( lx - p.x ) / band, 0.f, 1.f ) );
                if( p.z < band ) w = fminr( w, clampf( ( p.z - 0.f ) / band, 0.f, 1.f ) );
                if( p.z > lz - band ) w = fminr( w, clampf( ( lz - p.z ) / band, 0.f, 1.f ) );
                v.x *= w; v.y *= w; v.z *= w;
            }
            if( colPhi( p.x, p.y, p.z ) < 0.f )
            {
                const V3 cv = colVec( p.x, p.y, p.z, BORA_COLLIDER_VELOCITY );
                p.x += cv.x * dt; p.y += cv.y * dt; p.z += cv.z * dt;
            }
            {
                const float len = std::sqrt( v.x * v.x + v.y * v.y + v.z * v.z );
                const int iter = 1 + imin( (int)( len * dt * 1.5f ), imax( maxsub, 1 ) );
                const float sub_dt = dt / (float)iter;
                bool col = false;
                for( int s = 0; s < iter; ++s )
                {
                    if( cfg.advection == 1 )
                    {
                        // RK2 (midpoint) in the projected grid velocity: an option of this
                        // build, not of the reference, restated here with the same lerp.
                        const float h = 0.5f * sub_dt;
                        const V3 k1 = lerpV( comp, p.x, p.y, p.z );
                        const V3 k2 = lerpV( comp, p.x + k1.x * h, p.y + k1.y * h, p.z + k1.z * h );
                        p.x += k2.x * sub_dt; p.y += k2.y * sub_dt; p.z += k2.z * sub_dt;
                    }
                    else
                    {
                        p.x += v.x * sub_dt; p.y += v.y * sub_dt; p.z += v.z * sub_dt;
                    }
                    if( p.y <= wall )
                    {
                        if( p.x < 0.f ) { p.x = 0.f; if( v.x < 0.f ) v.x = 0.f; }
                        if( p.y < 0.f ) { p.y = 0.f; if( v.y < 0.f ) v.y = 0.f; }
                        if( p.z < 0.f ) { p.z = 0.f; if( v.z < 0.f ) v.z = 0.f; }
                        if( p.x > (float)nx ) { p.x = (float)nx; if( v.x > 0.f ) v.x = 0.f; }
                        if( p.y > (float)ny ) { p.y = (float)ny; if( v.y > 0.f ) v.y = 0.f; }
                        if( p.z > (float)nz ) { p.z = (float)nz; if( v.z > 0.f ) v.z = 0.f; }
                    }
                    const float phi = colPhi( p.x, p.y, p.z );
                    if( phi < 0.f )
                    {
                        const V3 nr = colVec( p.x, p.y, p.z, BORA_COLLIDER_NORMAL );
                        // Vec3f::normalized (base/header/Vector3.h:350-354)
                        const double dn = 1.0f / std::sqrt( nr.x * nr.x + nr.y * nr.y + nr.z * nr.z + 1e-30f );
                        const float ux = (float)( nr.x * dn ), uy = (float)( nr.y * dn ), uz = (float)( nr.z * dn );
                        p.x -= ux * phi; p.y -= uy * phi; p.z -= uz * phi;
                        col = true;
                    }
                }
                if( col )
                {
                    const float phi = colPhi( p.x, p.y, p.z );
                    if( phi > 3.f || phi < 0.f ) removed[(size_t)ix] = 1;
                }
                if( !inside( p ) ) removed[(size_t)ix] = 1;
            }
            v.x += ef.x * dt; v.y += ef.y * dt; v.z += ef.z * dt;
            pos[(size_t)ix] = p;
            vel[(size_t)ix] = v;
        }
    }

    // ---------------------------------------------------------------------------------
    // Array::remove (base/header/Array.h:996-1024) on every particle attribute: each
    // killed slot below the new size takes the last surviving particle above it.
    template <class T> static void removeMasked( std::vector<T>& a, const std::vector<uint8_t>& m )
    {
        const size_t size = a.size();
        if( size == 0 ) return;
        size_t end = size - 1, del = 0;
        for( size_t n = 0; n < m.size(); ++n )
        {
            if( n >= size ) break;
            if( m[n] )
            {
                del++;
                for( size_t q = end; q >= n + 1; --q )
                {
                    if( m[q] == 0 ) { a[n] = a[q]; end = q - 1; break; }
                }
            }
        }
        a.resize( size - del );
    }
    void compact()
    {
        removeMasked( pos, removed );
        removeMasked( vel, removed );
        removeMasked( adj, removed );
        removeMasked( pid, removed );
        removeMasked( vort, removed );
        removeMasked( curv, removed );
    }

    // =================================================================================
    // FLIPMethod::postProcess (base/source/FLIPMethod.cu:300-405): the surface pipeline
    // that follows the step in FLIPMethod::advanceOneFrame. The particle attributes
    // Particles::vorticity / ::curvature (base/header/Particles.h:28) ride along with the
    // particles through compact(). Cells of an 8^3 tile beyond the grid are skipped (the
    // reference's 4^3 tiles never extend past its grid).
    std::vector<float> vort, curv;
    float presBackground = 0.f;

    // Rasterization::ParticlesToSurfaceAndVelocity (base/source/Rasterization.cu:311-398)
    // with influence 1.5 and droplet radius 0.5 (FLIPMethod.cu:320): weights
    // max(0, (1 - (d/1.5)^2)^3) over the 3^3 cells around the particle's cell
    // (Grid::neighborCells, base/header/Grid.h:353-370), accumulated in particle order
    // into pres/velo (FLIPMethod.cu:320 passes _sPresField as the mass field) and
    // surf/comp (the weighted position); then surf = distance from the weighted mean
    // position to the cell centre - 0.5 (5 where nothing landed) and velo = weighted mean
    // velocity.
    void splatSurface()
    {
        std::fill( surf.begin(), surf.end(), 0.f );
        std::fill( pres.begin(), pres.end(), 0.f );
        std::fill( comp.begin(), comp.end(), V3{ 0.f, 0.f, 0.f } );
        std::fill( velo.begin(), velo.end(), V3{ 0.f, 0.f, 0.f } );
        const float h = 1.5f, r = 0.5f;
        for( size_t n = 0; n < pos.size(); ++n )
        {
            const V3 p = pos[n], v = vel[n];
            if( !inside( p ) ) continue;
            const int i0 = clampi( (int)p.x - 1, 0, nx - 1 ), i1 = clampi( (int)p.x + 1, 0, nx - 1 );
            const int j0 = clampi( (int)p.y - 1, 0, ny - 1 ), j1 = clampi( (int)p.y + 1, 0, ny - 1 );
            const int k0 = clampi( (int)p.z - 1, 0, nz - 1 ), k1 = clampi( (int)p.z + 1, 0, nz - 1 );
            for( int k = k0; k <= k1; ++k )
                for( int j = j0; j <= j1; ++j )
                    for( int i = i0; i <= i1; ++i )
                    {
                        const float dx = p.x - ( (float)i + .5f ), dy = p.y - ( (float)j + .5f ), dz = p.z - ( (float)k + .5f );
                        const float dist = std::sqrt( dx * dx + dy * dy + dz * dz );  // Vec3f::length (Vector3.h:328-331)
                        const float s = dist / h;
                        const float t = 1.f - s * s;
                        const float w = fmaxr( 0.f, t * t * t );
                        const int64_t q = findIndex( i, j, k );
                        if( q == kNull ) continue;
                        pres[(size_t)q] += w;
                        velo[(size_t)q].x += w * v.x; velo[(size_t)q].y += w * v.y; velo[(size_t)q].z += w * v.z;
                        surf[(size_t)q] += w;
                        comp[(size_t)q].x += w * p.x; comp[(size_t)q].y += w * p.y; comp[(size_t)q].z += w * p.z;
                    }
        }
        surfBackground = 10.f;
        for( size_t n = 0; n < surf.size(); ++n )
        {
            int i, j, k;
            findIndices( n, i, j, k );
            if( surf[n] > 1e-30f )
            {
                comp[n].x /= surf[n]; comp[n].y /= surf[n]; comp[n].z /= surf[n];
                const float dx = comp[n].x - ( (float)i + .5f ), dy = comp[n].y - ( (float)j + .5f ),
                            dz = comp[n].z - ( (float)k + .5f );
                surf[n] = std::sqrt( dx * dx + dy * dy + dz * dz ) - r;  // Vec3f::distanceTo (Vector3.h:364-367)
            }
            else
            {
                surf[n] = 5.f;
            }
            if( pres[n] > 1e-30f )
            {
                velo[n].x /= pres[n]; velo[n].y /= pres[n]; velo[n].z /= pres[n];
            }
            else
            {
                velo[n] = V3{ 0.f, 0.f, 0.f };
            }
        }
    }

    // The water-tank scan (FLIPMethod.cu:322-366): a depth-first fill from the corner
    // cell (nx-1, ny-1, nz-1) and from every air cell (surf > 0; inactive tiles read the
    // background 10) of the layer j = wall, through air cells, expanding only cells at or
    // below the wall; air cells at or below the wall that it does not reach become liquid
    // (surf = -5). literal = true restates the loop as the reference executes it: the
    // popped cell is read through a reference to the stack's last element
    // (FLIPMethod.cu:335-337), and the iteration's first push_back constructs the new cell
    // in that same slot, so the remaining neighbour tests of the iteration are made around
    // the first pushed cell instead. literal = false is the 6-connected fill that the loop
    // describes (the device path's rule). A negative wall level skips the scan (the
    // reference converts it to size_t, which is undefined), and with the wall at or above
    // the grid top only the corner seeds it (the reference would read past its tile table).
    void tankScan( bool literal )
    {
        if( !cfg.enable_tank || voxelWall < 0.f ) return;
        const size_t wall = (size_t)voxelWall;
        std::vector<uint8_t> scan( (size_t)nx * ny * nz, 0 );
        auto S = [&]( int i, int j, int k ) { return at( surf, i, j, k, surfBackground ); };
        auto sc = [&]( int i, int j, int k ) -> uint8_t& { return scan[( (size_t)k * ny + j ) * nx + i]; };
        struct C3 { int i, j, k; };
        std::vector<C3> cells;
        cells.reserve( (size_t)nx * nz );
        cells.push_back( C3{ nx - 1, ny - 1, nz - 1 } );
        if( wall < (size_t)ny )
            for( int k = 0; k < nz; ++k )
                for( int i = 0; i < nx; ++i )
                    if( S( i, (int)wall, k ) > 0.f ) cells.push_back( C3{ i, (int)wall, k } );
        while( !cells.empty() )
        {
            C3 c = cells.back();
            cells.pop_back();
            sc( c.i, c.j, c.k ) = 1;
            if( (size_t)c.j > wall ) continue;
            bool first = true;
            auto push = [&]( C3 q ) {
                cells.push_back( q );
                if( literal && first ) c = q;
                first = false;
            };
            if( c.i - 1 >= 0 && S( c.i - 1, c.j, c.k ) > 0.f && sc( c.i - 1, c.j, c.k ) == 0 ) push( C3{ c.i - 1, c.j, c.k } );
            if( c.i + 1 < nx && S( c.i + 1, c.j, c.k ) > 0.f && sc( c.i + 1, c.j, c.k ) == 0 ) push( C3{ c.i + 1, c.j, c.k } );
            if( c.j - 1 >= 0 && S( c.i, c.j - 1, c.k ) > 0.f && sc( c.i, c.j - 1, c.k ) == 0 ) push( C3{ c.i, c.j - 1, c.k } );
            if( c.j + 1 < ny && S( c.i, c.j + 1, c.k ) > 0.f && sc( c.i, c.j + 1, c.k ) == 0 ) push( C3{ c.i, c.j + 1, c.k } );
            if( c.k - 1 >= 0 && S( c.i, c.j, c.k - 1 ) > 0.f && sc( c.i, c.j, c.k - 1 ) == 0 ) push( C3{ c.i, c.j, c.k - 1 } );
            if( c.k + 1 < nz && S( c.i, c.j, c.k + 1 ) > 0.f && sc( c.i, c.j, c.k + 1 ) == 0 ) push( C3{ c.i, c.j, c.k + 1 } );
        }
        for( size_t n = 0; n < surf.size(); ++n )
        {
            int i, j, k;
            findIndices( n, i, j, k );
            if( !real( i, j, k ) || (size_t)j > wall ) continue;
            if( surf[n] > 0.f && sc( i, j, k ) == 0 ) surf[n] = -5.f;
        }
    }

    // Rasterization::ReinitializeSurface (base/source/Rasterization.cu:400-486): `iters`
    // Godunov upwind steps (dt 0.3) of phi_t = sign(phi0)(1 - |grad phi|) with
    // sign = phi / sqrt(phi^2 + 1); differences are mirrored at the grid faces, or, for
    // the water tank, the faces read the level y - wall (-1 / +1 below / above). surf and
    // pres swap after each step, as the reference swaps the two fields' storage.
    void redistance( int iters )
    {
        const int I = nx - 1, J = ny - 1, K = nz - 1;
        const float dt = 0.3f;
        surfBackground = 10.f;
        presBackground = 10.f;
        const bool tank = cfg.enable_tank != 0;
        const float level = voxelWall;
        const long long nc = (long long)surf.size();
        for( int it = 0; it < iters; ++it )
        {
#pragma omp parallel for schedule(static)
            for( long long n = 0; n < nc; ++n )
            {
                int i, j, k;
                findIndices( (size_t)n, i, j, k );
                const float v = surf[(size_t)n];
                if( !real( i, j, k ) ) { pres[(size_t)n] = v; continue; }
                auto S = [&]( int a, int b, int c ) { return at( surf, a, b, c, 10.f ); };
                float vi0, vi1, vj0, vj1, vk0, vk1;
                if( tank )
                {
                    const float ll = ( (float)j + .5f ) - level;
                    vj0 = j == 0 ? ll - 1.f : S( i, j - 1, k );
                    vj1 = j == J ? ll + 1.f : S( i, j + 1, k );
                    vi0 = i == 0 ? ll : S( i - 1, j, k );
                    vi1 = i == I ? ll : S( i + 1, j, k );
                    vk0 = k == 0 ? ll : S( i, j, k - 1 );
                    vk1 = k == K ? ll : S( i, j, k + 1 );
                }
                else
                {
                    vi0 = i == 0 ? 2.f * v - S( i + 1, j, k ) : S( i - 1, j, k );
                    vi1 = i == I ? 2.f * v - S( i - 1, j, k ) : S( i + 1, j, k );
                    vj0 = j == 0 ? 2.f * v - S( i, j + 1, k ) : S( i, j - 1, k );
                    vj1 = j == J ? 2.f * v - S( i, j - 1, k ) : S( i, j + 1, k );
                    vk0 = k == 0 ? 2.f * v - S( i, j, k + 1 ) : S( i, j, k - 1 );
                    vk1 = k == K ? 2.f * v - S( i, j, k - 1 ) : S( i, j, k + 1 );
                }
                const float dx0 = v - vi0, dx1 = vi1 - v, dy0 = v - vj0, dy1 = vj1 - v, dz0 = v - vk0, dz1 = vk1 - v;
                auto sq = []( float x ) { return x * x; };
                const float a = sq( fmaxr( dx0, 0.f ) ) + sq( fminr( dx1, 0.f ) ) + sq( fmaxr( dy0, 0.f ) ) +
                                sq( fminr( dy1, 0.f ) ) + sq( fmaxr( dz0, 0.f ) ) + sq( fminr( dz1, 0.f ) );
                const float b = sq( fminr( dx0, 0.f ) ) + sq( fmaxr( dx1, 0.f ) ) + sq( fminr( dy0, 0.f ) ) +
                                sq( fmaxr( dy1, 0.f ) ) + sq( fminr( dz0, 0.f ) ) + sq( fmaxr( dz1, 0.f ) );
                const float sign = v / std::sqrt( v * v + 1.f );
                pres[(size_t)n] = ( v - dt * fmaxr( sign, 0.f ) * ( std::sqrt( a ) - 1.f ) ) -
                                  dt * fminr( sign, 0.f ) * ( std::sqrt( b ) - 1.f );
            }
            std::swap( surf, pres );
        }
    }

    // FieldOP::curl, sparse (base/source/FieldOP.cu:338-369): central differences of velo
    // (background 0), mirrored at the grid faces, into comp.
    void curlToComp()
    {
        const int I = nx - 1, J = ny - 1, K = nz - 1;
        const V3 bg{ 0.f, 0.f, 0.f };
        const long long nc = (long long)velo.size();
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < nc; ++n )
        {
            int i, j, k;
            findIndices( (size_t)n, i, j, k );
            if( !real( i, j, k ) ) continue;
            const V3 v = velo[(size_t)n];
            auto F = [&]( int a, int b, int c ) { return at( velo, a, b, c, bg ); };
            auto mir = [&]( V3 o ) { return V3{ v.x * 2.f - o.x, v.y * 2.f - o.y, v.z * 2.f - o.z }; };
            const V3 x0 = i == 0 ? mir( F( i + 1, j, k ) ) : F( i - 1, j, k );
            const V3 x1 = i == I ? mir( F( i - 1, j, k ) ) : F( i + 1, j, k );
            const V3 y0 = j == 0 ? mir( F( i, j + 1, k ) ) : F( i, j - 1, k );
            const V3 y1 = j == J ? mir( F( i, j - 1, k ) ) : F( i, j + 1, k );
            const V3 z0 = k == 0 ? mir( F( i, j, k + 1 ) ) : F( i, j, k - 1 );
            const V3 z1 = k == K ? mir( F( i, j, k - 1 ) ) : F( i, j, k + 1 );
            comp[(size_t)n] = V3{ ( y1.z - y0.z ) * 0.5f - ( z1.y - z0.y ) * 0.5f, ( z1.x - z0.x ) * 0.5f - ( x1.z - x0.z ) * 0.5f,
                                  ( x1.y - x0.y ) * 0.5f - ( y1.x - y0.x ) * 0.5f };
        }
    }

    // FieldOP::normalGradient, sparse (FieldOP.cu:79-110): central differences of surf
    // (background 10), mirrored at the faces, normalised (Vec3f::normalized,
    // base/header/Vector3.h:350-354), into comp.
    void normalToComp()
    {
        const int I = nx - 1, J = ny - 1, K = nz - 1;
        const long long nc = (long long)surf.size();
        const float bg = surfBackground;
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < nc; ++n )
        {
            int i, j, k;
            findIndices( (size_t)n, i, j, k );
            if( !real( i, j, k ) ) continue;
            const float v = surf[(size_t)n];
            auto S = [&]( int a, int b, int c ) { return at( surf, a, b, c, bg ); };
            const float vi0 = i == 0 ? 2.f * v - S( i + 1, j, k ) : S( i - 1, j, k );
            const float vi1 = i == I ? 2.f * v - S( i - 1, j, k ) : S( i + 1, j, k );
            const float vj0 = j == 0 ? 2.f * v - S( i, j + 1, k ) : S( i, j - 1, k );
            const float vj1 = j == J ? 2.f * v - S( i, j - 1, k ) : S( i, j + 1, k );
            const float vk0 = k == 0 ? 2.f * v - S( i, j, k + 1 ) : S( i, j, k - 1 );
            const float vk1 = k == K ? 2.f * v - S( i, j, k - 1 ) : S( i, j, k + 1 );
            const float gx = ( vi1 - vi0 ) * 0.5f, gy = ( vj1 - vj0 ) * 0.5f, gz = ( vk1 - vk0 ) * 0.5f;
            const float d = 1.f / std::sqrt( gx * gx + gy * gy + gz * gz + 1e-30f );
            comp[(size_t)n] = V3{ gx * d, gy * d, gz * d };
        }
    }

    // FieldOP::curvature of a vector field, sparse (FieldOP.cu:273-301): divergence of
    // comp (background 0) by central differences mirrored at the faces, into pres.
    void curvatureToPres()
    {
        const int I = nx - 1, J = ny - 1, K = nz - 1;
        const V3 bg{ 0.f, 0.f, 0.f };
        const long long nc = (long long)comp.size();
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < nc; ++n )
        {
            int i, j, k;
            findIndices( (size_t)n, i, j, k );
            if( !real( i, j, k ) ) continue;
            const V3 s = comp[(size_t)n];
            auto N = [&]( int a, int b, int c ) { return at( comp, a, b, c, bg ); };
            const float si0 = i == 0 ? s.x * 2.f - N( i + 1, j, k ).x : N( i - 1, j, k ).x;
            const float si1 = i == I ? s.x * 2.f - N( i - 1, j, k ).x : N( i + 1, j, k ).x;
            const float sj0 = j == 0 ? s.y * 2.f - N( i, j + 1, k ).y : N( i, j - 1, k ).y;
            const float sj1 = j == J ? s.y * 2.f - N( i, j - 1, k ).y : N( i, j + 1, k ).y;
            const float sk0 = k == 0 ? s.z * 2.f - N( i, j, k + 1 ).z : N( i, j, k - 1 ).z;
            const float sk1 = k == K ? s.z * 2.f - N( i, j, k - 1 ).z : N( i, j, k + 1 ).z;
            pres[(size_t)n] = ( si1 - si0 ) * 0.5f + ( sj1 - sj0 ) * 0.5f + ( sk1 - sk0 ) * 0.5f;
        }
    }

    // FLIPMethod.cu:370-404: curl -> per-particle vorticity (decayed by
    // (1 - vortPresRate)^dt, the larger of that and |world curl| - 0.2 kept), normal
    // gradient -> curvature -> per-particle curvature (pres background 10 here, as
    // ReinitializeSurface left it), then pres cleared to 0 with background 0.
    void particleAttributes( float dt, float vort_pres_rate )
    {
        if( vort.size() != pos.size() ) vort.resize( pos.size(), 0.f );
        if( curv.size() != pos.size() ) curv.resize( pos.size(), 0.f );
        curlToComp();
        const float dis = powf( 1.f - vort_pres_rate, dt );
        const long long np = (long long)pos.size();
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < np; ++n )
        {
            const V3 p = pos[(size_t)n];
            const V3 c = lerpV( comp, p.x, p.y, p.z );
            const float wx = c.x * scale[0], wy = c.y * scale[1], wz = c.z * scale[2];  // Grid::worldVector
            float v = std::sqrt( wx * wx + wy * wy + wz * wz );
            v = fmaxr( 0.f, v - 0.2f );
            float& q = vort[(size_t)n];
            q -= q * dis;
            q = fmaxr( v, q );
        }
        normalToComp();
        curvatureToPres();
#pragma omp parallel for schedule(static)
        for( long long n = 0; n < np; ++n )
        {
            const V3 p = pos[(size_t)n];
            curv[(size_t)n] = lerpS( pres, presBackground, p.x, p.y, p.z );
        }
        std::fill( pres.begin(), pres.end(), 0.f );
        presBackground = 0.f;
    }

    void postProcess( float dt, float vort_pres_rate, int redist_iteration, bool literal_scan )
    {
        rebuild();  // FLIPMethod::prepareNextStep
        splatSurface();
        tankScan( literal_scan );
        redistance( redist_iteration );
        particleAttributes( dt, vort_pres_rate );
    }

    int step( float dt )
    {
        if( pos.empty() ) return 0;
        rebuild();
        p2g();
        markCells();
        buildSystem();
        const int it = solve();
        updateVelocity();
        updateParticles( dt );
        compact();
        return it;
    }
};

extern "C" {

void* ora_create( const OracleConfig* c )
{
    Oracle* o = new Oracle();
    o->initialize( *c );
    return o;
}

void ora_destroy( void* h ) { delete (Oracle*)h; }

void ora_set_threads( int n ) { if( n > 0 ) omp_set_num_threads( n ); }
int ora_get_threads() { return omp_get_max_threads(); }

// CollisionSource::update (CollisionSource.h:66-126) from a level set's active voxels
// (frame cells ijk, phi in world units, velocities in world units per second or NULL, the
// level set's background): SparseFrame::buildFromPoints's rule - a tile is the collider's
// when an active voxel lies in it or in one of its 26 neighbours, here over 8^3 tiles - and
// samples phi / h, v / scale at the voxels, background / h on the collider's other cells.
void ora_set_collider_voxels( void* h, const int32_t* ijk, const float* phi, const float* vel, size_t count,
                              float background )
{
    Oracle* o = (Oracle*)h;
    std::memset( &o->cols, 0, sizeof( o->cols ) );
    o->col_tslot.clear();
    o->col_tphi.clear();
    o->col_tvel.clear();
    if( count == 0 ) return;
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    const int tx = ( nx + 7 ) / 8, ty = ( ny + 7 ) / 8, tz = ( nz + 7 ) / 8;
    const size_t ntv = (size_t)tx * ty * tz;
    auto lin = [&]( int a, int b, int d ) { return (size_t)a + (size_t)tx * ( (size_t)b + (size_t)ty * d ); };
    std::vector<uint8_t> hit( ntv, 0 );
    for( size_t v = 0; v < count; ++v )
    {
        const int i = ijk[3 * v], j = ijk[3 * v + 1], k = ijk[3 * v + 2];
        if( i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz ) continue;
        hit[lin( i / 8, j / 8, k / 8 )] = 1;
    }
    o->col_tslot.assign( ntv, -1 );
    int nslots = 0;
    for( int d = 0; d < tz; ++d )
        for( int b = 0; b < ty; ++b )
            for( int a = 0; a < tx; ++a )
            {
                bool any = false;
                for( int dd = d - 1; dd <= d + 1 && !any; ++dd )
                    for( int bb = b - 1; bb <= b + 1 && !any; ++bb )
                        for( int aa = a - 1; aa <= a + 1 && !any; ++aa )
                            if( aa >= 0 && bb >= 0 && dd >= 0 && aa < tx && bb < ty && dd < tz && hit[lin( aa, bb, dd )] )
                                any = true;
                if( any ) o->col_tslot[lin( a, b, d )] = nslots++;
            }
    const float hsz = o->scale[0];
    const float bg = background / hsz;
    o->col_tphi.assign( (size_t)nslots * 512, bg );
    if( vel ) o->col_tvel.assign( (size_t)nslots * 512 * 3, 0.f );
    for( size_t v = 0; v < count; ++v )
    {
        const int i = ijk[3 * v], j = ijk[3 * v + 1], k = ijk[3 * v + 2];
        if( i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz ) continue;
        const size_t q = (size_t)o->col_tslot[lin( i / 8, j / 8, k / 8 )] * 512 + bora_collider_local( i, j, k );
        o->col_tphi[q] = phi[v] / hsz;
        if( vel )
            for( int a = 0; a < 3; ++a ) o->col_tvel[3 * q + a] = vel[3 * v + a] / o->scale[a];
    }
    o->cols.tslot = o->col_tslot.data();
    o->cols.tphi = o->col_tphi.data();
    o->cols.tvel = vel ? o->col_tvel.data() : nullptr;
    o->cols.tbg = bg;
    o->cols.ttx = tx;
    o->cols.tty = ty;
}

void ora_set_colliders( void* h, int n, const float* boxes, float band )
{
    Oracle* o = (Oracle*)h;
    std::memset( &o->cols, 0, sizeof( o->cols ) );
    o->cols.count = n < BORA_MAX_COLLIDERS ? n : BORA_MAX_COLLIDERS;
    o->cols.band = band;
    for( int q = 0; q < o->cols.count; ++q )
        for( int c = 0; c < 3; ++c )
        {
            o->cols.box[q].lo[c] = boxes[q * 9 + c];
            o->cols.box[q].hi[c] = boxes[q * 9 + 3 + c];
            o->cols.box[q].vel[c] = boxes[q * 9 + 6 + c];
        }
}

void ora_set_particles( void* h, const float* pos, const float* vel, const int32_t* id, size_t n )
{
    Oracle* o = (Oracle*)h;
    o->pos.resize( n ); o->vel.resize( n ); o->adj.assign( n, 0.f ); o->pid.resize( n );
    o->vort.assign( n, 0.f ); o->curv.assign( n, 0.f );
    for( size_t i = 0; i < n; ++i )
    {
        o->pos[i] = V3{ pos[3 * i], pos[3 * i + 1], pos[3 * i + 2] };
        o->vel[i] = V3{ vel[3 * i], vel[3 * i + 1], vel[3 * i + 2] };
        o->pid[i] = id ? id[i] : (int32_t)i;
    }
}

// Random.h:30-38, Rand( seed, 0, 1 ): an integer hash of the seed scaled to [0, 1].
static float bora_rand01( unsigned int seed )
{
    unsigned int i = ( seed ^ 12345391u ) * 2654435769u;
    i ^= ( i << 6 ) ^ ( i >> 26 );
    i *= 2654435769u;
    i += ( i << 5 ) ^ ( i >> 12 );
    return ( 1.0f - 0.0f ) * (float)i / (float)( UINT_MAX ) + 0.0f;
}

// FLIPMethod::fillWaterTank (base/source/FLIPMethod.cu:407-478): per cell below the wall
// level two jittered particles, the cell centre, and `per_cell` more in the 4-cell band
// under the wall, appended in (k, j, i) order; their world positions (Grid::worldPoint)
// come back to voxel space as particlesToVoxel does (FLIPMethod.cu:499-514). Returns the
// number of particles added (ids continue after the largest id).
size_t ora_fill_water_tank( void* h, int per_cell )
{
    Oracle* o = (Oracle*)h;
    const float wall = o->voxelWall;
    if( wall <= 0.f ) return 0;
    int32_t next = 0;
    for( int32_t q : o->pid ) next = q + 1 > next ? q + 1 : next;
    const size_t n0 = o->pos.size();
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    const int hh = clampi( (int)wall + 1, 0, ny );
    auto add = [&]( V3 p ) {
        V3 w{ p.x * o->scale[0] + o->translate[0], p.y * o->scale[1] + o->translate[1], p.z * o->scale[2] + o->translate[2] };
        V3 v{ ( w.x - o->translate[0] ) / o->scale[0], ( w.y - o->translate[1] ) / o->scale[1], ( w.z - o->translate[2] ) / o->scale[2] };
        o->pos.push_back( v );
        o->vel.push_back( V3{ 0.f, 0.f, 0.f } );
        o->adj.push_back( 0.f );
        o->pid.push_back( next++ );
        o->vort.push_back( 0.f );
        o->curv.push_back( 0.f );
    };
    for( int k = 0; k < nz; ++k )
        for( int j = 0; j < hh; ++j )
            for( int i = 0; i < nx; ++i )
            {
                const unsigned ui = (unsigned)i, uj = (unsigned)j, uk = (unsigned)k;
                const V3 cen{ i + .5f, j + .5f, k + .5f };
                const float band = wall - cen.y;
                const float dx0 = bora_rand01( ui * 45651u + uk * 75561u + uj * 65551u );
                const float dy0 = bora_rand01( ui * 51221u + uk * 99331u + uj * 11221u );
                const float dz0 = bora_rand01( ui * 81221u + uk * 45331u + uj * 66551u );
                const float dx1 = bora_rand01( ui * 53454u + uk * 12234u + uj * 23853u );
                const float dy1 = bora_rand01( ui * 76335u + uk * 94762u + uj * 93654u );
                const float dz1 = bora_rand01( ui * 98547u + uk * 23443u + uj * 53218u );
                const V3 p0{ ( cen.x - 0.5f ) + dx0, ( cen.y - 0.5f ) + dy0, ( cen.z - 0.5f ) + dz0 };
                const V3 p1{ ( cen.x - 0.5f ) + dx1, ( cen.y - 0.5f ) + dy1, ( cen.z - 0.5f ) + dz1 };
                if( p0.y <= wall ) add( p0 );
                if( p1.y <= wall ) add( p1 );
                if( cen.y <= wall ) add( cen );
                if( band > 0.f && band < 4.f )
                    for( int n = 0; n < per_cell; ++n )
                    {
                        const unsigned un = (unsigned)n;
                        const float dx = bora_rand01( ui * 45651u + uk * 75561u + uj * 65551u + un * 44222u );
                        const float dy = bora_rand01( ui * 51221u + uk * 99331u + uj * 11221u + un * 59374u );
                        const float dz = bora_rand01( ui * 81221u + uk * 45331u + uj * 66551u + un * 12333u );
                        const V3 pp{ ( cen.x - 0.5f ) + dx, ( cen.y - 0.5f ) + dy, ( cen.z - 0.5f ) + dz };
                        if( pp.y <= wall ) add( pp );
                    }
            }
    return o->pos.size() - n0;
}

size_t ora_num_particles( void* h ) { return ( (Oracle*)h )->pos.size(); }

void ora_get_particles( void* h, float* pos, float* vel, float* adj, int32_t* id )
{
    Oracle* o = (Oracle*)h;
    for( size_t i = 0; i < o->pos.size(); ++i )
    {
        if( pos ) { pos[3 * i] = o->pos[i].x; pos[3 * i + 1] = o->pos[i].y; pos[3 * i + 2] = o->pos[i].z; }
        if( vel ) { vel[3 * i] = o->vel[i].x; vel[3 * i + 1] = o->vel[i].y; vel[3 * i + 2] = o->vel[i].z; }
        if( adj ) adj[i] = o->adj[i];
        if( id ) id[i] = o->pid[i];
    }
}

size_t ora_get_removed( void* h, uint8_t* out )
{
    Oracle* o = (Oracle*)h;
    if( out ) std::memcpy( out, o->removed.data(), o->removed.size() );
    return o->removed.size();
}

void ora_rebuild( void* h ) { ( (Oracle*)h )->rebuild(); }
void ora_p2g( void* h ) { ( (Oracle*)h )->p2g(); }
void ora_mark( void* h ) { ( (Oracle*)h )->markCells(); }
void ora_build_system( void* h ) { ( (Oracle*)h )->buildSystem(); }
int ora_solve( void* h ) { return ( (Oracle*)h )->solve(); }
void ora_update_velocity( void* h ) { ( (Oracle*)h )->updateVelocity(); }
void ora_update_particles( void* h, float dt ) { ( (Oracle*)h )->updateParticles( dt ); }
void ora_compact( void* h ) { ( (Oracle*)h )->compact(); }
int ora_step( void* h, float dt ) { return ( (Oracle*)h )->step( dt ); }
double ora_last_rel( void* h ) { return ( (Oracle*)h )->lastRel; }

// FLIPMethod::postProcess and its parts. flags: bit 0 = the reference's tank scan as
// executed (see tankScan).
void ora_post_process( void* h, float dt, float vort_pres_rate, int redist_iteration, int flags )
{
    ( (Oracle*)h )->postProcess( dt, vort_pres_rate, redist_iteration, flags & 1 );
}
void ora_post_splat( void* h ) { ( (Oracle*)h )->splatSurface(); }
void ora_post_tank_scan( void* h, int literal ) { ( (Oracle*)h )->tankScan( literal != 0 ); }
void ora_post_redistance( void* h, int iters ) { ( (Oracle*)h )->redistance( iters ); }
void ora_post_attributes( void* h, float dt, float vort_pres_rate ) { ( (Oracle*)h )->particleAttributes( dt, vort_pres_rate ); }

// Particle vorticity and curvature, in particle order (any pointer may be NULL).
void ora_get_attributes( void* h, float* vort, float* curv )
{
    Oracle* o = (Oracle*)h;
    const size_t n = o->pos.size();
    for( size_t i = 0; i < n; ++i )
    {
        if( vort ) vort[i] = i < o->vort.size() ? o->vort[i] : 0.f;
        if( curv ) curv[i] = i < o->curv.size() ? o->curv[i] : 0.f;
    }
}
void ora_set_attributes( void* h, const float* vort, const float* curv )
{
    Oracle* o = (Oracle*)h;
    const size_t n = o->pos.size();
    o->vort.assign( n, 0.f );
    o->curv.assign( n, 0.f );
    for( size_t i = 0; i < n; ++i )
    {
        if( vort ) o->vort[i] = vort[i];
        if( curv ) o->curv[i] = curv[i];
    }
}

// out: fx, fy, fz, block, frame nx, ny, nz, active tiles
void ora_frame_info( void* h, int64_t* out )
{
    Oracle* o = (Oracle*)h;
    out[0] = o->fx; out[1] = o->fy; out[2] = o->fz; out[3] = o->B;
    out[4] = o->nx; out[5] = o->ny; out[6] = o->nz; out[7] = (int64_t)( o->coords.size() / 3 );
}

// out: translate[3], scale[3], voxel wall level, voxel gravity[3]
void ora_grid_xform( void* h, float* out )
{
    Oracle* o = (Oracle*)h;
    for( int a = 0; a < 3; ++a ) { out[a] = o->translate[a]; out[3 + a] = o->scale[a]; }
    out[6] = o->voxelWall;
    out[7] = o->voxelForce.x; out[8] = o->voxelForce.y; out[9] = o->voxelForce.z;
}

void ora_get_tiles( void* h, int64_t* ijk )
{
    Oracle* o = (Oracle*)h;
    std::memcpy( ijk, o->coords.data(), o->coords.size() * sizeof( int64_t ) );
}

void ora_get_markers( void* h, int32_t* out )
{
    Oracle* o = (Oracle*)h;
    std::memcpy( out, o->markers.data(), o->markers.size() * sizeof( int32_t ) );
}

size_t ora_field_size( void* h ) { return ( (Oracle*)h )->ncells(); }

// which: 0 mass, 1 surf(count), 2 pres, 3 velo (3 floats), 4 comp (3 floats), 5 mark (int64)
void ora_get_field( void* h, int which, void* out )
{
    Oracle* o = (Oracle*)h;
    const size_t n = o->ncells();
    switch( which )
    {
        case 0: std::memcpy( out, o->mass.data(), n * 4 ); break;
        case 1: std::memcpy( out, o->surf.data(), n * 4 ); break;
        case 2: std::memcpy( out, o->pres.data(), n * 4 ); break;
        case 3: std::memcpy( out, o->velo.data(), n * 12 ); break;
        case 4: std::memcpy( out, o->comp.data(), n * 12 ); break;
        case 5: std::memcpy( out, o->mark.data(), n * 8 ); break;
        default: break;
    }
}

void ora_set_field( void* h, int which, const void* in )
{
    Oracle* o = (Oracle*)h;
    const size_t n = o->ncells();
    switch( which )
    {
        case 0: std::memcpy( o->mass.data(), in, n * 4 ); break;
        case 1: std::memcpy( o->surf.data(), in, n * 4 ); break;
        case 2: std::memcpy( o->pres.data(), in, n * 4 ); break;
        case 3: std::memcpy( o->velo.data(), in, n * 12 ); break;
        case 4: std::memcpy( o->comp.data(), in, n * 12 ); break;
        case 5: std::memcpy( o->mark.data(), in, n * 8 ); break;
        default: break;
    }
}

size_t ora_num_unknowns( void* h ) { return ( (Oracle*)h )->b.size(); }

void ora_get_system( void* h, float* b, float* x, int64_t* cells, float* vals, int64_t* cols )
{
    Oracle* o = (Oracle*)h;
    const size_t n = o->b.size();
    if( b ) std::memcpy( b, o->b.data(), n * 4 );
    if( x ) std::memcpy( x, o->x.data(), n * 4 );
    if( cells ) std::memcpy( cells, o->fluidCells.data(), n * 8 );
    if( vals ) std::memcpy( vals, o->Avals.data(), n * 7 * 4 );
    if( cols ) std::memcpy( cols, o->Acols.data(), n * 7 * 8 );
}

void ora_set_solution( void* h, const float* x )
{
    Oracle* o = (Oracle*)h;
    std::memcpy( o->x.data(), x, o->x.size() * 4 );
}

// max_i |b_i - (A x)_i| in double for the current x (the projected-system residual).
double ora_residual_max( void* h )
{
    Oracle* o = (Oracle*)h;
    double m = 0.0;
    for( size_t r = 0; r < o->b.size(); ++r )
    {
        double acc = 0.0;
        for( int c = 0; c < 7; ++c )
        {
            const int64_t n = o->Acols[r * 7 + c];
            if( n != kNull ) acc += (double)o->Avals[r * 7 + c] * (double)o->x[(size_t)n];
        }
        const double e = std::fabs( (double)o->b[r] - acc );
        if( e > m ) m = e;
    }
    return m;
}

}  // extern "C"
