// Shared device definitions of the GB300 FLIP substep.
//
// Layout in HBM (one simulation):
//   * virtual grid nx*ny*nz cells (padded to a multiple of 4 per axis and re-centred
//     exactly like SparseFrame::initialize, base/source/SparseFrame.cu:28-73), covered
//     by 8^3-cell tiles TX*TY*TZ;
//   * tile table tile_slot[TX*TY*TZ] (int32, -1 = inactive) -> O(1) cell lookup, and
//     for each active slot its linear tile index and its 27 neighbour slots;
//   * cell fields are structure-of-arrays over active slots x 512 cells, x fastest
//     inside the tile (the reference's storage order, SparseField.h:57-112, at tile
//     edge 8);
//   * particles are structure-of-arrays (px,py,pz,vx,vy,vz,id), double buffered, and
//     sorted every step by "dual cell" = the base cell of the reference's P2G stencil
//     (max(int(p-0.5),0) per axis, Rasterization.cu:139-141).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define BORA_TILE 8
#define BORA_TILE_CELLS 512
#define BORA_DEAD_KEY 0xFFFFFFFFu

// Cell types (FluidProjection::CELLTYPE, base/header/FluidProjection.h:32-39).
#define BORA_AIR 0
#define BORA_SOLID 1
#define BORA_WALL 2
#define BORA_FLUID 4
#define BORA_MASKED 0xFF  // cell of an edge tile that lies beyond the grid

// Stencil code of a fluid cell (uint16): bits 0..5 = the -x,+x,-y,+y,-z,+z neighbour is
// fluid; bits 8..11 = diagonal of the 7-point operator (6 + #air - #solid/wall
// neighbours, FluidProjection.cu:234-244); bit 15 = the cell is fluid.
#define BORA_CODE_FLUID 0x8000u

#define BORA_MAX_COLLIDERS 8

struct BoraBoxDev
{
    float lo[3], hi[3], vel[3];
};

// Colliders: analytic boxes sampled at cell centres, or (fphi != null) signed distances
// and velocities given per cell of the frame grid (x fastest), as CollisionSource samples
// its SDF and velocity grids at cell centres (CollisionSource.h:66-126).
struct BoraColliderDev
{
    int count;
    float band;
    BoraBoxDev box[BORA_MAX_COLLIDERS];
    const float* fphi;  // [nx*ny*nz] voxel units, or null
    const float* fvel;  // [3*nx*ny*nz] voxel units per second, or null (zero)
    // sparse collider (CollisionSource::update from a level set's active voxels): the
    // collider's own 8^3 tiles over the frame's tile grid
    const int32_t* tslot;  // [tx*ty*tz] collider tile slot or -1, or null (no sparse collider)
    const uint8_t* tnear;  // [tx*ty*tz] 1 where a collider tile lies within one tile
    const float* tphi;     // [slots*512] signed distance, voxel units
    const float* tvel;     // [slots*512*3] velocity, voxel units per second, or null (zero)
    float tbg;             // the level set's background, voxel units
    int ttx, tty;          // tile grid extents in x and y (for the lookup)
};

__host__ __device__ inline bool bora_col_active( const BoraColliderDev& s )
{
    return s.count > 0 || s.fphi != nullptr || s.tslot != nullptr;
}

// the sparse collider's slot of the tile holding cell (i,j,k), or -1
__host__ __device__ inline int bora_col_tile_slot( const BoraColliderDev& s, int i, int j, int k )
{
    return s.tslot[(size_t)( i >> 3 ) + (size_t)s.ttx * ( (size_t)( j >> 3 ) + (size_t)s.tty * (size_t)( k >> 3 ) )];
}

// Grid constants shared by every kernel of one simulation.
struct BoraGridDev
{
    int nx, ny, nz;     // frame grid (cells)
    int tx, ty, tz;     // tiles per axis
    float voxel_wall;   // wall level in voxel units (FLIPMethod.cu:44-46)
    float gravity[3];   // voxel units (FLIPMethod.cu:42)
    float col_vel_scale;
    int maxsubsteps;
    int enable_tank;
    float damping_band;  // voxel units
    int advection;       // BORA_ADVECT_EULER / BORA_ADVECT_RK2
    BoraColliderDev cols;
};

__host__ __device__ inline int bora_imin( int a, int b ) { return a < b ? a : b; }
__host__ __device__ inline int bora_imax( int a, int b ) { return a > b ? a : b; }
__host__ __device__ inline int bora_clampi( int x, int lo, int hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }
__host__ __device__ inline float bora_clampf( float x, float lo, float hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }

// float -> int with C truncation; saturates for |x| >= 2^31 (device cvt.rzi semantics).
__device__ inline int bora_trunc( float x ) { return __float2int_rz( x ); }

// Local index of a cell inside its tile (x fastest).
__host__ __device__ inline int bora_local( int i, int j, int k ) { return ( i & 7 ) | ( ( j & 7 ) << 3 ) | ( ( k & 7 ) << 6 ); }

// Neighbour direction index 0..26 of an offset in {-1,0,1}^3.
__host__ __device__ inline int bora_dir( int dx, int dy, int dz ) { return ( dx + 1 ) + 3 * ( dy + 1 ) + 9 * ( dz + 1 ); }

// The rebuild's binning rule for one particle (SparseFrame::buildFromPoints,
// SparseFrame.cu:101-103 at tile edge 8): a live particle activates its tile
// (max(int(p)/8, 0), clamped to the table) and gets the key virtual tile * 512 + local index
// of its dual cell (the base cell max(int(p - 0.5), 0) of the P2G stencil, Rasterization.cu:
// 139-141); killed particles get BORA_DEAD_KEY, live ones outside the grid (Grid::inside,
// Grid.h:408-417) BORA_DEAD_KEY - 1 (they still activate their clamped tile).
__device__ inline void bora_bin_tile( int tx, int ty, int tz, float x, float y, float z, int& ti, int& tj, int& tk )
{
    ti = bora_imin( bora_imax( bora_trunc( x ) / BORA_TILE, 0 ), tx - 1 );
    tj = bora_imin( bora_imax( bora_trunc( y ) / BORA_TILE, 0 ), ty - 1 );
    tk = bora_imin( bora_imax( bora_trunc( z ) / BORA_TILE, 0 ), tz - 1 );
}
__device__ inline uint32_t bora_bin_live_key( int nx, int ny, int nz, int tx, int ty, float x, float y, float z )
{
    if( x < 0.f || x > (float)nx || y < 0.f || y > (float)ny || z < 0.f || z > (float)nz ) return BORA_DEAD_KEY - 1;
    const int di = bora_imax( bora_trunc( x - 0.5f ), 0 );
    const int dj = bora_imax( bora_trunc( y - 0.5f ), 0 );
    const int dk = bora_imax( bora_trunc( z - 0.5f ), 0 );
    const uint32_t vt = (uint32_t)( ( (size_t)( dk >> 3 ) * ty + ( dj >> 3 ) ) * tx + ( di >> 3 ) );
    return vt * BORA_TILE_CELLS + (uint32_t)bora_local( di, dj, dk );
}
// both parts, the tile flag stored in tile_flag
__device__ inline uint32_t bora_bin_key( int nx, int ny, int nz, int tx, int ty, int tz, int32_t id, float x, float y,
                                         float z, uint8_t* __restrict__ tile_flag )
{
    if( id < 0 ) return BORA_DEAD_KEY;
    int ti, tj, tk;
    bora_bin_tile( tx, ty, tz, x, y, z, ti, tj, tk );
    tile_flag[( (size_t)tk * ty + tj ) * tx + ti] = 1;
    return bora_bin_live_key( nx, ny, nz, tx, ty, x, y, z );
}

// ---- analytic box colliders sampled at cell centres -------------------------------
// The reference samples an OpenVDB level set into sparse fields and lerps the samples
// (base/header/CollisionSource.h:66-150). Colliders here are analytic boxes: cell-centre
// samples are evaluated on the fly (clamped signed distance, the nearest box's velocity
// inside the band, normalised central-difference normal) and queried with
// SparseField::lerp's rule (base/header/SparseField.h:150-173).
__device__ inline float bora_box_sdf( const BoraBoxDev& b, float px, float py, float pz )
{
    const float cx = ( b.lo[0] + b.hi[0] ) * 0.5f;
    const float cy = ( b.lo[1] + b.hi[1] ) * 0.5f;
    const float cz = ( b.lo[2] + b.hi[2] ) * 0.5f;
    const float hx = ( b.hi[0] - b.lo[0] ) * 0.5f;
    const float hy = ( b.hi[1] - b.lo[1] ) * 0.5f;
    const float hz = ( b.hi[2] - b.lo[2] ) * 0.5f;
    const float qx = fabsf( px - cx ) - hx;
    const float qy = fabsf( py - cy ) - hy;
    const float qz = fabsf( pz - cz ) - hz;
    const float ox = qx > 0.f ? qx : 0.f;
    const float oy = qy > 0.f ? qy : 0.f;
    const float oz = qz > 0.f ? qz : 0.f;
    const float outside = sqrtf( ox * ox + oy * oy + oz * oz );
    float m = qx > qy ? qx : qy;
    m = m > qz ? m : qz;
    const float inside = m < 0.f ? m : 0.f;
    return outside + inside;
}

__device__ inline float bora_col_phi_cell( const BoraColliderDev& s, int nx, int ny, int i, int j, int k, int* arg )
{
    if( s.tslot )
    {
        if( arg ) *arg = 0;
        const int sl = bora_col_tile_slot( s, i, j, k );
        return sl < 0 ? s.tbg : s.tphi[(size_t)sl * 512 + ( ( i & 7 ) | ( ( j & 7 ) << 3 ) | ( ( k & 7 ) << 6 ) )];
    }
    if( s.fphi )
    {
        if( arg ) *arg = 0;
        return s.fphi[(size_t)i + (size_t)nx * ( (size_t)j + (size_t)ny * k )];
    }
    const float px = (float)i + 0.5f, py = (float)j + 0.5f, pz = (float)k + 0.5f;
    float best = s.band;
    int a = -1;
    for( int n = 0; n < s.count; ++n )
    {
        const float d = bora_box_sdf( s.box[n], px, py, pz );
        if( a < 0 || d < best ) { best = d; a = n; }
    }
    if( best > s.band ) best = s.band;
    if( best < -s.band ) best = -s.band;
    if( arg ) *arg = a;
    return best;
}

// which: 0 phi, 1 normal, 2 velocity
__device__ inline void bora_col_sample( const BoraColliderDev& s, int nx, int ny, int nz, int i, int j, int k,
                                        int which, float out[3] )
{
    int a;
    if( which == 0 )
    {
        out[0] = bora_col_phi_cell( s, nx, ny, i, j, k, &a );
        out[1] = out[2] = 0.f;
        return;
    }
    if( s.tslot && which == 2 )
    {
        const int sl = bora_col_tile_slot( s, i, j, k );
        const size_t c = (size_t)sl * 512 + ( ( i & 7 ) | ( ( j & 7 ) << 3 ) | ( ( k & 7 ) << 6 ) );
        const bool have = sl >= 0 && s.tvel;
        out[0] = have ? s.tvel[3 * c] : 0.f;
        out[1] = have ? s.tvel[3 * c + 1] : 0.f;
        out[2] = have ? s.tvel[3 * c + 2] : 0.f;
        return;
    }
    if( s.tslot && bora_col_tile_slot( s, i, j, k ) < 0 )  // the gradient field's background
    {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    if( which == 2 && s.fphi )
    {
        const size_t c = (size_t)i + (size_t)nx * ( (size_t)j + (size_t)ny * k );
        out[0] = s.fvel ? s.fvel[3 * c] : 0.f;
        out[1] = s.fvel ? s.fvel[3 * c + 1] : 0.f;
        out[2] = s.fvel ? s.fvel[3 * c + 2] : 0.f;
        return;
    }
    if( which == 2 )
    {
        const float phi = bora_col_phi_cell( s, nx, ny, i, j, k, &a );
        if( a >= 0 && phi < s.band )
        {
            out[0] = s.box[a].vel[0]; out[1] = s.box[a].vel[1]; out[2] = s.box[a].vel[2];
        }
        else
        {
            out[0] = out[1] = out[2] = 0.f;
        }
        return;
    }
    const int i0 = i > 0 ? i - 1 : 0, i1 = i < nx - 1 ? i + 1 : nx - 1;
    const int j0 = j > 0 ? j - 1 : 0, j1 = j < ny - 1 ? j + 1 : ny - 1;
    const int k0 = k > 0 ? k - 1 : 0, k1 = k < nz - 1 ? k + 1 : nz - 1;
    const float gx = ( bora_col_phi_cell( s, nx, ny, i1, j, k, 0 ) - bora_col_phi_cell( s, nx, ny, i0, j, k, 0 ) ) * 0.5f;
    const float gy = ( bora_col_phi_cell( s, nx, ny, i, j1, k, 0 ) - bora_col_phi_cell( s, nx, ny, i, j0, k, 0 ) ) * 0.5f;
    const float gz = ( bora_col_phi_cell( s, nx, ny, i, j, k1, 0 ) - bora_col_phi_cell( s, nx, ny, i, j, k0, 0 ) ) * 0.5f;
    const double d = 1.0f / sqrtf( gx * gx + gy * gy + gz * gz + 1e-30f );
    out[0] = (float)( gx * d );
    out[1] = (float)( gy * d );
    out[2] = (float)( gz * d );
}

__device__ inline void bora_col_lerp( const BoraColliderDev& s, int nx, int ny, int nz, float px, float py, float pz,
                                      int which, float out[3] )
{
    const int i = bora_clampi( bora_trunc( px - 0.5f ), 0, nx - 2 );
    const int j = bora_clampi( bora_trunc( py - 0.5f ), 0, ny - 2 );
    const int k = bora_clampi( bora_trunc( pz - 0.5f ), 0, nz - 2 );
    const float x = bora_clampf( px - ( (float)i + 0.5f ), 0.f, 1.f );
    const float y = bora_clampf( py - ( (float)j + 0.5f ), 0.f, 1.f );
    const float z = bora_clampf( pz - ( (float)k + 0.5f ), 0.f, 1.f );
    float f000[3], f100[3], f001[3], f101[3], f010[3], f110[3], f011[3], f111[3];
    bora_col_sample( s, nx, ny, nz, i, j, k, which, f000 );
    bora_col_sample( s, nx, ny, nz, i + 1, j, k, which, f100 );
    bora_col_sample( s, nx, ny, nz, i, j, k + 1, which, f001 );
    bora_col_sample( s, nx, ny, nz, i + 1, j, k + 1, which, f101 );
    bora_col_sample( s, nx, ny, nz, i, j + 1, k, which, f010 );
    bora_col_sample( s, nx, ny, nz, i + 1, j + 1, k, which, f110 );
    bora_col_sample( s, nx, ny, nz, i, j + 1, k + 1, which, f011 );
    bora_col_sample( s, nx, ny, nz, i + 1, j + 1, k + 1, which, f111 );
#pragma unroll
    for( int c = 0; c < 3; ++c )
    {
        const float c00 = f000[c] * ( 1.f - x ) + f100[c] * x;
        const float c01 = f001[c] * ( 1.f - x ) + f101[c] * x;
        const float c10 = f010[c] * ( 1.f - x ) + f110[c] * x;
        const float c11 = f011[c] * ( 1.f - x ) + f111[c] * x;
        const float c0 = c00 * ( 1.f - y ) + c10 * y;
        const float c1 = c01 * ( 1.f - y ) + c11 * y;
        out[c] = c0 * ( 1.f - z ) + c1 * z;
    }
}

__device__ inline float bora_col_phi( const BoraGridDev& g, float px, float py, float pz )
{
    if( !bora_col_active( g.cols ) ) return 5.f;  // reference background without a collider (CollisionSource.h:56,130)
    float v[3];
    bora_col_lerp( g.cols, g.nx, g.ny, g.nz, px, py, pz, 0, v );
    return v[0];
}
